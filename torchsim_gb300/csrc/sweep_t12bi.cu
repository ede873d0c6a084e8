// Forward plus the T1, T2, B1 and inversion-efficiency tangents in one pass.
#include "epg_sweep.cuh"

namespace tsg {
const SweepEntry kSweepT12BI[] = {
    TSG_SWEEP_ENTRY(MODE_T12BI, 2, 5, 15, false),
    TSG_SWEEP_ENTRY(MODE_T12BI, 4, 5, 15, false),
    TSG_SWEEP_ENTRY(MODE_T12BI, 2, 10, 15, false),
    TSG_SWEEP_ENTRY(MODE_T12BI, 4, 4, 15, false),
    TSG_SWEEP_ENTRY(MODE_T12BI, 4, 8, 15, false),
    TSG_SWEEP_ENTRY(MODE_T12BI, 4, 16, 15, false),
    TSG_SWEEP_ENTRY(MODE_T12BI, 4, 32, 15, false),
};
const int kSweepT12BICount = sizeof(kSweepT12BI) / sizeof(kSweepT12BI[0]);
}  // namespace tsg
