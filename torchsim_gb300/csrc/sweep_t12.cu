// Forward plus the T1 and T2 tangents in one pass.
#include "epg_sweep.cuh"

namespace tsg {
const SweepEntry kSweepT12[] = {
    TSG_SWEEP_ENTRY(MODE_T12, 10, 1, 3, false),
    TSG_SWEEP_ENTRY(MODE_T12, 2, 5, 3, false),
    TSG_SWEEP_ENTRY(MODE_T12, 6, 2, 3, false),
    TSG_SWEEP_ENTRY(MODE_T12, 4, 5, 3, false),
    TSG_SWEEP_ENTRY(MODE_T12, 2, 10, 3, false),
    TSG_SWEEP_ENTRY(MODE_T12, 4, 4, 3, false),
    TSG_SWEEP_ENTRY(MODE_T12, 6, 4, 3, false),
    TSG_SWEEP_ENTRY(MODE_T12, 8, 4, 3, false),
    TSG_SWEEP_ENTRY(MODE_T12, 4, 8, 3, false),
    TSG_SWEEP_ENTRY(MODE_T12, 8, 8, 3, false),
    TSG_SWEEP_ENTRY(MODE_T12, 4, 16, 3, false),
    TSG_SWEEP_ENTRY(MODE_T12, 4, 32, 3, false),
};
const int kSweepT12Count = sizeof(kSweepT12) / sizeof(kSweepT12[0]);
}  // namespace tsg
