// Forward plus the T1, T2 and B1 tangents in one pass (dictionary Jacobian).
#include "epg_sweep.cuh"

namespace tsg {
const SweepEntry kSweepT12B[] = {
    TSG_SWEEP_ENTRY(MODE_T12B, 2, 5, 7, false),
    TSG_SWEEP_ENTRY(MODE_T12B, 6, 2, 7, false),
    TSG_SWEEP_ENTRY(MODE_T12B, 4, 5, 7, false),
    TSG_SWEEP_ENTRY(MODE_T12B, 2, 10, 7, false),
    TSG_SWEEP_ENTRY(MODE_T12B, 4, 4, 7, false),
    TSG_SWEEP_ENTRY(MODE_T12B, 6, 4, 7, false),
    TSG_SWEEP_ENTRY(MODE_T12B, 4, 8, 7, false),
    TSG_SWEEP_ENTRY(MODE_T12B, 4, 16, 7, false),
    TSG_SWEEP_ENTRY(MODE_T12B, 4, 32, 7, false),
    TSG_SWEEP_ENTRY_MINB(MODE_T12B, 4, 5, 7, false, 5),
    TSG_SWEEP_ENTRY_MINB(MODE_T12B, 4, 5, 7, false, 6),
    TSG_SWEEP_ENTRY_MINB(MODE_T12B, 2, 10, 7, false, 8),
    TSG_SWEEP_ENTRY_MINB(MODE_T12B, 4, 4, 7, false, 6),
    // Budgets that hold the relaxation-folded tangent step.
    TSG_SWEEP_ENTRY_MINB(MODE_T12B, 4, 5, 7, false, 4),
    TSG_SWEEP_ENTRY_MINB(MODE_T12B, 2, 10, 7, false, 6),
    TSG_SWEEP_ENTRY_MINB(MODE_T12B, 2, 10, 7, false, 7),
};
const int kSweepT12BCount = sizeof(kSweepT12B) / sizeof(kSweepT12B[0]);
}  // namespace tsg
