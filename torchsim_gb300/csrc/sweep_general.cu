// Forward plus one general direction (tissue, durations and flips), the
// reference's simulate_jvp, src/torchsim/_epg_cpu.cpp:3136-3285.
#include "epg_sweep.cuh"

namespace tsg {
const SweepEntry kSweepGeneral[] = {
    TSG_SWEEP_ENTRY(MODE_GENERAL, 10, 1, 0, true),
    TSG_SWEEP_ENTRY(MODE_GENERAL, 2, 5, 0, true),
    TSG_SWEEP_ENTRY(MODE_GENERAL, 6, 2, 0, true),
    TSG_SWEEP_ENTRY(MODE_GENERAL, 4, 5, 0, true),
    TSG_SWEEP_ENTRY(MODE_GENERAL, 2, 10, 0, true),
    TSG_SWEEP_ENTRY(MODE_GENERAL, 4, 4, 0, true),
    TSG_SWEEP_ENTRY(MODE_GENERAL, 6, 4, 0, true),
    TSG_SWEEP_ENTRY(MODE_GENERAL, 8, 4, 0, true),
    TSG_SWEEP_ENTRY(MODE_GENERAL, 4, 8, 0, true),
    TSG_SWEEP_ENTRY(MODE_GENERAL, 4, 16, 0, true),
    TSG_SWEEP_ENTRY(MODE_GENERAL, 4, 32, 0, true),
};
const int kSweepGeneralCount = sizeof(kSweepGeneral) / sizeof(kSweepGeneral[0]);
}  // namespace tsg
