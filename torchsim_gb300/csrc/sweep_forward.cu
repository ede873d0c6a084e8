// Forward-only sweeps (no tangents): the plain form of the real-subspace
// forward, src/torchsim/_epg_cpu.cpp:3041-3128.
#include "epg_sweep.cuh"

namespace tsg {
const SweepEntry kSweepForward[] = {
    TSG_SWEEP_ENTRY(MODE_FORWARD, 10, 1, 0, false),
    TSG_SWEEP_ENTRY(MODE_FORWARD, 20, 1, 0, false),
    TSG_SWEEP_ENTRY(MODE_FORWARD, 2, 5, 0, false),
    TSG_SWEEP_ENTRY(MODE_FORWARD, 6, 2, 0, false),
    TSG_SWEEP_ENTRY(MODE_FORWARD, 4, 5, 0, false),
    TSG_SWEEP_ENTRY(MODE_FORWARD, 2, 10, 0, false),
    TSG_SWEEP_ENTRY(MODE_FORWARD, 4, 4, 0, false),
    TSG_SWEEP_ENTRY(MODE_FORWARD, 6, 4, 0, false),
    TSG_SWEEP_ENTRY(MODE_FORWARD, 8, 4, 0, false),
    TSG_SWEEP_ENTRY(MODE_FORWARD, 4, 8, 0, false),
    TSG_SWEEP_ENTRY(MODE_FORWARD, 8, 8, 0, false),
    TSG_SWEEP_ENTRY(MODE_FORWARD, 4, 16, 0, false),
    TSG_SWEEP_ENTRY(MODE_FORWARD, 8, 16, 0, false),
    TSG_SWEEP_ENTRY(MODE_FORWARD, 4, 32, 0, false),
    TSG_SWEEP_ENTRY(MODE_FORWARD, 8, 32, 0, false),
    TSG_SWEEP_ENTRY(MODE_FORWARD, 10, 2, 0, false),
};
const int kSweepForwardCount = sizeof(kSweepForward) / sizeof(kSweepForward[0]);
}  // namespace tsg
