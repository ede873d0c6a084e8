// Gauss-Newton evaluation sweeps: forward plus the T1 and T2 tangents (M0 is
// free), reduced against the measured samples to each voxel's cost, J^T J
// and J^T r in natural parameters, so neither the signal nor the Jacobian
// touches HBM. The reference forms the full Jacobian blocks, (V, 3, 880)
// complex, with one forward and one tangent pass per column
// (recon/_gauss_newton.py:633-651 -> recon/_operator.py:459-484) and then an
// augmented least-squares solve per voxel (_gauss_newton.py:247-307).
#include "epg_sweep.cuh"

namespace tsg {
const SweepEntry kSweepGN[] = {
    // One voxel per lane with three blocks of 128 threads per SM (164
    // registers): 12 warps per SM where the unbounded kernel holds 8.
    TSG_GN_ENTRY_MINB(10, 1, 3),
    TSG_GN_ENTRY(10, 1), TSG_GN_ENTRY(2, 5), TSG_GN_ENTRY(6, 2), TSG_GN_ENTRY(4, 5), TSG_GN_ENTRY(2, 10), TSG_GN_ENTRY(4, 4), TSG_GN_ENTRY(8, 4), TSG_GN_ENTRY(4, 8), TSG_GN_ENTRY(8, 8), TSG_GN_ENTRY(4, 16), TSG_GN_ENTRY(4, 32),
};
const int kSweepGNCount = sizeof(kSweepGN) / sizeof(kSweepGN[0]);
}  // namespace tsg
