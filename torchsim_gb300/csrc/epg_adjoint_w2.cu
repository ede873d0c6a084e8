// Reverse-sweep kernels with 2 warps per block (orders per lane, lanes per
// voxel), checkpointed and trajectory mode.
#include "epg_adjoint.cuh"

namespace tsg {

extern const AdjointEntry kAdjointW2[];
extern const int kAdjointW2Count;
extern const AdjointEntry kAdjointTrajectoryW2[];
extern const int kAdjointTrajectoryW2Count;

const AdjointEntry kAdjointW2[] = {
    TSG_ADJOINT_ENTRY(10, 1, 2), TSG_ADJOINT_ENTRY(20, 1, 2), TSG_ADJOINT_ENTRY(2, 5, 2),
    TSG_ADJOINT_ENTRY(6, 2, 2),  TSG_ADJOINT_ENTRY(4, 5, 2),  TSG_ADJOINT_ENTRY(2, 10, 2),
    TSG_ADJOINT_ENTRY(4, 4, 2),  TSG_ADJOINT_ENTRY(6, 4, 2),  TSG_ADJOINT_ENTRY(4, 8, 2),
    TSG_ADJOINT_ENTRY(8, 8, 2),  TSG_ADJOINT_ENTRY(4, 16, 2), TSG_ADJOINT_ENTRY(4, 32, 2),
    TSG_ADJOINT_ENTRY(10, 2, 2),
};
const int kAdjointW2Count = sizeof(kAdjointW2) / sizeof(kAdjointW2[0]);

const AdjointEntry kAdjointTrajectoryW2[] = {
    TSG_ADJOINT_TRAJECTORY_ENTRY(10, 1, 2), TSG_ADJOINT_TRAJECTORY_ENTRY(20, 1, 2),
    TSG_ADJOINT_TRAJECTORY_ENTRY(2, 5, 2),  TSG_ADJOINT_TRAJECTORY_ENTRY(6, 2, 2),
    TSG_ADJOINT_TRAJECTORY_ENTRY(4, 5, 2),  TSG_ADJOINT_TRAJECTORY_ENTRY(2, 10, 2),
    TSG_ADJOINT_TRAJECTORY_ENTRY(4, 4, 2),  TSG_ADJOINT_TRAJECTORY_ENTRY(6, 4, 2),
    TSG_ADJOINT_TRAJECTORY_ENTRY(4, 8, 2),  TSG_ADJOINT_TRAJECTORY_ENTRY(8, 8, 2),
    TSG_ADJOINT_TRAJECTORY_ENTRY(4, 16, 2), TSG_ADJOINT_TRAJECTORY_ENTRY(4, 32, 2),
    TSG_ADJOINT_TRAJECTORY_ENTRY(10, 2, 2),
};
const int kAdjointTrajectoryW2Count =
    sizeof(kAdjointTrajectoryW2) / sizeof(kAdjointTrajectoryW2[0]);

}  // namespace tsg
