// Reverse-sweep kernels with 4 warps per block (orders per lane, lanes per
// voxel), checkpointed and trajectory mode.
#include "epg_adjoint.cuh"

namespace tsg {

extern const AdjointEntry kAdjointW4[];
extern const int kAdjointW4Count;
extern const AdjointEntry kAdjointTrajectoryW4[];
extern const int kAdjointTrajectoryW4Count;

const AdjointEntry kAdjointW4[] = {
    TSG_ADJOINT_ENTRY(10, 1, 4), TSG_ADJOINT_ENTRY(20, 1, 4), TSG_ADJOINT_ENTRY(2, 5, 4),
    TSG_ADJOINT_ENTRY(6, 2, 4),  TSG_ADJOINT_ENTRY(4, 5, 4),  TSG_ADJOINT_ENTRY(2, 10, 4),
    TSG_ADJOINT_ENTRY(4, 4, 4),  TSG_ADJOINT_ENTRY(6, 4, 4),  TSG_ADJOINT_ENTRY(4, 8, 4),
    TSG_ADJOINT_ENTRY(8, 8, 4),  TSG_ADJOINT_ENTRY(4, 16, 4), TSG_ADJOINT_ENTRY(4, 32, 4),
    TSG_ADJOINT_ENTRY(10, 2, 4),
};
const int kAdjointW4Count = sizeof(kAdjointW4) / sizeof(kAdjointW4[0]);

const AdjointEntry kAdjointTrajectoryW4[] = {
    TSG_ADJOINT_TRAJECTORY_ENTRY(10, 1, 4), TSG_ADJOINT_TRAJECTORY_ENTRY(20, 1, 4),
    TSG_ADJOINT_TRAJECTORY_ENTRY(2, 5, 4),  TSG_ADJOINT_TRAJECTORY_ENTRY(6, 2, 4),
    TSG_ADJOINT_TRAJECTORY_ENTRY(4, 5, 4),  TSG_ADJOINT_TRAJECTORY_ENTRY(2, 10, 4),
    TSG_ADJOINT_TRAJECTORY_ENTRY(4, 4, 4),  TSG_ADJOINT_TRAJECTORY_ENTRY(6, 4, 4),
    TSG_ADJOINT_TRAJECTORY_ENTRY(4, 8, 4),  TSG_ADJOINT_TRAJECTORY_ENTRY(8, 8, 4),
    TSG_ADJOINT_TRAJECTORY_ENTRY(4, 16, 4), TSG_ADJOINT_TRAJECTORY_ENTRY(4, 32, 4),
    TSG_ADJOINT_TRAJECTORY_ENTRY(10, 2, 4),
};
const int kAdjointTrajectoryW4Count =
    sizeof(kAdjointTrajectoryW4) / sizeof(kAdjointTrajectoryW4[0]);

}  // namespace tsg
