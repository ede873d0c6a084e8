// The adjoint's reduction kernels and the table of reverse-sweep kernels by
// block size. The reverse sweep itself is in epg_adjoint.cuh; its
// instantiations are split over epg_adjoint_w2.cu and epg_adjoint_w4.cu so
// they compile in parallel.
#include "tsg_internal.h"

namespace tsg {

extern const AdjointEntry kAdjointW2[];
extern const int kAdjointW2Count;
extern const AdjointEntry kAdjointW4[];
extern const int kAdjointW4Count;
extern const AdjointEntry kAdjointTrajectoryW2[];
extern const int kAdjointTrajectoryW2Count;
extern const AdjointEntry kAdjointTrajectoryW4[];
extern const int kAdjointTrajectoryW4Count;

const AdjointEntry* adjoint_table(int warps, bool trajectory, int* count) {
    if (warps == 2) {
        *count = trajectory ? kAdjointTrajectoryW2Count : kAdjointW2Count;
        return trajectory ? kAdjointTrajectoryW2 : kAdjointW2;
    }
    if (warps == 4) {
        *count = trajectory ? kAdjointTrajectoryW4Count : kAdjointW4Count;
        return trajectory ? kAdjointTrajectoryW4 : kAdjointW4;
    }
    *count = 0;
    return nullptr;
}

// Sums the per-warp event partials and scatters them to the events the ops
// came from; adds into the outputs. One block per (op, train): each thread
// sums a fixed stride of warps, then a fixed tree over the threads, so the
// sum does not depend on scheduling.
__global__ void __launch_bounds__(kEventReduceThreads)
    reduce_event_gradients(const float2* partial, int64_t warps, int64_t n_ops, int64_t trains,
                           int64_t events, const OpSource* src, float* grad_flip,
                           float* grad_duration) {
    __shared__ float2 s_sum[kEventReduceThreads];
    const int64_t op = blockIdx.x;
    const int64_t t = blockIdx.y;
    const float2* p = partial + t * warps * n_ops + op;
    float2 acc = make_float2(0.f, 0.f);
    for (int64_t w = threadIdx.x; w < warps; w += kEventReduceThreads) {
        const float2 v = p[w * n_ops];
        acc.x += v.x;
        acc.y += v.y;
    }
    s_sum[threadIdx.x] = acc;
    __syncthreads();
    for (int half = kEventReduceThreads / 2; half > 0; half >>= 1) {
        if (threadIdx.x < half) {
            s_sum[threadIdx.x].x += s_sum[threadIdx.x + half].x;
            s_sum[threadIdx.x].y += s_sum[threadIdx.x + half].y;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const OpSource s = src[t * n_ops + op];
        if (grad_flip && s.rf_event >= 0) grad_flip[t * events + s.rf_event] += s_sum[0].x;
        if (grad_duration && s.dt_event >= 0) grad_duration[t * events + s.dt_event] += s_sum[0].y;
    }
}

// Sums the per-train tissue partials in train order; adds into the outputs.
__global__ void reduce_tissue_gradients(const float* partial, int64_t atoms, int64_t trains,
                                        float* g_t1, float* g_t2, float* g_m0, float* g_b1,
                                        float* g_inv) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= atoms) return;
    float v[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    for (int64_t t = 0; t < trains; ++t) {
        const float* p = partial + (t * atoms + i) * 5;
#pragma unroll
        for (int k = 0; k < 5; ++k) v[k] += p[k];
    }
    if (g_t1) g_t1[i] += v[0];
    if (g_t2) g_t2[i] += v[1];
    if (g_m0) g_m0[i] += v[2];
    if (g_b1) g_b1[i] += v[3];
    if (g_inv) g_inv[i] += v[4];
}

}  // namespace tsg
