// One persistent launch over many sequences of uneven length, state count and
// voxel count (the reference runs one launch per sequence, each sized to its
// own problem: sequence/_epg_triton.py:17120-17300).
//
// The work list holds (sequence, voxel tile) units, largest first. Each CTA
// takes the next unit from a global counter (one atomicAdd, no waiting on
// other CTAs), stages that sequence's program in shared memory and runs the
// forward sweep for its voxels. Orders per lane (R) are fixed at compile
// time; lanes per voxel (L = ceil(states/R)) are per sequence, so one kernel
// serves every echo-train length: voxels take floor(32/L) slots of a warp and
// the shift's cross-lane moves respect the voxel boundaries through the lane's
// index within its voxel, exactly as in the fixed-shape sweep.
#include "tsg_internal.h"

namespace tsg {

namespace {

constexpr int kBatchOpChunk = 512;

template <int R>
__device__ __forceinline__ void shift_runtime(float (&p)[R], float (&m)[R], int q, int L,
                                              bool kill, int kill_r) {
    const float in_p = __shfl_up_sync(0xffffffffu, p[R - 1], 1);
    const float in_m = __shfl_down_sync(0xffffffffu, m[0], 1);
#pragma unroll
    for (int r = 0; r < R - 1; ++r) m[r] = m[r + 1];
#pragma unroll
    for (int r = R - 1; r > 0; --r) p[r] = p[r - 1];
    m[R - 1] = (q == L - 1) ? 0.f : in_m;
    p[0] = (q == 0) ? -m[0] : in_p;
    if (kill) {
#pragma unroll
        for (int r = 0; r < R; ++r)
            if (r == kill_r) p[r] = 0.f;
    }
}

}  // namespace

template <int R>
__global__ void __launch_bounds__(256) epg_batched_kernel(
    const Op* __restrict__ ops, const tsg_batch_sequence* __restrict__ seqs,
    const tsg_batch_unit* __restrict__ units, int64_t unit_count, int* __restrict__ counter,
    const float* __restrict__ t1v, const float* __restrict__ t2v, const float* __restrict__ m0v,
    const float* __restrict__ b1v, float2* __restrict__ out) {
    __shared__ Op s_ops[kBatchOpChunk];
    __shared__ int s_unit;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    while (true) {
        __syncthreads();
        if (threadIdx.x == 0) s_unit = atomicAdd(counter, 1);
        __syncthreads();
        const int64_t unit_index = s_unit;
        if (unit_index >= unit_count) break;
        const tsg_batch_unit u = units[unit_index];
        const tsg_batch_sequence sq = seqs[u.sequence];
        const int L = sq.lanes_per_voxel;
        const int vpw = 32 / L;
        const int q = lane % L;
        const int slot = lane / L;
        const int local = (warp * vpw + slot);
        const bool active = slot < vpw && local < u.voxel_count;
        const int64_t voxel = sq.voxel_offset + u.voxel_begin + (active ? local : 0);
        const float t1 = t1v[voxel];
        const float t2 = t2v[voxel];
        const float m0 = m0v ? m0v[voxel] : 1.f;
        const float b1 = b1v ? b1v[voxel] : 1.f;
        const float r1 = 1000.f / t1;
        const float r2 = 1000.f / t2;
        const int S = sq.states;
        const bool kill = L * R > S;
        const int kill_r = S - q * R;
        float P[R], M[R], Z[R];
#pragma unroll
        for (int r = 0; r < R; ++r) P[r] = M[r] = Z[r] = 0.f;
        if (q == 0) Z[0] = 1.f;
        float last_dt = __int_as_float(0x7fffffff);
        float e1 = 1.f, e2 = 1.f;
        float2* orow = out + sq.output_offset + int64_t(u.voxel_begin + local) * sq.outputs;
        for (int base = 0; base < sq.op_count; base += kBatchOpChunk) {
            const int count = min(kBatchOpChunk, sq.op_count - base);
            __syncthreads();
            for (int i = threadIdx.x; i < count; i += blockDim.x)
                s_ops[i] = ops[sq.op_offset + base + i];
            __syncthreads();
            for (int i = 0; i < count; ++i) {
                const Op op = s_ops[i];
                const uint32_t code = op.code;
                if (code & OP_RELAX) {
                    if (op.dt != last_dt) {
                        last_dt = op.dt;
                        e1 = expf(-r1 * op.dt);
                        e2 = expf(-r2 * op.dt);
                    }
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        P[r] *= e2;
                        M[r] *= e2;
                        Z[r] *= e1;
                    }
                    if (q == 0) Z[0] += 1.f - e1;
                }
                for (int s = 0; s < op_shift1(code); ++s) shift_runtime<R>(P, M, q, L, kill, kill_r);
                const int rf = op_rf(code);
                if (rf == RF_ROTATE) {
                    float si, co;
                    sincosf(op.flip * b1, &si, &co);
                    const float ch = 0.5f * (1.f + co), sh = 0.5f * (1.f - co), hs = 0.5f * si;
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        const float p = P[r], m = M[r], z = Z[r];
                        P[r] = fmaf(ch, p, fmaf(sh, m, -si * z));
                        M[r] = fmaf(sh, p, fmaf(ch, m, si * z));
                        Z[r] = fmaf(hs, p - m, co * z);
                    }
                } else if (rf == RF_INVERT) {
#pragma unroll
                    for (int r = 0; r < R; ++r) Z[r] = -Z[r];
                }
                for (int s = 0; s < op_shift2(code); ++s) shift_runtime<R>(P, M, q, L, kill, kill_r);
                if (code & OP_SPOIL1) {
#pragma unroll
                    for (int r = 0; r < R; ++r) P[r] = M[r] = 0.f;
                }
                if ((code & OP_RECORD) && q == 0 && active)
                    __stcs(orow + op.record, make_float2(0.f, m0 * P[0]));
                for (int s = 0; s < op_shift3(code); ++s) shift_runtime<R>(P, M, q, L, kill, kill_r);
                if (code & OP_SPOIL2) {
#pragma unroll
                    for (int r = 0; r < R; ++r) P[r] = M[r] = 0.f;
                }
            }
        }
    }
}

}  // namespace tsg

using namespace tsg;

extern "C" int tsg_epg_batched_forward(const void* ops, const tsg_batch_sequence* sequences,
                                       const tsg_batch_unit* units, int64_t unit_count,
                                       int32_t* counter, const tsg_tissue* tissue, void* out,
                                       int orders_per_lane, int warps_per_block, int blocks,
                                       void* stream) {
    if (unit_count < 0 || (unit_count > 0 && (!ops || !sequences || !units || !counter || !out)))
        return fail(TSG_ERR_ARGUMENT, "null batch buffer");
    if (!tissue || (unit_count > 0 && (!tissue->t1_ms || !tissue->t2_ms)))
        return fail(TSG_ERR_ARGUMENT, "t1 and t2 are required");
    if (tissue->inversion) return fail(TSG_ERR_UNSUPPORTED, "batched sequences take no inversion map");
    if (warps_per_block < 1 || warps_per_block > 8 || blocks < 1)
        return fail(TSG_ERR_ARGUMENT, "invalid persistent launch shape");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    TSG_CUDA(cudaMemsetAsync(counter, 0, sizeof(int32_t), s));
    if (unit_count == 0) return TSG_OK;
    const Op* o = static_cast<const Op*>(ops);
    float2* y = static_cast<float2*>(out);
    const dim3 grid{unsigned(blocks)}, block{unsigned(32 * warps_per_block)};
    switch (orders_per_lane) {
        case 2:
            epg_batched_kernel<2><<<grid, block, 0, s>>>(o, sequences, units, unit_count, counter,
                                                          tissue->t1_ms, tissue->t2_ms, tissue->m0,
                                                          tissue->b1, y);
            break;
        case 4:
            epg_batched_kernel<4><<<grid, block, 0, s>>>(o, sequences, units, unit_count, counter,
                                                          tissue->t1_ms, tissue->t2_ms, tissue->m0,
                                                          tissue->b1, y);
            break;
        case 8:
            epg_batched_kernel<8><<<grid, block, 0, s>>>(o, sequences, units, unit_count, counter,
                                                          tissue->t1_ms, tissue->t2_ms, tissue->m0,
                                                          tissue->b1, y);
            break;
        default:
            return fail(TSG_ERR_UNSUPPORTED, "orders_per_lane must be 2, 4 or 8");
    }
    TSG_CUDA(cudaGetLastError());
    return TSG_OK;
}
