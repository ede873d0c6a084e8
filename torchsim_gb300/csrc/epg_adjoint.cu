// The checkpointed first-order adjoint of the real-subspace EPG sweep.
//
// The reference records the entry state of EVERY event and sweeps back over
// that trajectory (src/torchsim/_epg_cpu.cpp:5985-6232; on the GPU in waves
// of 256 MiB, sequence/_epg_triton.py:17604-17612). Here the forward sweep
// stores the state only every C ops (the checkpoints); the reverse sweep
// walks the segments from last to first: it reloads a segment's checkpoint,
// re-runs the segment forward keeping each op's pre-RF state in shared
// memory, and then applies the transposed micro-steps op by op in reverse.
//
// Gradient algebra per op (the reference's, rearranged so that only the
// pre-RF state is kept): with the cotangent taken at the pre-RF point,
//   A2 = sum(pb*p + mb*m),  A1 = sum(zb*z) - zb[0]
// are E2*dL/dE2 and E1*dL/dE1 of the op's relaxation (a shift between the
// relaxation and the pulse leaves these inner products unchanged), so
//   dL/dT2 += A2*dt*1000/T2^2, dL/dT1 += A1*dt*1000/T1^2,
//   dL/d(duration) = -R2*A2 - R1*A1.
// The rotation's cotangent and dL/dalpha follow _epg_cpu.cpp:6140-6183.
//
// Per-event gradients (flip, duration) are summed over a warp's voxels with
// shuffles and written per warp; a second kernel adds the warps up in a fixed
// order, so the result does not depend on scheduling (no atomics).
#include "tsg_internal.h"

namespace tsg {

namespace {

// Transpose of shift_pair: F+ cotangents move one order down, F- cotangents
// one order up, and the F+[0] = -F-[0] coupling returns -pb[0] to mb[1]
// (_epg_cpu.cpp:5950-5971). Requires R >= 2.
template <int R, int L>
__device__ __forceinline__ void shift_pair_adjoint(float (&pb)[R], float (&mb)[R], int q,
                                                   bool kill, int kill_r) {
    static_assert(R >= 2, "the adjoint keeps at least two orders per lane");
    const float carry = -pb[0];
    float in_p = 0.f, in_m = 0.f;
    if constexpr (L > 1) {
        in_p = __shfl_down_sync(0xffffffffu, pb[0], 1);
        in_m = __shfl_up_sync(0xffffffffu, mb[R - 1], 1);
    }
#pragma unroll
    for (int r = 0; r < R - 1; ++r) pb[r] = pb[r + 1];
#pragma unroll
    for (int r = R - 1; r > 0; --r) mb[r] = mb[r - 1];
    if constexpr (L > 1) {
        pb[R - 1] = (q == L - 1) ? 0.f : in_p;
        mb[0] = (q == 0) ? 0.f : in_m;
    } else {
        pb[R - 1] = 0.f;
        mb[0] = 0.f;
    }
    if (q == 0) mb[1] += carry;
    // The slot at order `states` only receives F- cotangent from below; it
    // must stay empty or it would leak back through the rotation.
    if (kill) {
#pragma unroll
        for (int r = 0; r < R; ++r)
            if (r == kill_r) mb[r] = 0.f;
    }
}

template <int R, int L>
__device__ __forceinline__ void shift_pair_fwd(float (&p)[R], float (&m)[R], int q, bool kill,
                                               int kill_r) {
    float in_p = 0.f, in_m = 0.f;
    if constexpr (L > 1) {
        in_p = __shfl_up_sync(0xffffffffu, p[R - 1], 1);
        in_m = __shfl_down_sync(0xffffffffu, m[0], 1);
    }
#pragma unroll
    for (int r = 0; r < R - 1; ++r) m[r] = m[r + 1];
#pragma unroll
    for (int r = R - 1; r > 0; --r) p[r] = p[r - 1];
    if constexpr (L > 1) {
        m[R - 1] = (q == L - 1) ? 0.f : in_m;
        p[0] = (q == 0) ? -m[0] : in_p;
    } else {
        m[R - 1] = 0.f;
        p[0] = -m[0];
    }
    if (kill) {
#pragma unroll
        for (int r = 0; r < R; ++r)
            if (r == kill_r) p[r] = 0.f;
    }
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

__device__ __forceinline__ float seed_of(const AdjointArgs& a, int64_t idx) {
    if (a.seed_layout == TSG_LAYOUT_PLANES) return a.seed[idx];
    // 1j * (i v) = -v: the cotangent of v is minus the real part.
    return -a.seed[2 * idx];
}

}  // namespace

template <int R, int L>
__global__ void __launch_bounds__(256) epg_adjoint_kernel(const AdjointArgs a) {
    extern __shared__ float s_stage[];  // [C][3][R][blockDim]
    constexpr int VPW = 32 / L;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int q = lane % L;
    const int64_t warp_global = int64_t(blockIdx.x) * (blockDim.x >> 5) + warp;
    const int64_t atom = warp_global * VPW + lane / L;
    const int64_t train = blockIdx.y;
    const bool active = atom < a.atoms;
    const int64_t ac = active ? atom : 0;
    const int S = a.states;
    const int C = a.ckpt_every;
    const int T = blockDim.x;

    const float t1 = a.t1[ac];
    const float t2 = a.t2[ac];
    const float m0 = a.m0 ? a.m0[ac] : 1.f;
    const float b1 = a.b1 ? a.b1[ac] : 1.f;
    const float eff = a.inv ? a.inv[ac] : 1.f;
    const float r1 = 1000.f / t1;
    const float r2 = 1000.f / t2;
    const float w1 = 1000.f / (t1 * t1);
    const float w2 = 1000.f / (t2 * t2);

    const bool kill = L * R > S;
    const int kill_r = S - q * R;

    const Op* ops = a.ops + train * a.n_ops;
    const int64_t row = train * a.atoms + atom;
    const float* seeds = a.seed;
    (void)seeds;

    float P[R], M[R], Z[R];
    float pb[R], mb[R], zb[R];
#pragma unroll
    for (int r = 0; r < R; ++r) pb[r] = mb[r] = zb[r] = 0.f;

    float g_t1 = 0.f, g_t2 = 0.f, g_m0 = 0.f, g_b1 = 0.f, g_inv = 0.f;
    float2* event_out = a.event_partial + (train * a.warps_per_train + warp_global) * a.n_ops;

    const int n_seg = (a.n_ops + C - 1) / C;
    for (int seg = n_seg - 1; seg >= 0; --seg) {
        const int o0 = seg * C;
        const int o1 = min(o0 + C, a.n_ops);
        // Reload the state entering op o0.
        {
            const float* src = a.ckpt + (row * a.ckpt_count + seg) * (3 * int64_t(S));
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int o = q * R + r;
                const bool live = active && o < S;
                P[r] = live ? src[o] : 0.f;
                M[r] = live ? src[S + o] : 0.f;
                Z[r] = live ? src[2 * S + o] : 0.f;
            }
        }
        // Forward over the segment, keeping each op's pre-RF state.
        float last_dt = __int_as_float(0x7fffffff);
        float e1 = 1.f, e2 = 1.f;
        for (int i = o0; i < o1; ++i) {
            const Op op = ops[i];
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
            for (int s = 0; s < op_shift1(code); ++s) shift_pair_fwd<R, L>(P, M, q, kill, kill_r);
            float* st = s_stage + size_t(i - o0) * 3 * R * T + threadIdx.x;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                st[(0 * R + r) * T] = P[r];
                st[(1 * R + r) * T] = M[r];
                st[(2 * R + r) * T] = Z[r];
            }
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
                for (int r = 0; r < R; ++r) Z[r] *= -eff;
            }
            for (int s = 0; s < op_shift2(code); ++s) shift_pair_fwd<R, L>(P, M, q, kill, kill_r);
            if (code & OP_SPOIL1) {
#pragma unroll
                for (int r = 0; r < R; ++r) P[r] = M[r] = 0.f;
            }
            if ((code & OP_RECORD) && q == 0 && active)
                g_m0 = fmaf(seed_of(a, row * a.outputs + op.record), P[0], g_m0);
            for (int s = 0; s < op_shift3(code); ++s) shift_pair_fwd<R, L>(P, M, q, kill, kill_r);
            if (code & OP_SPOIL2) {
#pragma unroll
                for (int r = 0; r < R; ++r) P[r] = M[r] = 0.f;
            }
        }
        // Reverse over the segment.
        last_dt = __int_as_float(0x7fffffff);
        for (int i = o1 - 1; i >= o0; --i) {
            const Op op = ops[i];
            const uint32_t code = op.code;
            if (code & OP_SPOIL2) {
#pragma unroll
                for (int r = 0; r < R; ++r) pb[r] = mb[r] = 0.f;
            }
            for (int s = 0; s < op_shift3(code); ++s)
                shift_pair_adjoint<R, L>(pb, mb, q, kill, kill_r);
            if ((code & OP_RECORD) && q == 0 && active)
                pb[0] = fmaf(seed_of(a, row * a.outputs + op.record), m0, pb[0]);
            if (code & OP_SPOIL1) {
#pragma unroll
                for (int r = 0; r < R; ++r) pb[r] = mb[r] = 0.f;
            }
            for (int s = 0; s < op_shift2(code); ++s)
                shift_pair_adjoint<R, L>(pb, mb, q, kill, kill_r);
            const float* st = s_stage + size_t(i - o0) * 3 * R * T + threadIdx.x;
            float p_[R], m_[R], z_[R];
#pragma unroll
            for (int r = 0; r < R; ++r) {
                p_[r] = st[(0 * R + r) * T];
                m_[r] = st[(1 * R + r) * T];
                z_[r] = st[(2 * R + r) * T];
            }
            const int rf = op_rf(code);
            float g_flip = 0.f;
            if (rf == RF_ROTATE) {
                float si, co;
                sincosf(op.flip * b1, &si, &co);
                const float ch = 0.5f * (1.f + co), sh = 0.5f * (1.f - co);
                const float hs = 0.5f * si, hc = 0.5f * co;
                float ga = 0.f;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const float w = p_[r] - m_[r];
                    const float d = mb[r] - pb[r];
                    ga = fmaf(d, fmaf(hs, w, co * z_[r]), ga);
                    ga = fmaf(zb[r], fmaf(hc, w, -si * z_[r]), ga);
                    const float npb = fmaf(ch, pb[r], fmaf(sh, mb[r], hs * zb[r]));
                    const float nmb = fmaf(sh, pb[r], fmaf(ch, mb[r], -hs * zb[r]));
                    zb[r] = fmaf(si, d, co * zb[r]);
                    pb[r] = npb;
                    mb[r] = nmb;
                }
                g_flip = ga * b1;
                g_b1 = fmaf(ga, op.flip, g_b1);
            } else if (rf == RF_INVERT) {
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    g_inv = fmaf(-zb[r], z_[r], g_inv);
                    zb[r] *= -eff;
                }
            }
            float g_dt = 0.f;
            if (code & OP_RELAX) {
                if (op.dt != last_dt) {
                    last_dt = op.dt;
                    e1 = expf(-r1 * op.dt);
                    e2 = expf(-r2 * op.dt);
                }
                float A2 = 0.f, A1 = 0.f;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    A2 = fmaf(pb[r], p_[r], fmaf(mb[r], m_[r], A2));
                    A1 = fmaf(zb[r], z_[r], A1);
                }
                if (q == 0) A1 -= zb[0];
                g_t2 = fmaf(A2, op.dt * w2, g_t2);
                g_t1 = fmaf(A1, op.dt * w1, g_t1);
                g_dt = -r2 * A2 - r1 * A1;
            }
            for (int s = 0; s < op_shift1(code); ++s)
                shift_pair_adjoint<R, L>(pb, mb, q, kill, kill_r);
            if (code & OP_RELAX) {
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    pb[r] *= e2;
                    mb[r] *= e2;
                    zb[r] *= e1;
                }
            }
            // Event gradients of this op: summed over the warp's voxels.
            const float sf = warp_sum(active ? g_flip : 0.f);
            const float sd = warp_sum(active ? g_dt : 0.f);
            if (lane == 0) event_out[i] = make_float2(sf, sd);
        }
        __syncwarp();
    }
    // Per-voxel gradients: add the voxel's lanes together.
    float v[5] = {g_t1, g_t2, g_m0, g_b1, g_inv};
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        float x = active ? v[k] : 0.f;
#pragma unroll
        for (int off = 1; off < L; off <<= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
        v[k] = x;
    }
    if (active && q == 0) {
        float* dst = a.tissue_partial + row * 5;
#pragma unroll
        for (int k = 0; k < 5; ++k) dst[k] = v[k];
    }
}

template <int R, int L>
void launch_adjoint(const AdjointArgs& a, dim3 grid, dim3 block, size_t smem, cudaStream_t s) {
    epg_adjoint_kernel<R, L><<<grid, block, smem, s>>>(a);
}

#define TSG_ADJOINT_ENTRY(R, L) \
    {R, L, &launch_adjoint<R, L>, reinterpret_cast<const void*>(&epg_adjoint_kernel<R, L>)}

const AdjointEntry kAdjoint[] = {
    TSG_ADJOINT_ENTRY(10, 1), TSG_ADJOINT_ENTRY(20, 1), TSG_ADJOINT_ENTRY(5, 2),
    TSG_ADJOINT_ENTRY(10, 2), TSG_ADJOINT_ENTRY(4, 4), TSG_ADJOINT_ENTRY(5, 4),
    TSG_ADJOINT_ENTRY(8, 4), TSG_ADJOINT_ENTRY(4, 8), TSG_ADJOINT_ENTRY(4, 16),
    TSG_ADJOINT_ENTRY(8, 16), TSG_ADJOINT_ENTRY(4, 32),
};
const int kAdjointCount = sizeof(kAdjoint) / sizeof(kAdjoint[0]);

// Sums the per-warp event partials in warp order and scatters them to the
// events the ops came from; adds into the outputs.
__global__ void reduce_event_gradients(const float2* partial, int64_t warps, int64_t n_ops,
                                       int64_t trains, int64_t events, const OpSource* src,
                                       float* grad_flip, float* grad_duration) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n_ops * trains) return;
    const int64_t t = i / n_ops;
    const int64_t op = i % n_ops;
    float f = 0.f, d = 0.f;
    const float2* p = partial + t * warps * n_ops + op;
    for (int64_t w = 0; w < warps; ++w) {
        const float2 v = p[w * n_ops];
        f += v.x;
        d += v.y;
    }
    const OpSource s = src[i];
    if (grad_flip && s.rf_event >= 0) grad_flip[t * events + s.rf_event] += f;
    if (grad_duration && s.dt_event >= 0) grad_duration[t * events + s.dt_event] += d;
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
