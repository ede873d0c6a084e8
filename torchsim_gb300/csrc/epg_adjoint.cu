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
// Per segment, the segment's ops are staged in shared memory, and each op's
// transcendentals (sin, cos of the flip, the two relaxation factors) are
// evaluated once per voxel -- lane q of a voxel takes every L-th op -- and
// kept in shared memory for both the re-run and the reverse pass. The
// per-order arithmetic runs on paired FP32 instructions over order pairs, as
// in the forward sweep.
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

__device__ __forceinline__ float2 dup(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

template <int RP, int L>
__device__ __forceinline__ void shift_fwd(float2 (&p)[RP], float2 (&m)[RP], int q, bool kill,
                                          int kill_r) {
    float in_p = 0.f, in_m = 0.f;
    if constexpr (L > 1) {
        in_p = __shfl_up_sync(0xffffffffu, p[RP - 1].y, 1);
        in_m = __shfl_down_sync(0xffffffffu, m[0].x, 1);
    }
    float top = 0.f;
    if constexpr (L > 1) top = (q == L - 1) ? 0.f : in_m;
#pragma unroll
    for (int k = 0; k < RP; ++k) {
        m[k].x = m[k].y;
        m[k].y = (k + 1 < RP) ? m[k + 1].x : top;
    }
    float bottom = -m[0].x;
    if constexpr (L > 1) bottom = (q == 0) ? -m[0].x : in_p;
#pragma unroll
    for (int k = RP - 1; k >= 0; --k) {
        p[k].y = p[k].x;
        p[k].x = (k > 0) ? p[k - 1].y : bottom;
    }
    if (kill) {
#pragma unroll
        for (int k = 0; k < RP; ++k) {
            if (2 * k == kill_r) p[k].x = 0.f;
            if (2 * k + 1 == kill_r) p[k].y = 0.f;
        }
    }
}

// Transpose of shift_fwd: F+ cotangents move one order down, F- cotangents
// one order up, and the F+[0] = -F-[0] coupling returns -pb[0] to mb[1]
// (_epg_cpu.cpp:5950-5971). Order 1 is the second half of the first pair.
template <int RP, int L>
__device__ __forceinline__ void shift_adjoint(float2 (&pb)[RP], float2 (&mb)[RP], int q, bool kill,
                                              int kill_r) {
    const float carry = -pb[0].x;
    float in_p = 0.f, in_m = 0.f;
    if constexpr (L > 1) {
        in_p = __shfl_down_sync(0xffffffffu, pb[0].x, 1);
        in_m = __shfl_up_sync(0xffffffffu, mb[RP - 1].y, 1);
    }
    float top = 0.f;
    if constexpr (L > 1) top = (q == L - 1) ? 0.f : in_p;
#pragma unroll
    for (int k = 0; k < RP; ++k) {
        pb[k].x = pb[k].y;
        pb[k].y = (k + 1 < RP) ? pb[k + 1].x : top;
    }
    float bottom = 0.f;
    if constexpr (L > 1) bottom = (q == 0) ? 0.f : in_m;
#pragma unroll
    for (int k = RP - 1; k >= 0; --k) {
        mb[k].y = mb[k].x;
        mb[k].x = (k > 0) ? mb[k - 1].y : bottom;
    }
    if (q == 0) mb[0].y += carry;
    // The slot at order `states` only receives F- cotangent from below; it
    // must stay empty or it would leak back through the rotation.
    if (kill) {
#pragma unroll
        for (int k = 0; k < RP; ++k) {
            if (2 * k == kill_r) mb[k].x = 0.f;
            if (2 * k + 1 == kill_r) mb[k].y = 0.f;
        }
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

// Dynamic shared memory: ops [C] (16 B each), then per op and voxel slot the
// transcendentals (sin, cos, e1, e2) [C][VPB] float4, then the pre-RF states
// [C][3][RP][T] float2.
template <int RP, int L>
__global__ void __launch_bounds__(256) epg_adjoint_kernel(const AdjointArgs a) {
    extern __shared__ __align__(16) unsigned char s_raw[];
    constexpr int VPW = 32 / L;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int q = lane % L;
    const int slot = lane / L;
    const int T = blockDim.x;
    const int VPB = (T >> 5) * VPW;
    const int vslot = warp * VPW + (slot < VPW ? slot : 0);
    const int64_t warp_global = int64_t(blockIdx.x) * (T >> 5) + warp;
    const int64_t atom = warp_global * VPW + slot;
    const int64_t train = blockIdx.y;
    const bool active = slot < VPW && atom < a.atoms;
    const int64_t ac = active ? atom : 0;
    const int S = a.states;
    const int C = a.ckpt_every;

    Op* s_ops = reinterpret_cast<Op*>(s_raw);
    float4* s_tr = reinterpret_cast<float4*>(s_raw + sizeof(Op) * C);
    float2* s_stage = reinterpret_cast<float2*>(s_raw + sizeof(Op) * C + sizeof(float4) * C * VPB);

    const float t1 = a.t1[ac];
    const float t2 = a.t2[ac];
    const float m0 = a.m0 ? a.m0[ac] : 1.f;
    const float b1 = a.b1 ? a.b1[ac] : 1.f;
    const float eff = a.inv ? a.inv[ac] : 1.f;
    const float r1 = 1000.f / t1;
    const float r2 = 1000.f / t2;
    const float w1 = 1000.f / (t1 * t1);
    const float w2 = 1000.f / (t2 * t2);

    constexpr int R = 2 * RP;
    const bool kill = L * R > S;
    const int kill_r = S - q * R;
    const float2 neg1 = dup(-1.f);

    const Op* ops = a.ops + train * a.n_ops;
    const int64_t row = train * a.atoms + atom;

    float2 P[RP], M[RP], Z[RP];
    float2 pb[RP], mb[RP], zb[RP];
#pragma unroll
    for (int k = 0; k < RP; ++k) pb[k] = mb[k] = zb[k] = dup(0.f);

    float g_t1 = 0.f, g_t2 = 0.f, g_m0 = 0.f, g_b1 = 0.f, g_inv = 0.f;
    float2* event_out = a.event_partial + (train * a.warps_per_train + warp_global) * a.n_ops;

    const int n_seg = (a.n_ops + C - 1) / C;
    for (int seg = n_seg - 1; seg >= 0; --seg) {
        const int o0 = seg * C;
        const int o1 = min(o0 + C, a.n_ops);
        const int cnt = o1 - o0;
        __syncthreads();
        for (int i = threadIdx.x; i < cnt; i += T) s_ops[i] = ops[o0 + i];
        __syncthreads();
        // This segment's transcendentals, one op per lane of each voxel.
        for (int i = q; i < cnt; i += L) {
            const Op op = s_ops[i];
            float si = 0.f, co = 1.f, e1 = 1.f, e2 = 1.f;
            if (op_rf(op.code) == RF_ROTATE) sincosf(op.flip * b1, &si, &co);
            if (op.code & OP_RELAX) {
                e1 = expf(-r1 * op.dt);
                e2 = expf(-r2 * op.dt);
            }
            if (slot < VPW) s_tr[i * VPB + vslot] = make_float4(si, co, e1, e2);
        }
        __syncwarp();
        // Reload the state entering op o0.
        {
            const float* src = a.ckpt + (row * a.ckpt_count + seg) * (3 * int64_t(S));
#pragma unroll
            for (int k = 0; k < RP; ++k) {
                const int o = q * R + 2 * k;
                const bool l0 = active && o < S, l1 = active && o + 1 < S;
                P[k] = make_float2(l0 ? src[o] : 0.f, l1 ? src[o + 1] : 0.f);
                M[k] = make_float2(l0 ? src[S + o] : 0.f, l1 ? src[S + o + 1] : 0.f);
                Z[k] = make_float2(l0 ? src[2 * S + o] : 0.f, l1 ? src[2 * S + o + 1] : 0.f);
            }
        }
        // Forward over the segment, keeping each op's pre-RF state.
        for (int i = 0; i < cnt; ++i) {
            const Op op = s_ops[i];
            const uint32_t code = op.code;
            const float4 tr = s_tr[i * VPB + vslot];
            if (code & OP_RELAX) {
                const float2 E1 = dup(tr.z), E2 = dup(tr.w);
#pragma unroll
                for (int k = 0; k < RP; ++k) {
                    P[k] = mul2(P[k], E2);
                    M[k] = mul2(M[k], E2);
                    Z[k] = mul2(Z[k], E1);
                }
                if (q == 0) Z[0].x += 1.f - tr.z;
            }
            for (int s = 0; s < op_shift1(code); ++s) shift_fwd<RP, L>(P, M, q, kill, kill_r);
            float2* st = s_stage + size_t(i) * 3 * RP * T + threadIdx.x;
#pragma unroll
            for (int k = 0; k < RP; ++k) {
                st[(0 * RP + k) * T] = P[k];
                st[(1 * RP + k) * T] = M[k];
                st[(2 * RP + k) * T] = Z[k];
            }
            const int rf = op_rf(code);
            if (rf == RF_ROTATE) {
                const float si = tr.x, co = tr.y;
                const float2 ch = dup(0.5f * (1.f + co)), sh = dup(0.5f * (1.f - co));
                const float2 hs = dup(0.5f * si), si2 = dup(si), nsi2 = dup(-si), co2 = dup(co);
#pragma unroll
                for (int k = 0; k < RP; ++k) {
                    const float2 p = P[k], m = M[k], z = Z[k];
                    P[k] = fma2(ch, p, fma2(sh, m, mul2(nsi2, z)));
                    M[k] = fma2(sh, p, fma2(ch, m, mul2(si2, z)));
                    Z[k] = fma2(hs, fma2(neg1, m, p), mul2(co2, z));
                }
            } else if (rf == RF_INVERT) {
#pragma unroll
                for (int k = 0; k < RP; ++k) Z[k] = mul2(Z[k], dup(-eff));
            }
            for (int s = 0; s < op_shift2(code); ++s) shift_fwd<RP, L>(P, M, q, kill, kill_r);
            if (code & OP_SPOIL1) {
#pragma unroll
                for (int k = 0; k < RP; ++k) P[k] = M[k] = dup(0.f);
            }
            if ((code & OP_RECORD) && q == 0 && active)
                g_m0 = fmaf(seed_of(a, row * a.outputs + op.record), P[0].x, g_m0);
            for (int s = 0; s < op_shift3(code); ++s) shift_fwd<RP, L>(P, M, q, kill, kill_r);
            if (code & OP_SPOIL2) {
#pragma unroll
                for (int k = 0; k < RP; ++k) P[k] = M[k] = dup(0.f);
            }
        }
        // Reverse over the segment.
        for (int i = cnt - 1; i >= 0; --i) {
            const Op op = s_ops[i];
            const uint32_t code = op.code;
            const float4 tr = s_tr[i * VPB + vslot];
            if (code & OP_SPOIL2) {
#pragma unroll
                for (int k = 0; k < RP; ++k) pb[k] = mb[k] = dup(0.f);
            }
            for (int s = 0; s < op_shift3(code); ++s) shift_adjoint<RP, L>(pb, mb, q, kill, kill_r);
            if ((code & OP_RECORD) && q == 0 && active)
                pb[0].x = fmaf(seed_of(a, row * a.outputs + op.record), m0, pb[0].x);
            if (code & OP_SPOIL1) {
#pragma unroll
                for (int k = 0; k < RP; ++k) pb[k] = mb[k] = dup(0.f);
            }
            for (int s = 0; s < op_shift2(code); ++s) shift_adjoint<RP, L>(pb, mb, q, kill, kill_r);
            const float2* st = s_stage + size_t(i) * 3 * RP * T + threadIdx.x;
            float2 p_[RP], m_[RP], z_[RP];
#pragma unroll
            for (int k = 0; k < RP; ++k) {
                p_[k] = st[(0 * RP + k) * T];
                m_[k] = st[(1 * RP + k) * T];
                z_[k] = st[(2 * RP + k) * T];
            }
            const int rf = op_rf(code);
            float g_flip = 0.f;
            if (rf == RF_ROTATE) {
                const float si = tr.x, co = tr.y;
                const float2 ch = dup(0.5f * (1.f + co)), sh = dup(0.5f * (1.f - co));
                const float2 hs = dup(0.5f * si), nhs = dup(-0.5f * si), hc = dup(0.5f * co);
                const float2 si2 = dup(si), nsi2 = dup(-si), co2 = dup(co);
                float2 ga = dup(0.f);
#pragma unroll
                for (int k = 0; k < RP; ++k) {
                    const float2 w = fma2(neg1, m_[k], p_[k]);
                    const float2 d = fma2(neg1, pb[k], mb[k]);
                    ga = fma2(d, fma2(hs, w, mul2(co2, z_[k])), ga);
                    ga = fma2(zb[k], fma2(hc, w, mul2(nsi2, z_[k])), ga);
                    const float2 npb = fma2(ch, pb[k], fma2(sh, mb[k], mul2(hs, zb[k])));
                    const float2 nmb = fma2(sh, pb[k], fma2(ch, mb[k], mul2(nhs, zb[k])));
                    zb[k] = fma2(si2, d, mul2(co2, zb[k]));
                    pb[k] = npb;
                    mb[k] = nmb;
                }
                const float gsum = ga.x + ga.y;
                g_flip = gsum * b1;
                g_b1 = fmaf(gsum, op.flip, g_b1);
            } else if (rf == RF_INVERT) {
                float2 acc = dup(0.f);
#pragma unroll
                for (int k = 0; k < RP; ++k) {
                    acc = fma2(zb[k], z_[k], acc);
                    zb[k] = mul2(zb[k], dup(-eff));
                }
                g_inv -= acc.x + acc.y;
            }
            float g_dt = 0.f;
            if (code & OP_RELAX) {
                float2 A2 = dup(0.f), A1 = dup(0.f);
#pragma unroll
                for (int k = 0; k < RP; ++k) {
                    A2 = fma2(pb[k], p_[k], fma2(mb[k], m_[k], A2));
                    A1 = fma2(zb[k], z_[k], A1);
                }
                const float a2 = A2.x + A2.y;
                float a1 = A1.x + A1.y;
                if (q == 0) a1 -= zb[0].x;
                g_t2 = fmaf(a2, op.dt * w2, g_t2);
                g_t1 = fmaf(a1, op.dt * w1, g_t1);
                g_dt = -r2 * a2 - r1 * a1;
            }
            for (int s = 0; s < op_shift1(code); ++s) shift_adjoint<RP, L>(pb, mb, q, kill, kill_r);
            if (code & OP_RELAX) {
                const float2 E1 = dup(tr.z), E2 = dup(tr.w);
#pragma unroll
                for (int k = 0; k < RP; ++k) {
                    pb[k] = mul2(pb[k], E2);
                    mb[k] = mul2(mb[k], E2);
                    zb[k] = mul2(zb[k], E1);
                }
            }
            // Event gradients of this op: summed over the warp's voxels.
            const float sf = warp_sum(active ? g_flip : 0.f);
            const float sd = warp_sum(active ? g_dt : 0.f);
            if (lane == 0) event_out[o0 + i] = make_float2(sf, sd);
        }
    }
    // Per-voxel gradients: add the voxel's lanes together (lanes q of one
    // voxel are consecutive; a butterfly over the voxel's group).
    float v[5] = {g_t1, g_t2, g_m0, g_b1, g_inv};
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        float x = active ? v[k] : 0.f;
        float sum = 0.f;
#pragma unroll
        for (int j = 0; j < L; ++j) sum += __shfl_sync(0xffffffffu, x, lane - q + j);
        v[k] = sum;
    }
    if (active && q == 0) {
        float* dst = a.tissue_partial + row * 5;
#pragma unroll
        for (int k = 0; k < 5; ++k) dst[k] = v[k];
    }
}

template <int RP, int L>
void launch_adjoint(const AdjointArgs& a, dim3 grid, dim3 block, size_t smem, cudaStream_t s) {
    epg_adjoint_kernel<RP, L><<<grid, block, smem, s>>>(a);
}

// Entries take orders per lane R (even): the kernel keeps R/2 pairs.
#define TSG_ADJOINT_ENTRY(R, L)                         \
    {R, L, &launch_adjoint<(R) / 2, L>,                 \
     reinterpret_cast<const void*>(&epg_adjoint_kernel<(R) / 2, L>)}

const AdjointEntry kAdjoint[] = {
    TSG_ADJOINT_ENTRY(10, 1), TSG_ADJOINT_ENTRY(20, 1), TSG_ADJOINT_ENTRY(2, 5),
    TSG_ADJOINT_ENTRY(6, 2), TSG_ADJOINT_ENTRY(4, 5), TSG_ADJOINT_ENTRY(2, 10),
    TSG_ADJOINT_ENTRY(4, 4), TSG_ADJOINT_ENTRY(6, 4), TSG_ADJOINT_ENTRY(4, 8),
    TSG_ADJOINT_ENTRY(8, 8), TSG_ADJOINT_ENTRY(4, 16), TSG_ADJOINT_ENTRY(4, 32),
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
