// The per-voxel EPG sweep: one pass over a compiled pulse program that
// carries the F+/F-/Z state of every voxel in registers for the whole
// sequence, optionally with forward-mode tangents beside it.
//
// Thread mapping: a voxel's configuration orders are spread over L warp lanes
// (lanes_per_voxel), R consecutive orders per lane (orders_per_lane), so a
// warp holds 32/L voxels. The gradient shift moves F+ one order up and F- one
// order down; within a lane that is a register move, across lanes a warp
// shuffle. The program (ops) is staged in shared memory and read as a
// broadcast, since every voxel of a block follows the same train.
//
// Semantics follow the reference's real-subspace kernels: relaxation with
// recovery, the real 3x3 RF rotation in alpha = flip*B1, inversion Z *= -eff,
// the shift with F+[0] = -F-[0] and truncation at `states` orders, spoiling,
// and the record m0*F+[0] (src/torchsim/_epg_cpu.cpp:3010-3128 forward,
// :3136-3285 tangent).
#pragma once

#include "tsg_internal.h"

namespace tsg {

template <int TM, bool GEN>
struct SystemLayout {
    static constexpr bool T1 = (TM & TSG_TANGENT_T1) != 0;
    static constexpr bool T2 = (TM & TSG_TANGENT_T2) != 0;
    static constexpr bool B1 = (TM & TSG_TANGENT_B1) != 0;
    static constexpr bool INV = (TM & TSG_TANGENT_INVERSION) != 0;
    static constexpr int I_T1 = 0;
    static constexpr int I_T2 = I_T1 + (T1 ? 1 : 0);
    static constexpr int I_B1 = I_T2 + (T2 ? 1 : 0);
    static constexpr int I_INV = I_B1 + (B1 ? 1 : 0);
    static constexpr int I_GEN = I_INV + (INV ? 1 : 0);
    static constexpr int N = I_GEN + (GEN ? 1 : 0);
    static constexpr int NA = N > 0 ? N : 1;
};

// One gradient shift of a (F+, F-) pair spread over L lanes of R orders.
template <int R, int L>
__device__ __forceinline__ void shift_pair(float (&p)[R], float (&m)[R], int q, bool kill,
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
    // Orders at and above `states` stay empty: the only way in is F+ moving
    // up from the top kept order, so that one slot is cleared after a shift.
    if (kill) {
#pragma unroll
        for (int r = 0; r < R; ++r)
            if (r == kill_r) p[r] = 0.f;
    }
}

__device__ __forceinline__ void put_sample(int layout, float* a, float* b, int64_t idx, float v) {
    if (layout == TSG_LAYOUT_PLANES) {
        if (a) __stcs(a + idx, 0.f);
        __stcs(b + idx, v);
    } else if (layout == TSG_LAYOUT_COMPLEX) {
        __stcs(reinterpret_cast<float2*>(a) + idx, make_float2(0.f, v));
    } else {
        __stcs(reinterpret_cast<float2*>(a) + idx, make_float2(-v, 0.f));
    }
}

template <int R, int L, int TM, bool GEN, bool GN = false>
__global__ void __launch_bounds__(256) epg_sweep_kernel(const SweepArgs a) {
    using S = SystemLayout<TM, GEN>;
    constexpr int NT = S::N;
    constexpr int VPW = 32 / L;
    __shared__ Op s_ops[kOpChunk];
    __shared__ float2 s_dir[GEN ? kOpChunk : 1];

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int q = lane % L;
    const int64_t atom = (int64_t(blockIdx.x) * (blockDim.x >> 5) + warp) * VPW + lane / L;
    const int64_t train = blockIdx.y;
    const bool active = atom < a.atoms;
    const int64_t ac = active ? atom : 0;

    const float t1 = a.t1[ac];
    const float t2 = a.t2[ac];
    const float m0 = a.m0 ? a.m0[ac] : 1.f;
    const float b1 = a.b1 ? a.b1[ac] : 1.f;
    const float eff = a.inv ? a.inv[ac] : 1.f;
    const float r1 = 1000.f / t1;
    const float r2 = 1000.f / t2;
    // dE/dT = E * 1000 dt / T^2 for E = exp(-1000 dt / T).
    const float w1 = 1000.f / (t1 * t1);
    const float w2 = 1000.f / (t2 * t2);
    float g_t1 = 0.f, g_t2 = 0.f, g_m0 = 0.f, g_b1 = 0.f, g_inv = 0.f;
    if constexpr (GEN) {
        g_t1 = a.g_t1 ? a.g_t1[ac] : 0.f;
        g_t2 = a.g_t2 ? a.g_t2[ac] : 0.f;
        g_m0 = a.g_m0 ? a.g_m0[ac] : 0.f;
        g_b1 = (a.g_b1 && a.b1) ? a.g_b1[ac] : 0.f;
        g_inv = (a.g_inv && a.inv) ? a.g_inv[ac] : 0.f;
    }

    const bool kill = L * R > a.states;
    const int kill_r = a.states - q * R;

    float P[R], M[R], Z[R];
    float dP[S::NA][R], dM[S::NA][R], dZ[S::NA][R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        P[r] = M[r] = Z[r] = 0.f;
#pragma unroll
        for (int j = 0; j < S::NA; ++j) dP[j][r] = dM[j][r] = dZ[j][r] = 0.f;
    }
    if (q == 0) Z[0] = 1.f;

    float last_dt = __int_as_float(0x7fffffff);  // NaN: first relax computes
    float e1 = 1.f, e2 = 1.f, k1 = 0.f, k2 = 0.f;

    // Gauss-Newton sums: float over chunks of 32 samples, then into doubles.
    static_assert(!GN || (S::T1 && S::T2), "GN sweeps carry the T1 and T2 tangents");
    float cs[10];
    double cd[10];
    int in_chunk = 0;
#pragma unroll
    for (int k = 0; k < 10; ++k) {
        cs[k] = 0.f;
        cd[k] = 0.0;
    }
    const float2* yrow = nullptr;
    if constexpr (GN) {
        const int64_t mrow = a.measured_rows ? a.measured_rows[ac] : (train * a.atoms + ac);
        yrow = a.measured + mrow * a.outputs;
    }

    const Op* ops = a.ops + train * a.n_ops;
    const float2* dirs = GEN ? a.op_dir + train * a.n_ops : nullptr;
    const int64_t row = train * a.atoms + atom;

    for (int base = 0; base < a.n_ops; base += kOpChunk) {
        const int count = min(kOpChunk, a.n_ops - base);
        __syncthreads();
        for (int i = threadIdx.x; i < count; i += blockDim.x) {
            s_ops[i] = ops[base + i];
            if constexpr (GEN) s_dir[i] = dirs[base + i];
        }
        __syncthreads();
        for (int i = 0; i < count; ++i) {
            const Op op = s_ops[i];
            const uint32_t code = op.code;
            if (a.ckpt != nullptr && ((base + i) % a.ckpt_every) == 0 && active) {
                // State entering this op, for the adjoint's segments.
                const int k = (base + i) / a.ckpt_every;
                const int S = a.states;
                float* dst = a.ckpt + (row * a.ckpt_count + k) * (3 * int64_t(S));
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const int o = q * R + r;
                    if (o < S) {
                        dst[o] = P[r];
                        dst[S + o] = M[r];
                        dst[2 * S + o] = Z[r];
                    }
                }
            }
            float ddt = 0.f, dfl = 0.f;
            if constexpr (GEN) {
                ddt = s_dir[i].x;
                dfl = s_dir[i].y;
            }
            const int rf = op_rf(code);
            const bool relax = (code & OP_RELAX) != 0;
            if (relax && op.dt != last_dt) {
                last_dt = op.dt;
                e1 = expf(-r1 * op.dt);
                e2 = expf(-r2 * op.dt);
                k1 = e1 * (op.dt * w1);
                k2 = e2 * (op.dt * w2);
            }
            const int n1 = op_shift1(code);
            if constexpr (NT == 0) {
                if (relax && rf == RF_ROTATE && n1 == 0) {
                    // Relaxation folded into the rotation: one 3x3 per order
                    // with the recovery of order 0 added after.
                    const float alpha = op.flip * b1;
                    float si, co;
                    sincosf(alpha, &si, &co);
                    const float ch = 0.5f * (1.f + co), sh = 0.5f * (1.f - co), hs = 0.5f * si;
                    const float cpp = ch * e2, cpm = sh * e2, cpz = si * e1;
                    const float czp = hs * e2, czz = co * e1;
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        const float p = P[r], m = M[r], z = Z[r];
                        P[r] = fmaf(cpp, p, fmaf(cpm, m, -cpz * z));
                        M[r] = fmaf(cpm, p, fmaf(cpp, m, cpz * z));
                        Z[r] = fmaf(czp, p - m, czz * z);
                    }
                    if (q == 0) {
                        const float rec = 1.f - e1;
                        P[0] = fmaf(-si, rec, P[0]);
                        M[0] = fmaf(si, rec, M[0]);
                        Z[0] = fmaf(co, rec, Z[0]);
                    }
                    goto after_rf;
                }
            }
            if (relax) {
                float e1g = 0.f, e2g = 0.f;
                if constexpr (GEN) {
                    e1g = e1 * (op.dt * g_t1 * w1 - r1 * ddt);
                    e2g = e2 * (op.dt * g_t2 * w2 - r2 * ddt);
                }
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    if constexpr (S::T1) {
                        dP[S::I_T1][r] *= e2;
                        dM[S::I_T1][r] *= e2;
                        dZ[S::I_T1][r] = fmaf(dZ[S::I_T1][r], e1, Z[r] * k1);
                    }
                    if constexpr (S::T2) {
                        dP[S::I_T2][r] = fmaf(dP[S::I_T2][r], e2, P[r] * k2);
                        dM[S::I_T2][r] = fmaf(dM[S::I_T2][r], e2, M[r] * k2);
                        dZ[S::I_T2][r] *= e1;
                    }
                    if constexpr (S::B1) {
                        dP[S::I_B1][r] *= e2;
                        dM[S::I_B1][r] *= e2;
                        dZ[S::I_B1][r] *= e1;
                    }
                    if constexpr (S::INV) {
                        dP[S::I_INV][r] *= e2;
                        dM[S::I_INV][r] *= e2;
                        dZ[S::I_INV][r] *= e1;
                    }
                    if constexpr (GEN) {
                        dP[S::I_GEN][r] = fmaf(dP[S::I_GEN][r], e2, P[r] * e2g);
                        dM[S::I_GEN][r] = fmaf(dM[S::I_GEN][r], e2, M[r] * e2g);
                        dZ[S::I_GEN][r] = fmaf(dZ[S::I_GEN][r], e1, Z[r] * e1g);
                    }
                    P[r] *= e2;
                    M[r] *= e2;
                    Z[r] *= e1;
                }
                if (q == 0) {
                    Z[0] += 1.f - e1;
                    if constexpr (S::T1) dZ[S::I_T1][0] -= k1;
                    if constexpr (GEN) dZ[S::I_GEN][0] -= e1g;
                }
            }
            for (int s = 0; s < n1; ++s) {
                shift_pair<R, L>(P, M, q, kill, kill_r);
#pragma unroll
                for (int j = 0; j < NT; ++j) shift_pair<R, L>(dP[j], dM[j], q, kill, kill_r);
            }
            if (rf == RF_ROTATE) {
                const float alpha = op.flip * b1;
                float si, co;
                sincosf(alpha, &si, &co);
                const float ch = 0.5f * (1.f + co), sh = 0.5f * (1.f - co);
                const float hs = 0.5f * si, hc = 0.5f * co;
                float at_b1 = 0.f, at_gen = 0.f;
                if constexpr (S::B1) at_b1 = op.flip;
                if constexpr (GEN) at_gen = dfl * b1 + op.flip * g_b1;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const float p = P[r], m = M[r], z = Z[r];
                    const float w = p - m;
                    float U = 0.f, V = 0.f;
                    if constexpr (S::B1 || GEN) {
                        U = fmaf(-hs, w, -co * z);
                        V = fmaf(hc, w, -si * z);
                    }
#pragma unroll
                    for (int j = 0; j < NT; ++j) {
                        const float dp = dP[j][r], dm = dM[j][r], dz = dZ[j][r];
                        float np = fmaf(ch, dp, fmaf(sh, dm, -si * dz));
                        float nm = fmaf(sh, dp, fmaf(ch, dm, si * dz));
                        float nz = fmaf(hs, dp - dm, co * dz);
                        float at = 0.f;
                        if (S::B1 && j == S::I_B1) at = at_b1;
                        if (GEN && j == S::I_GEN) at = at_gen;
                        if ((S::B1 && j == S::I_B1) || (GEN && j == S::I_GEN)) {
                            np = fmaf(at, U, np);
                            nm = fmaf(-at, U, nm);
                            nz = fmaf(at, V, nz);
                        }
                        dP[j][r] = np;
                        dM[j][r] = nm;
                        dZ[j][r] = nz;
                    }
                    P[r] = fmaf(ch, p, fmaf(sh, m, -si * z));
                    M[r] = fmaf(sh, p, fmaf(ch, m, si * z));
                    Z[r] = fmaf(hs, w, co * z);
                }
            } else if (rf == RF_INVERT) {
                const float f = -eff;
#pragma unroll
                for (int r = 0; r < R; ++r) {
#pragma unroll
                    for (int j = 0; j < NT; ++j) {
                        float nz = dZ[j][r] * f;
                        if (S::INV && j == S::I_INV) nz = nz - Z[r];
                        if (GEN && j == S::I_GEN) nz = fmaf(Z[r], -g_inv, nz);
                        dZ[j][r] = nz;
                    }
                    Z[r] *= f;
                }
            }
        after_rf:
            for (int s = 0; s < op_shift2(code); ++s) {
                shift_pair<R, L>(P, M, q, kill, kill_r);
#pragma unroll
                for (int j = 0; j < NT; ++j) shift_pair<R, L>(dP[j], dM[j], q, kill, kill_r);
            }
            if (code & OP_SPOIL1) {
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    P[r] = M[r] = 0.f;
#pragma unroll
                    for (int j = 0; j < NT; ++j) dP[j][r] = dM[j][r] = 0.f;
                }
            }
            if constexpr (GN) {
                if ((code & OP_RECORD) && q == 0 && active) {
                    // API signal s = -v (v = m0 F+[0]); r = s - y. Columns of
                    // dv: T1, T2 (tangents), M0 (F+[0]); J^T J and J^T r
                    // carry the sign of s twice or not at all.
                    const float2 y = yrow[op.record];
                    const float v = m0 * P[0];
                    const float res = v + y.x;  // -(r.real)
                    const float j1 = m0 * dP[S::I_T1][0];
                    const float j2 = m0 * dP[S::I_T2][0];
                    const float j3 = P[0];
                    cs[0] = fmaf(res, res, fmaf(y.y, y.y, cs[0]));
                    cs[1] = fmaf(j1, j1, cs[1]);
                    cs[2] = fmaf(j1, j2, cs[2]);
                    cs[3] = fmaf(j1, j3, cs[3]);
                    cs[4] = fmaf(j2, j2, cs[4]);
                    cs[5] = fmaf(j2, j3, cs[5]);
                    cs[6] = fmaf(j3, j3, cs[6]);
                    cs[7] = fmaf(j1, res, cs[7]);
                    cs[8] = fmaf(j2, res, cs[8]);
                    cs[9] = fmaf(j3, res, cs[9]);
                    if (++in_chunk == 32) {
#pragma unroll
                        for (int k = 0; k < 10; ++k) {
                            cd[k] += double(cs[k]);
                            cs[k] = 0.f;
                        }
                        in_chunk = 0;
                    }
                }
            }
            if ((code & OP_RECORD) && q == 0 && active && !GN) {
                const int64_t idx = row * a.outputs + op.record;
                if (a.sig_b != nullptr || a.layout != TSG_LAYOUT_PLANES) {
                    if (a.sig_a != nullptr || a.sig_b != nullptr)
                        put_sample(a.layout, a.sig_a, a.sig_b, idx, m0 * P[0]);
                }
                const int64_t jrow = row * a.jac_cols;
                if constexpr (S::T1)
                    if (a.col_t1 >= 0)
                        put_sample(a.layout, a.jac_a, a.jac_b, (jrow + a.col_t1) * a.outputs + op.record,
                                   m0 * dP[S::I_T1][0]);
                if constexpr (S::T2)
                    if (a.col_t2 >= 0)
                        put_sample(a.layout, a.jac_a, a.jac_b, (jrow + a.col_t2) * a.outputs + op.record,
                                   m0 * dP[S::I_T2][0]);
                if constexpr (S::B1)
                    if (a.col_b1 >= 0)
                        put_sample(a.layout, a.jac_a, a.jac_b, (jrow + a.col_b1) * a.outputs + op.record,
                                   m0 * dP[S::I_B1][0]);
                if constexpr (S::INV)
                    if (a.col_inv >= 0)
                        put_sample(a.layout, a.jac_a, a.jac_b,
                                   (jrow + a.col_inv) * a.outputs + op.record, m0 * dP[S::I_INV][0]);
                if constexpr (GEN)
                    if (a.col_gen >= 0)
                        put_sample(a.layout, a.jac_a, a.jac_b,
                                   (jrow + a.col_gen) * a.outputs + op.record,
                                   fmaf(g_m0, P[0], m0 * dP[S::I_GEN][0]));
                if (a.col_m0 >= 0)
                    put_sample(a.layout, a.jac_a, a.jac_b, (jrow + a.col_m0) * a.outputs + op.record, P[0]);
            }
            for (int s = 0; s < op_shift3(code); ++s) {
                shift_pair<R, L>(P, M, q, kill, kill_r);
#pragma unroll
                for (int j = 0; j < NT; ++j) shift_pair<R, L>(dP[j], dM[j], q, kill, kill_r);
            }
            if (code & OP_SPOIL2) {
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    P[r] = M[r] = 0.f;
#pragma unroll
                    for (int j = 0; j < NT; ++j) dP[j][r] = dM[j][r] = 0.f;
                }
            }
        }
    }
    if constexpr (GN) {
        if (q == 0 && active) {
            double* dst = a.gn_out + row * 10;
#pragma unroll
            for (int k = 0; k < 10; ++k) dst[k] = cd[k] + double(cs[k]);
        }
    }
}

template <int R, int L, int TM, bool GEN, bool GN = false>
void launch_sweep(const SweepArgs& a, dim3 grid, dim3 block, size_t smem, cudaStream_t stream) {
    epg_sweep_kernel<R, L, TM, GEN, GN><<<grid, block, smem, stream>>>(a);
}

}  // namespace tsg

#define TSG_SWEEP_ENTRY(MODE, R, L, TM, GEN) \
    {MODE, R, L, &::tsg::launch_sweep<R, L, TM, GEN, false>}
#define TSG_GN_ENTRY(R, L) {::tsg::MODE_GN, R, L, &::tsg::launch_sweep<R, L, 3, false, true>}
