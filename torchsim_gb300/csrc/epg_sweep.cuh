// The per-voxel EPG sweep: one pass over a compiled pulse program that
// carries the F+/F-/Z state of every voxel in registers for the whole
// sequence, optionally with forward-mode tangents beside it.
//
// Thread mapping: a voxel's configuration orders are spread over L warp lanes
// (lanes_per_voxel), R = 2*RP consecutive orders per lane (orders_per_lane),
// so a warp holds floor(32/L) voxels. Each lane keeps its orders as RP pairs
// in float2 registers and does the relaxation and the RF rotation of two
// orders with one paired FP32 instruction (__ffma2_rn / __fmul2_rn): the
// recursion is issue-bound, and pairing halves the arithmetic instructions.
// Pairs are strided: the lane's local order l (0 <= l < R) sits in pair
// l % RP, in .x for l < RP and in .y above. The gradient shift moves F+ one
// order up and F- one order down; with strided pairs that moves whole pairs
// (pair k takes pair k - 1, or k + 1) except one pair at the lane's edge, so
// where a shift directly follows the rotation the moves fold into the
// rotation's own results. Across lanes the shift is a warp shuffle. The
// program (ops) is staged in shared memory and read as a broadcast, since
// every voxel of a block follows the same train.
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

__device__ __forceinline__ float2 dup(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }

// The lane's local order l of a strided pair array (l a compile-time index
// after unrolling).
template <int RP>
__device__ __forceinline__ float order_at(const float2 (&a)[RP], int l) {
    return l < RP ? a[l % RP].x : a[l % RP].y;
}

// One gradient shift of a (F+, F-) pair of strided order-pair arrays spread
// over L lanes: F- moves one order down (the top order takes what the next
// lane held at its order 0, or nothing at the voxel's top), then F+ one order
// up with F+[0] = -F-[0] at the voxel's first lane. `kill_k` (or -1) and
// `kill_hi` name the slot of order `states`, cleared after the shift: the
// only way into the orders past the kept ones is F+ moving up.
template <int RP, int L>
__device__ __forceinline__ void shift_pair(float2 (&p)[RP], float2 (&m)[RP], int q, int kill_k,
                                           bool kill_hi) {
    float in_p = 0.f, in_m = 0.f;
    if constexpr (L > 1) {
        in_p = __shfl_up_sync(0xffffffffu, p[RP - 1].y, 1);
        in_m = __shfl_down_sync(0xffffffffu, m[0].x, 1);
    }
    float top = 0.f;
    if constexpr (L > 1) top = (q == L - 1) ? 0.f : in_m;
    const float m_edge = m[0].y;
#pragma unroll
    for (int k = 0; k + 1 < RP; ++k) m[k] = m[k + 1];
    m[RP - 1] = make_float2(m_edge, top);
    float bottom = -m[0].x;
    if constexpr (L > 1) bottom = (q == 0) ? -m[0].x : in_p;
    const float p_edge = p[RP - 1].x;
#pragma unroll
    for (int k = RP - 1; k > 0; --k) p[k] = p[k - 1];
    p[0] = make_float2(bottom, p_edge);
#pragma unroll
    for (int k = 0; k < RP; ++k) {
        if (k == kill_k) {
            if (kill_hi) p[k].y = 0.f;
            else p[k].x = 0.f;
        }
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

// Whether the relaxation-folded tangent step fits the register budget of a
// launch with at least `minb` blocks of 128 threads per SM: it holds about
// 34 + RP (1 + 12 NT) registers (108 at RP 2, NT 3; 71 at RP 1, NT 3, by
// ptxas), against 65536 / (128 minb) a thread. (At equal occupancy the
// folded and unfolded steps measured alike on the dictionary sweep; beyond
// the budget the folded one spills.)
constexpr bool fold_fits(int rp, int nt, int minb) {
    return minb <= 1 || 65536 / (128 * minb) >= 34 + rp * (1 + 12 * nt);
}

// The real rotation about x by alpha, scaled by the relaxation (E1 on Z,
// E2 on F+ and F-; 1 and 1 for the rotation alone), in sum/difference form:
// with s = p + m and d = p - m, A = E2 s / 2 and B = E2 cos(a) d / 2 -
// E1 sin(a) z, the rotated state is p' = A + B, m' = A - B, z' = E2 sin(a)
// d / 2 + E1 cos(a) z, and d/dalpha of (p', m', z') is (-z', z', B).
struct Rotation {
    float2 half_e2;  // E2 / 2
    float2 hco;      // E2 cos / 2
    float2 nsi;      // -E1 sin
    float2 hsi;      // E2 sin / 2
    float2 co;       // E1 cos
};

__device__ __forceinline__ Rotation rotation(float si, float co, float e1, float e2) {
    const float h = 0.5f * e2;
    return {dup(h), dup(h * co), dup(-e1 * si), dup(h * si), dup(e1 * co)};
}

// Rotates one pair of orders in place; leaves d and B for the derivative.
__device__ __forceinline__ void rotate_pair(const Rotation& c, float2& p, float2& m, float2& z,
                                            float2& d, float2& B) {
    const float2 s = add2(p, m);
    d = fma2(dup(-1.f), m, p);
    const float2 A = mul2(c.half_e2, s);
    B = fma2(c.hco, d, mul2(c.nsi, z));
    p = add2(A, B);
    m = fma2(dup(-1.f), B, A);
    z = fma2(c.hsi, d, mul2(c.co, z));
}

// Rotates a tangent pair whose angle moves by `at` per unit: adds
// at (-z', z', B) of the signal (z' its rotated Z, B from its rotation).
__device__ __forceinline__ void rotate_pair_moved(const Rotation& c, float2& p, float2& m,
                                                  float2& z, float at, float2 zs, float2 Bs) {
    const float2 s = add2(p, m);
    const float2 d = fma2(dup(-1.f), m, p);
    const float2 A = mul2(c.half_e2, s);
    const float2 B = fma2(dup(-at), zs, fma2(c.hco, d, mul2(c.nsi, z)));
    p = add2(A, B);
    m = fma2(dup(-1.f), B, A);
    z = fma2(dup(at), Bs, fma2(c.hsi, d, mul2(c.co, z)));
}

// The refocusing op of a CPMG echo: relax, shift, rotate, shift, nothing
// else; straight-line too.
constexpr uint32_t kEchoMask = kFastMask | OP_RECORD;
constexpr uint32_t kEchoBits = OP_RELAX | (1u << OP_SHIFT1_SHIFT) |
                               (uint32_t(RF_ROTATE) << OP_RF_SHIFT) | (1u << OP_SHIFT2_SHIFT);

template <int RP, int L, int TM, bool GEN, bool GN = false, int MINB = 1>
__global__ void __launch_bounds__(MINB > 1 ? 128 : 256, MINB) epg_sweep_kernel(const SweepArgs a) {
    using S = SystemLayout<TM, GEN>;
    constexpr int NT = S::N;
    constexpr int R = 2 * RP;
    constexpr int VPW = 32 / L;
    // Relaxation folded into the rotation: always for the signal alone;
    // with tangents where the register budget holds it.
    constexpr bool FOLD = NT == 0 || (!GEN && fold_fits(RP, NT, MINB));
    __shared__ Op s_ops[kOpChunk];
    __shared__ float2 s_dir[GEN ? kOpChunk : 1];

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int q = lane % L;
    const int slot = lane / L;
    const int64_t atom = (int64_t(blockIdx.x) * (blockDim.x >> 5) + warp) * VPW + slot;
    const int64_t train = blockIdx.y;
    // Lanes past the last whole voxel of the warp (32 % L of them) idle.
    const bool active = slot < VPW && atom < a.atoms;
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

    // The slot of order `states` in this lane, if the lane holds it and
    // the lanes hold more orders than are kept.
    const int kill_r = a.states - q * R;
    const bool kill = L * R > a.states && kill_r >= 0 && kill_r < R;
    const int kill_k = kill ? kill_r % RP : -1;
    const bool kill_hi = kill_r >= RP;
    const float2 neg1 = dup(-1.f);

    float2 P[RP], M[RP], Z[RP];
    float2 dP[S::NA][RP], dM[S::NA][RP], dZ[S::NA][RP];
#pragma unroll
    for (int k = 0; k < RP; ++k) {
        P[k] = M[k] = Z[k] = dup(0.f);
#pragma unroll
        for (int j = 0; j < S::NA; ++j) dP[j][k] = dM[j][k] = dZ[j][k] = dup(0.f);
    }
    if (q == 0) Z[0].x = 1.f;

    float last_dt = __int_as_float(0x7fffffff);  // NaN: first relax computes
    float e1 = 1.f, e2 = 1.f, k1 = 0.f, k2 = 0.f;

    // Gauss-Newton sums: float over chunks of 32 samples, then into doubles
    // kept in shared memory (they change once per chunk, so they need not
    // hold twenty registers for the whole sweep), one column per thread.
    static_assert(!GN || (S::T1 && S::T2), "GN sweeps carry the T1 and T2 tangents");
    __shared__ double s_cd[GN ? 10 * 256 : 1];
    double* cd = s_cd + threadIdx.x;  // cd[k * blockDim.x]: sum k of this thread
    float cs[10];
    int in_chunk = 0;
#pragma unroll
    for (int k = 0; k < 10; ++k) cs[k] = 0.f;
    if constexpr (GN) {
#pragma unroll
        for (int k = 0; k < 10; ++k) cd[k * blockDim.x] = 0.0;
    }
    const float2* yrow = nullptr;
    if constexpr (GN) {
        const int64_t mrow = a.measured_rows ? a.measured_rows[ac] : (train * a.atoms + ac);
        yrow = a.measured + mrow * a.outputs;
    }

    const Op* ops = a.ops + train * a.n_ops;
    const float2* dirs = GEN ? a.op_dir + train * a.n_ops : nullptr;
    const int64_t row = train * a.atoms + atom;
    // Strided trajectory: this lane's granules of op 0; each even op moves
    // the pointer on by one stored op's worth (3 planes x granules x 32).
    constexpr int kGran = (RP + 1) / 2;
    float4* traj_cur = nullptr;
    if constexpr (L == 1 && NT == 0 && !GEN && !GN) {
        if (a.traj != nullptr && a.traj_strided)
            traj_cur = reinterpret_cast<float4*>(a.traj) +
                       (train * ((a.atoms + 31) >> 5) + (ac >> 5)) *
                           int64_t((a.n_ops + 1) >> 1) * (3 * kGran * 32) +
                       (ac & 31);
    }
    // Output row bases, once: a record then only adds its sample index.
    // Column offsets (col * outputs) are the same for every thread.
    const int64_t sig_base = row * a.outputs;
    const int64_t jbase = row * a.jac_cols * a.outputs;
    // Distributed records: with at least as many lanes per voxel as output
    // columns (the signal, each tangent's column in system order, M0), lane
    // q of the voxel writes column q from its own row pointer, so one store
    // instruction serves every column; the values come from lane 0 by
    // shuffles. Otherwise lane 0 writes every column.
    constexpr bool DIST = !GN && L >= NT + 2;
    float* row_a = nullptr;  // this lane's column row: plane a, or the complex row
    float* row_b = nullptr;  // plane b of the planes layout
    if constexpr (DIST) {
        float* base_a = nullptr;
        float* base_b = nullptr;
        int64_t off = 0;
        int col = -1;
        if (q >= 1 && q <= NT) {
            const int j = q - 1;
            if constexpr (S::T1) if (j == S::I_T1) col = a.col_t1;
            if constexpr (S::T2) if (j == S::I_T2) col = a.col_t2;
            if constexpr (S::B1) if (j == S::I_B1) col = a.col_b1;
            if constexpr (S::INV) if (j == S::I_INV) col = a.col_inv;
            if constexpr (GEN) if (j == S::I_GEN) col = a.col_gen;
        } else if (q == NT + 1) {
            col = a.col_m0;
        }
        if (q == 0) {
            if ((a.sig_b != nullptr || a.layout != TSG_LAYOUT_PLANES) &&
                (a.sig_a != nullptr || a.sig_b != nullptr)) {
                base_a = a.sig_a;
                base_b = a.sig_b;
                off = sig_base;
            }
        } else if (col >= 0) {
            base_a = a.jac_a;
            base_b = a.jac_b;
            off = jbase + int64_t(col) * a.outputs;
        }
        if (active && q <= NT + 1) {
            if (a.layout == TSG_LAYOUT_PLANES) {
                row_a = base_a ? base_a + off : nullptr;
                row_b = base_b ? base_b + off : nullptr;
            } else if (base_a) {
                row_a = reinterpret_cast<float*>(reinterpret_cast<float2*>(base_a) + off);
            }
        }
    }
    // Each pulse's sin/cos is the same for all L lanes of a voxel: lane q
    // computes it for one of the next L ops and the voxel's lanes exchange
    // them with a shuffle, so each lane evaluates one sincosf per L pulses.
    float my_si = 0.f, my_co = 1.f;
    const int first_lane = lane - q;
    float ddt = 0.f, dfl = 0.f;

    auto pulse = [&](const Op& op, int g, float& si, float& co) {
        if constexpr (L > 1) {
            si = __shfl_sync(0xffffffffu, my_si, first_lane + g);
            co = __shfl_sync(0xffffffffu, my_co, first_lane + g);
        } else {
            sincosf(op.flip * b1, &si, &co);
        }
    };

    // Relaxation and rotation in one 3x3 per order for the signal alone,
    // with the recovery of order 0 added after.
    auto fold_signal = [&](float si, float co) {
        const Rotation c = rotation(si, co, e1, e2);
#pragma unroll
        for (int k = 0; k < RP; ++k) {
            float2 d, B;
            rotate_pair(c, P[k], M[k], Z[k], d, B);
        }
        if (q == 0) {
            const float rec = 1.f - e1;
            P[0].x = fmaf(-si, rec, P[0].x);
            M[0].x = fmaf(si, rec, M[0].x);
            Z[0].x = fmaf(co, rec, Z[0].x);
        }
    };

    // Relaxation folded into the rotation for the signal and every tangent:
    // with X0 the state before the interval, X = E X0 + r and dX = E dX0 +
    // dE X0 (+ dr), so the pulse acts through R E on X0, on dX0 + E^-1 dE X0
    // (T2 adds dt w2 (p, m), T1 dt w1 z), and the recovery r and its T1
    // derivative enter order 0 after the fact.
    auto fold_tangents = [&](const Op& op, float si, float co) {
        const Rotation c = rotation(si, co, e1, e2);
        float at_b1 = 0.f;
        if constexpr (S::B1) at_b1 = op.flip;
        const float2 g1 = dup(op.dt * w1), g2 = dup(op.dt * w2);
#pragma unroll
        for (int k = 0; k < RP; ++k) {
            const float2 p = P[k], m = M[k], z = Z[k];
            float2 d, B;
            rotate_pair(c, P[k], M[k], Z[k], d, B);
#pragma unroll
            for (int j = 0; j < NT; ++j) {
                if (S::T1 && j == S::I_T1) dZ[j][k] = fma2(g1, z, dZ[j][k]);
                if (S::T2 && j == S::I_T2) {
                    dP[j][k] = fma2(g2, p, dP[j][k]);
                    dM[j][k] = fma2(g2, m, dM[j][k]);
                }
                if (S::B1 && j == S::I_B1) {
                    // d alpha / d B1 = flip: (-Zn, Zn, V) of the relaxed
                    // state, V = B of the signal's rotation.
                    rotate_pair_moved(c, dP[j][k], dM[j][k], dZ[j][k], at_b1, Z[k], B);
                } else {
                    float2 dd, dB;
                    rotate_pair(c, dP[j][k], dM[j][k], dZ[j][k], dd, dB);
                }
            }
        }
        if (q == 0) {
            // The recovery (1 - e1) of order 0 and its T1 derivative (-k1)
            // through the pulse: R (0, 0, c) = (-si c, si c, co c); for B1
            // the recovery also moves Zn (used above without it) and V by
            // (co, -si) c.
            const float rec = 1.f - e1;
            if constexpr (S::B1) {
                dP[S::I_B1][0].x = fmaf(-at_b1 * co, rec, dP[S::I_B1][0].x);
                dM[S::I_B1][0].x = fmaf(at_b1 * co, rec, dM[S::I_B1][0].x);
                dZ[S::I_B1][0].x = fmaf(-at_b1 * si, rec, dZ[S::I_B1][0].x);
            }
            if constexpr (S::T1) {
                dP[S::I_T1][0].x = fmaf(si, k1, dP[S::I_T1][0].x);
                dM[S::I_T1][0].x = fmaf(-si, k1, dM[S::I_T1][0].x);
                dZ[S::I_T1][0].x = fmaf(-co, k1, dZ[S::I_T1][0].x);
            }
            P[0].x = fmaf(-si, rec, P[0].x);
            M[0].x = fmaf(si, rec, M[0].x);
            Z[0].x = fmaf(co, rec, Z[0].x);
        }
    };

    auto relax_all = [&](const Op& op) {
        const float2 E1 = dup(e1), E2 = dup(e2);
        float e1g = 0.f, e2g = 0.f;
        if constexpr (GEN) {
            e1g = e1 * (op.dt * g_t1 * w1 - r1 * ddt);
            e2g = e2 * (op.dt * g_t2 * w2 - r2 * ddt);
        }
#pragma unroll
        for (int k = 0; k < RP; ++k) {
            if constexpr (S::T1) {
                dP[S::I_T1][k] = mul2(dP[S::I_T1][k], E2);
                dM[S::I_T1][k] = mul2(dM[S::I_T1][k], E2);
                dZ[S::I_T1][k] = fma2(dZ[S::I_T1][k], E1, mul2(Z[k], dup(k1)));
            }
            if constexpr (S::T2) {
                dP[S::I_T2][k] = fma2(dP[S::I_T2][k], E2, mul2(P[k], dup(k2)));
                dM[S::I_T2][k] = fma2(dM[S::I_T2][k], E2, mul2(M[k], dup(k2)));
                dZ[S::I_T2][k] = mul2(dZ[S::I_T2][k], E1);
            }
            if constexpr (S::B1) {
                dP[S::I_B1][k] = mul2(dP[S::I_B1][k], E2);
                dM[S::I_B1][k] = mul2(dM[S::I_B1][k], E2);
                dZ[S::I_B1][k] = mul2(dZ[S::I_B1][k], E1);
            }
            if constexpr (S::INV) {
                dP[S::I_INV][k] = mul2(dP[S::I_INV][k], E2);
                dM[S::I_INV][k] = mul2(dM[S::I_INV][k], E2);
                dZ[S::I_INV][k] = mul2(dZ[S::I_INV][k], E1);
            }
            if constexpr (GEN) {
                dP[S::I_GEN][k] = fma2(dP[S::I_GEN][k], E2, mul2(P[k], dup(e2g)));
                dM[S::I_GEN][k] = fma2(dM[S::I_GEN][k], E2, mul2(M[k], dup(e2g)));
                dZ[S::I_GEN][k] = fma2(dZ[S::I_GEN][k], E1, mul2(Z[k], dup(e1g)));
            }
            P[k] = mul2(P[k], E2);
            M[k] = mul2(M[k], E2);
            Z[k] = mul2(Z[k], E1);
        }
        if (q == 0) {
            Z[0].x += 1.f - e1;
            if constexpr (S::T1) dZ[S::I_T1][0].x -= k1;
            if constexpr (GEN) dZ[S::I_GEN][0].x -= e1g;
        }
    };

    auto rotate_all = [&](const Op& op, float si, float co) {
        const Rotation c = rotation(si, co, 1.f, 1.f);
        float at_b1 = 0.f, at_gen = 0.f;
        if constexpr (S::B1) at_b1 = op.flip;
        if constexpr (GEN) at_gen = dfl * b1 + op.flip * g_b1;
#pragma unroll
        for (int k = 0; k < RP; ++k) {
            // d/dalpha of the rotation: dP = -Zn, dM = Zn, dZ = V, V = B.
            float2 d, B;
            rotate_pair(c, P[k], M[k], Z[k], d, B);
#pragma unroll
            for (int j = 0; j < NT; ++j) {
                if ((S::B1 && j == S::I_B1) || (GEN && j == S::I_GEN)) {
                    const float at = (S::B1 && j == S::I_B1) ? at_b1 : at_gen;
                    rotate_pair_moved(c, dP[j][k], dM[j][k], dZ[j][k], at, Z[k], B);
                } else {
                    float2 dd, dB;
                    rotate_pair(c, dP[j][k], dM[j][k], dZ[j][k], dd, dB);
                }
            }
        }
    };

    auto shift_all = [&]() {
        shift_pair<RP, L>(P, M, q, kill_k, kill_hi);
#pragma unroll
        for (int j = 0; j < NT; ++j) shift_pair<RP, L>(dP[j], dM[j], q, kill_k, kill_hi);
    };

    auto spoil_all = [&]() {
#pragma unroll
        for (int k = 0; k < RP; ++k) {
            P[k] = M[k] = dup(0.f);
#pragma unroll
            for (int j = 0; j < NT; ++j) dP[j][k] = dM[j][k] = dup(0.f);
        }
    };

    // The record of an op: the API samples m0 F+[0] of the signal and of
    // each tangent column, or (GN sweeps) the voxel's normal-equation sums.
    auto record = [&](const Op& op) {
        if constexpr (GN) {
            if (q == 0 && active) {
                // API signal s = -v (v = m0 F+[0]); r = s - y. Columns of
                // dv: T1, T2 (tangents), M0 (F+[0]); J^T J and J^T r carry
                // the sign of s twice or not at all.
                const float2 y = yrow[op.record];
                const float p0 = P[0].x;
                const float v = m0 * p0;
                const float res = v + y.x;  // -(r.real)
                const float j1 = m0 * dP[S::I_T1][0].x;
                const float j2 = m0 * dP[S::I_T2][0].x;
                const float j3 = p0;
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
                        cd[k * blockDim.x] += double(cs[k]);
                        cs[k] = 0.f;
                    }
                    in_chunk = 0;
                }
            }
        } else if constexpr (DIST) {
            const int rec = op.record;
            const float p0 = __shfl_sync(0xffffffffu, P[0].x, first_lane);
            if constexpr (NT == 0 && !GEN)
                if (q == 0 && active && a.traj_rec != nullptr)
                    a.traj_rec[(train * a.outputs + rec) * a.atoms + atom] = p0;
            float v = m0 * p0;  // lane 0: the signal
#pragma unroll
            for (int j = 0; j < NT; ++j) {
                const float d = __shfl_sync(0xffffffffu, dP[j][0].x, first_lane);
                if (q == j + 1) {
                    v = m0 * d;
                    if constexpr (GEN)
                        if (j == S::I_GEN) v = fmaf(g_m0, p0, v);
                }
            }
            if (q == NT + 1) v = p0;  // the M0 column
            if (a.layout == TSG_LAYOUT_PLANES) {
                if (row_b != nullptr) {
                    if (row_a != nullptr) __stcs(row_a + rec, 0.f);
                    __stcs(row_b + rec, v);
                }
            } else if (row_a != nullptr) {
                float2* dst = reinterpret_cast<float2*>(row_a) + rec;
                __stcs(dst, a.layout == TSG_LAYOUT_COMPLEX ? make_float2(0.f, v) : make_float2(-v, 0.f));
            }
        } else if (q == 0 && active) {
            const int rec = op.record;
            const float p0 = P[0].x;
            if constexpr (NT == 0 && !GEN)
                if (a.traj_rec != nullptr) a.traj_rec[(train * a.outputs + rec) * a.atoms + atom] = p0;
            if (a.sig_b != nullptr || a.layout != TSG_LAYOUT_PLANES) {
                if (a.sig_a != nullptr || a.sig_b != nullptr)
                    put_sample(a.layout, a.sig_a, a.sig_b, sig_base + rec, m0 * p0);
            }
            if constexpr (S::T1)
                if (a.col_t1 >= 0)
                    put_sample(a.layout, a.jac_a, a.jac_b, jbase + (a.col_t1 * a.outputs + rec),
                               m0 * dP[S::I_T1][0].x);
            if constexpr (S::T2)
                if (a.col_t2 >= 0)
                    put_sample(a.layout, a.jac_a, a.jac_b, jbase + (a.col_t2 * a.outputs + rec),
                               m0 * dP[S::I_T2][0].x);
            if constexpr (S::B1)
                if (a.col_b1 >= 0)
                    put_sample(a.layout, a.jac_a, a.jac_b, jbase + (a.col_b1 * a.outputs + rec),
                               m0 * dP[S::I_B1][0].x);
            if constexpr (S::INV)
                if (a.col_inv >= 0)
                    put_sample(a.layout, a.jac_a, a.jac_b, jbase + (a.col_inv * a.outputs + rec),
                               m0 * dP[S::I_INV][0].x);
            if constexpr (GEN)
                if (a.col_gen >= 0)
                    put_sample(a.layout, a.jac_a, a.jac_b, jbase + (a.col_gen * a.outputs + rec),
                               fmaf(g_m0, p0, m0 * dP[S::I_GEN][0].x));
            if (a.col_m0 >= 0)
                put_sample(a.layout, a.jac_a, a.jac_b, jbase + (a.col_m0 * a.outputs + rec), p0);
        }
    };

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
            const int g = i % L;
            if constexpr (L > 1) {
                if (g == 0) {
                    const int j = i + q;
                    float sj = 0.f, cj = 1.f;
                    if (j < count) {
                        const Op oj = s_ops[j];
                        if (op_rf(oj.code) == RF_ROTATE) sincosf(oj.flip * b1, &sj, &cj);
                    }
                    my_si = sj;
                    my_co = cj;
                }
            }
            if constexpr (NT == 0 && !GEN && !GN) {
                if (a.ckpt != nullptr && ((base + i) % a.ckpt_every) == 0 && active) {
                    // State entering this op, for the adjoint's segments;
                    // atoms innermost, so a warp's stores of one order are
                    // contiguous.
                    const int k = (base + i) / a.ckpt_every;
                    const int Sn = a.states;
                    const int64_t n = a.atoms;
                    float* dst = a.ckpt + (train * a.ckpt_count + k) * (3 * int64_t(Sn)) * n + atom;
#pragma unroll
                    for (int l = 0; l < R; ++l) {
                        const int o = q * R + l;
                        if (o < Sn) {
                            dst[o * n] = order_at(P, l);
                            dst[(Sn + o) * n] = order_at(M, l);
                            dst[(2 * Sn + o) * n] = order_at(Z, l);
                        }
                    }
                }
                if constexpr (L == 1) {
                    if (traj_cur != nullptr && ((base + i) & 1) == 0) {
                        // The registers as they are: granule g holds pairs
                        // 2g and 2g + 1 (the last one zero for odd RP).
                        if (active) {
#pragma unroll
                            for (int g = 0; g < kGran; ++g) {
                                const float2 p1 = 2 * g + 1 < RP ? P[2 * g + 1] : dup(0.f);
                                const float2 m1 = 2 * g + 1 < RP ? M[2 * g + 1] : dup(0.f);
                                const float2 z1 = 2 * g + 1 < RP ? Z[2 * g + 1] : dup(0.f);
                                traj_cur[g * 32] = make_float4(P[2 * g].x, P[2 * g].y, p1.x, p1.y);
                                traj_cur[(kGran + g) * 32] =
                                    make_float4(M[2 * g].x, M[2 * g].y, m1.x, m1.y);
                                traj_cur[(2 * kGran + g) * 32] =
                                    make_float4(Z[2 * g].x, Z[2 * g].y, z1.x, z1.y);
                            }
                        }
                        traj_cur += 3 * kGran * 32;
                    }
                }
                if (a.traj != nullptr && !a.traj_strided && active) {
                    // Every op's entry state as consecutive order pairs
                    // (2 pj, 2 pj + 1), in tiles of 32 atoms:
                    // [train][tile][op][plane][pair][32].
                    const int np = (a.states + 1) >> 1;
                    const int64_t tiles = (a.atoms + 31) >> 5;
                    float2* dst = a.traj +
                                  ((train * tiles + (atom >> 5)) * a.n_ops + base + i) *
                                      (3 * int64_t(np) * 32) +
                                  (atom & 31);
#pragma unroll
                    for (int kk = 0; kk < RP; ++kk) {
                        const int pj = q * RP + kk;
                        if (pj < np) {
                            dst[pj * 32] = make_float2(order_at(P, 2 * kk), order_at(P, 2 * kk + 1));
                            dst[(np + pj) * 32] =
                                make_float2(order_at(M, 2 * kk), order_at(M, 2 * kk + 1));
                            dst[(2 * np + pj) * 32] =
                                make_float2(order_at(Z, 2 * kk), order_at(Z, 2 * kk + 1));
                        }
                    }
                }
            }
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
            if constexpr (!GEN) {
                if ((code & kFastMask) == kFastBits) {
                    float si, co;
                    pulse(op, g, si, co);
                    if constexpr (NT == 0) fold_signal(si, co);
                    else if constexpr (FOLD) fold_tangents(op, si, co);
                    else {
                        relax_all(op);
                        rotate_all(op, si, co);
                    }
                    if (code & OP_RECORD) record(op);
                    shift_all();
                    continue;
                }
                if ((code & kEchoMask) == kEchoBits) {
                    relax_all(op);
                    shift_all();
                    float si, co;
                    pulse(op, g, si, co);
                    rotate_all(op, si, co);
                    shift_all();
                    continue;
                }
            }
            const int n1 = op_shift1(code);
            if (FOLD && relax && rf == RF_ROTATE && n1 == 0) {
                float si, co;
                pulse(op, g, si, co);
                if constexpr (NT == 0) fold_signal(si, co);
                else if constexpr (FOLD) fold_tangents(op, si, co);
            } else {
                if (relax) relax_all(op);
                for (int s = 0; s < n1; ++s) shift_all();
                if (rf == RF_ROTATE) {
                    float si, co;
                    pulse(op, g, si, co);
                    rotate_all(op, si, co);
                } else if (rf == RF_INVERT) {
                    const float2 f = dup(-eff);
#pragma unroll
                    for (int k = 0; k < RP; ++k) {
#pragma unroll
                        for (int j = 0; j < NT; ++j) {
                            float2 nz = mul2(dZ[j][k], f);
                            if (S::INV && j == S::I_INV) nz = fma2(neg1, Z[k], nz);
                            if (GEN && j == S::I_GEN) nz = fma2(Z[k], dup(-g_inv), nz);
                            dZ[j][k] = nz;
                        }
                        Z[k] = mul2(Z[k], f);
                    }
                }
            }
            for (int s = 0; s < op_shift2(code); ++s) shift_all();
            if (code & OP_SPOIL1) spoil_all();
            if (code & OP_RECORD) record(op);
            for (int s = 0; s < op_shift3(code); ++s) shift_all();
            if (code & OP_SPOIL2) spoil_all();
        }
    }
    if constexpr (GN) {
        if (q == 0 && active) {
            double* dst = a.gn_out + row * 10;
#pragma unroll
            for (int k = 0; k < 10; ++k) dst[k] = cd[k * blockDim.x] + double(cs[k]);
        }
    }
}

template <int RP, int L, int TM, bool GEN, bool GN = false, int MINB = 1>
void launch_sweep(const SweepArgs& a, dim3 grid, dim3 block, size_t smem, cudaStream_t stream) {
    epg_sweep_kernel<RP, L, TM, GEN, GN, MINB><<<grid, block, smem, stream>>>(a);
}

}  // namespace tsg

// Table entries take orders per lane R (even): the kernel keeps R/2 pairs.
#define TSG_SWEEP_ENTRY(MODE, R, L, TM, GEN) \
    {MODE, R, L, &::tsg::launch_sweep<(R) / 2, L, TM, GEN, false>, 0}
// A register-budget variant: at most 128 threads per block and at least
// MINB blocks resident per SM, i.e. 65536 / (128 * MINB) registers a thread.
#define TSG_SWEEP_ENTRY_MINB(MODE, R, L, TM, GEN, MINB) \
    {MODE, R, L, &::tsg::launch_sweep<(R) / 2, L, TM, GEN, false, MINB>, MINB}
#define TSG_GN_ENTRY(R, L) {::tsg::MODE_GN, R, L, &::tsg::launch_sweep<(R) / 2, L, 3, false, true>, 0}
#define TSG_GN_ENTRY_MINB(R, L, MINB) \
    {::tsg::MODE_GN, R, L, &::tsg::launch_sweep<(R) / 2, L, 3, false, true, MINB>, MINB}
