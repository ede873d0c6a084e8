// Helpers of the complex EPG sweeps (one pool, instant RF): the per-lane
// complex shift, the pulse's complex 3x3 and the sample store. Shared by the
// forward/tangent kernels (epg_complex.cu) and the adjoint
// (epg_complex_adjoint.cu).
#pragma once
#include "tsg_internal.h"

namespace tsg {

namespace complex_detail {

constexpr int kComplexOpChunk = 1024;

__device__ __forceinline__ float2 dup(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

struct ComplexArgs {
    const Op* ops;
    const float2* phase;  // [train][ops]: (pulse phase, receiver phase)
    int n_ops;
    int64_t atoms;
    int states;
    int outputs;
    const float* t1;
    const float* t2;
    const float* m0;
    const float* b1;
    const float* inv;
    const float* b1_phase;
    const float* b0;
    int layout;
    float* out_a;
    float* out_b;
    // Forward-mode columns (tangent kernels): (train*atoms+atom, col, output).
    float* jac_a;
    float* jac_b;
    int jac_cols;
    int col_t1, col_t2, col_b1, col_m0;
};

// The tangent systems a kernel carries: bit 1 T1, bit 2 T2, bit 4 B1.
template <int TM>
struct Tangents {
    static constexpr int T1 = (TM & 1) != 0, T2 = (TM & 2) != 0, B1 = (TM & 4) != 0;
    static constexpr int N = T1 + T2 + B1;
    static constexpr int NA = N > 0 ? N : 1;
    static constexpr int I_T1 = 0, I_T2 = T1, I_B1 = T1 + T2;
};

// One plane pair (re, im) shifted one order: `up` moves toward higher orders
// (F+), otherwise toward lower (F-). in_* come from the neighbouring lane.
template <int RP, int L>
__device__ __forceinline__ void shift_complex(float2 (&pr)[RP], float2 (&pi)[RP], float2 (&mr)[RP],
                                              float2 (&mi)[RP], int q, bool kill, int kill_r) {
    float in_pr = 0.f, in_pi = 0.f, in_mr = 0.f, in_mi = 0.f;
    if constexpr (L > 1) {
        in_pr = __shfl_up_sync(0xffffffffu, pr[RP - 1].y, 1);
        in_pi = __shfl_up_sync(0xffffffffu, pi[RP - 1].y, 1);
        in_mr = __shfl_down_sync(0xffffffffu, mr[0].x, 1);
        in_mi = __shfl_down_sync(0xffffffffu, mi[0].x, 1);
    }
    const bool top_lane = L == 1 || q == L - 1;
    const float top_r = top_lane ? 0.f : in_mr, top_i = top_lane ? 0.f : in_mi;
#pragma unroll
    for (int k = 0; k < RP; ++k) {
        mr[k].x = mr[k].y;
        mi[k].x = mi[k].y;
        mr[k].y = (k + 1 < RP) ? mr[k + 1].x : top_r;
        mi[k].y = (k + 1 < RP) ? mi[k + 1].x : top_i;
    }
    const bool first = L == 1 || q == 0;
    // F+[0] = conj(F-[0]) on the voxel's first lane.
    const float bottom_r = first ? mr[0].x : in_pr, bottom_i = first ? -mi[0].x : in_pi;
#pragma unroll
    for (int k = RP - 1; k >= 0; --k) {
        pr[k].y = pr[k].x;
        pi[k].y = pi[k].x;
        pr[k].x = (k > 0) ? pr[k - 1].y : bottom_r;
        pi[k].x = (k > 0) ? pi[k - 1].y : bottom_i;
    }
    if (kill) {
#pragma unroll
        for (int k = 0; k < RP; ++k) {
            if (2 * k == kill_r) pr[k].x = pi[k].x = 0.f;
            if (2 * k + 1 == kill_r) pr[k].y = pi[k].y = 0.f;
        }
    }
}

// The pulse's complex 3x3 in terms of (t00, t22) on the diagonal,
// A = t01 = conj(t10), B = t12 = (B_r, B_i) with t02 = (B_r, -B_i), and
// C = t21 = (C_r, C_i) with t20 = (C_r, -C_i). For the flip alpha and phase
// phi: t00 = (1 + cos a)/2, t22 = cos a, A = (1 - cos a)/2 e^{2i phi},
// B = i sin a e^{-i phi}, C = i (sin a / 2) e^{i phi}; its derivative in alpha
// has the same form with (-sin a / 2, -sin a, sin a / 2 e^{2i phi},
// i cos a e^{-i phi}, i (cos a / 2) e^{i phi}).
struct Pulse {
    float2 t00, t22, A_r, A_i, nA_i, B_r, B_i, nB_i, C_r, C_i, nC_i;
};

__device__ __forceinline__ Pulse pulse_of(float d00, float d22, float a, float bs, float cs,
                                          float c2, float s2, float cp, float sp) {
    // a: coefficient of e^{2i phi}; bs: of B (i bs e^{-i phi}); cs: of C.
    Pulse u;
    u.t00 = dup(d00);
    u.t22 = dup(d22);
    u.A_r = dup(a * c2);
    u.A_i = dup(a * s2);
    u.nA_i = dup(-a * s2);
    u.B_r = dup(bs * sp);
    u.B_i = dup(bs * cp);
    u.nB_i = dup(-bs * cp);
    u.C_r = dup(-cs * sp);
    u.C_i = dup(cs * cp);
    u.nC_i = dup(-cs * cp);
    return u;
}

// A pulse (or a derivative of one) from its entries: t00, t22, A = t01,
// B = t12 and C = t21, with t10 = conj(A), t02 = conj(B), t20 = conj(C).
__device__ __forceinline__ Pulse pulse_raw(float d00, float d22, float ar, float ai, float br,
                                           float bi, float cr, float ci) {
    Pulse u;
    u.t00 = dup(d00);
    u.t22 = dup(d22);
    u.A_r = dup(ar);
    u.A_i = dup(ai);
    u.nA_i = dup(-ai);
    u.B_r = dup(br);
    u.B_i = dup(bi);
    u.nB_i = dup(-bi);
    u.C_r = dup(cr);
    u.C_i = dup(ci);
    u.nC_i = dup(-ci);
    return u;
}

// (P, M, Z) -> pulse applied to (pr..zi); written to the six outputs.
__device__ __forceinline__ void apply(const Pulse& u, float2 pr, float2 pi, float2 mr, float2 mi,
                                      float2 zr, float2 zi, float2& opr, float2& opi, float2& omr,
                                      float2& omi, float2& ozr, float2& ozi) {
    opr = fma2(u.B_r, zr, fma2(u.B_i, zi, fma2(u.nA_i, mi, fma2(u.A_r, mr, mul2(u.t00, pr)))));
    opi = fma2(u.B_r, zi, fma2(u.nB_i, zr, fma2(u.A_i, mr, fma2(u.A_r, mi, mul2(u.t00, pi)))));
    omr = fma2(u.B_r, zr, fma2(u.nB_i, zi, fma2(u.A_i, pi, fma2(u.A_r, pr, mul2(u.t00, mr)))));
    omi = fma2(u.B_r, zi, fma2(u.B_i, zr, fma2(u.nA_i, pr, fma2(u.A_r, pi, mul2(u.t00, mi)))));
    ozr = fma2(u.C_r, mr, fma2(u.nC_i, mi, fma2(u.C_r, pr, fma2(u.C_i, pi, mul2(u.t22, zr)))));
    ozi = fma2(u.C_r, mi, fma2(u.C_i, mr, fma2(u.C_r, pi, fma2(u.nC_i, pr, mul2(u.t22, zi)))));
}

__device__ __forceinline__ void put(int layout, float* a, float* b, int64_t idx, float re,
                                    float im) {
    if (layout == TSG_LAYOUT_PLANES) {
        a[idx] = re;
        b[idx] = im;
    } else if (layout == TSG_LAYOUT_COMPLEX_IJ) {
        // The public MRF value 1j * s.
        reinterpret_cast<float2*>(a)[idx] = make_float2(-im, re);
    } else {
        reinterpret_cast<float2*>(a)[idx] = make_float2(re, im);
    }
}

// The transcendentals of one op for one voxel: the relaxation (e1, and the
// F+ factor e2 e^{-i 2 pi B0 dt} as tr + i ti), the pulse (sin/cos of the
// flip angle alpha = flip B1 and of the RF phase plus B1phase) and the
// receiver phase of a record. Left at the identity where the op has no such
// step.
struct OpTrig {
    float e1 = 1.f, tr = 1.f, ti = 0.f;
    float sa = 0.f, ca = 1.f, sp = 0.f, cp = 1.f;
    float sr = 0.f, cr = 1.f;
};

__device__ __forceinline__ OpTrig op_trig(const Op& op, float2 ph, float r1, float r2, float b1,
                                          float b1_phase, float b0, bool off_axis) {
    OpTrig t;
    const uint32_t code = op.code;
    if (code & OP_RELAX) {
        t.e1 = expf(-r1 * op.dt);
        const float e2 = expf(-r2 * op.dt);
        float so = 0.f, co = 1.f;
        if (off_axis) sincosf(-2.f * 3.14159265358979323846f * b0 * op.dt, &so, &co);
        t.tr = e2 * co;
        t.ti = e2 * so;
    }
    if (op_rf(code) == RF_ROTATE) {
        sincosf(op.flip * b1, &t.sa, &t.ca);
        sincosf(ph.x + b1_phase, &t.sp, &t.cp);
    }
    if (code & OP_RECORD) sincosf(ph.y, &t.sr, &t.cr);
    return t;
}

}  // namespace complex_detail

}  // namespace tsg
