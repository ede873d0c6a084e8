// The first-order adjoint of the complex EPG sweep (one pool, instant RF):
// gradients with respect to T1, T2, M0, B1, the inversion efficiency, the
// transmit phase (B1phase) and off-resonance (B0) per voxel, and the flip,
// duration and phase of every event -- the reference's complex
// simulate_vjp_range<INSTANT, ONE> (src/torchsim/_epg_cpu.cpp:4840-5985).
//
// Trajectory mode, as the real adjoint's: a forward sweep stores every op's
// entry state (the six real planes F+ re/im, F- re/im, Z re/im of each lane's
// order pairs, one tile per warp so that stores and loads are whole lines)
// and every recorded F+[0]; the reverse sweep streams them back through a
// cp.async ring and re-applies only each op's relaxation and pre-shift.
//
// Adjoint algebra (complex cotangents y_bar = dL/dRe y + i dL/dIm y; for
// y = a x the cotangent is x_bar = conj(a) y_bar, and a parameter p of a
// contributes Re(sum conj(y_bar) (da/dp) x)):
//   pulse    x_bar = T^H y_bar; T^H has T's form with B -> conj(C),
//            C -> conj(B); dL/dalpha, dL/dphi from T's derivatives.
//   record   v = m0 F+[0] e^{-i phi_r}: F+[0]_bar += m0 e^{i phi_r} g;
//            dL/dm0 = Re(conj(g) F+[0] e^{-i phi_r}), dL/dphi_r = Re(conj(g) (-i v)).
//   relax    F+ *= T, F- *= conj(T), T = e2 e^{i off}, off = -2 pi B0 dt;
//            with the pre-pulse states and cotangents (the shift commutes
//            with these inner products): dL/dlog e2 = <pb, p> + <mb, m>,
//            dL/doff = <pb, i p> + <mb, -i m>, dL/dlog e1 = <zb, z> - Re zb[0].
#include "epg_complex.cuh"

namespace tsg {

namespace {

using namespace complex_detail;

constexpr int kCxWarps = 2;
constexpr int kCxRing = 2;

struct ComplexAdjointArgs {
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
    // Forward: the signal (nullable), the trajectory
    // [train][warp][op][6 planes][lane][RP] float2 and the recorded F+[0]
    // [train][output][atom] float2.
    int layout;
    float* out_a;
    float* out_b;
    float2* traj;
    float2* traj_rec;
    // Reverse: the complex seed (planes or interleaved complex), partials
    // per (train, warp, op) 2 float2 (flip, duration), (pulse phase,
    // receiver phase) and per (train, atom) 7 floats (t1, t2, m0, b1,
    // inversion, b1 phase, b0).
    const float* seed_a;
    const float* seed_b;
    int seed_layout;
    float2* event_partial;
    float* tissue_partial;
    int64_t warps_per_train;
};

// Transpose of shift_complex on the cotangents: F+ cotangents move one order
// down, F- cotangents one order up, and F+[0] = conj(F-[0]) returns
// conj(pb[0]) to the F- order that became F-[0]. The slot at order `states`
// only receives F- cotangent from below; it is kept empty.
template <int RP, int L>
__device__ __forceinline__ void shift_complex_adjoint(float2 (&pr)[RP], float2 (&pi)[RP],
                                                      float2 (&mr)[RP], float2 (&mi)[RP], int q,
                                                      bool kill, int kill_r) {
    const float carry_r = pr[0].x, carry_i = -pi[0].x;
    float in_pr = 0.f, in_pi = 0.f, in_mr = 0.f, in_mi = 0.f;
    if constexpr (L > 1) {
        in_pr = __shfl_down_sync(0xffffffffu, pr[0].x, 1);
        in_pi = __shfl_down_sync(0xffffffffu, pi[0].x, 1);
        in_mr = __shfl_up_sync(0xffffffffu, mr[RP - 1].y, 1);
        in_mi = __shfl_up_sync(0xffffffffu, mi[RP - 1].y, 1);
    }
    const bool top_lane = L == 1 || q == L - 1;
#pragma unroll
    for (int k = 0; k < RP; ++k) {
        pr[k].x = pr[k].y;
        pi[k].x = pi[k].y;
        pr[k].y = (k + 1 < RP) ? pr[k + 1].x : (top_lane ? 0.f : in_pr);
        pi[k].y = (k + 1 < RP) ? pi[k + 1].x : (top_lane ? 0.f : in_pi);
    }
    const bool first = L == 1 || q == 0;
#pragma unroll
    for (int k = RP - 1; k >= 0; --k) {
        mr[k].y = mr[k].x;
        mi[k].y = mi[k].x;
        mr[k].x = (k > 0) ? mr[k - 1].y : (first ? 0.f : in_mr);
        mi[k].x = (k > 0) ? mi[k - 1].y : (first ? 0.f : in_mi);
    }
    if (first) {
        mr[0].y += carry_r;
        mi[0].y += carry_i;
    }
    if (kill) {
#pragma unroll
        for (int k = 0; k < RP; ++k) {
            if (2 * k == kill_r) mr[k].x = mi[k].x = 0.f;
            if (2 * k + 1 == kill_r) mr[k].y = mi[k].y = 0.f;
        }
    }
}

// The conjugate transpose of a pulse: the same form with B -> conj(C) and
// C -> conj(B).
__device__ __forceinline__ Pulse hermitian(const Pulse& u) {
    Pulse h = u;
    h.B_r = u.C_r;
    h.B_i = u.nC_i;
    h.nB_i = u.C_i;
    h.C_r = u.B_r;
    h.C_i = u.nB_i;
    h.nC_i = u.B_i;
    return h;
}

// d/dphi of a pulse: diagonal 0, A -> 2iA, B -> -iB, C -> iC.
__device__ __forceinline__ Pulse phase_derivative(const Pulse& u) {
    Pulse d;
    d.t00 = d.t22 = dup(0.f);
    d.A_r = mul2(dup(-2.f), u.A_i);
    d.A_i = mul2(dup(2.f), u.A_r);
    d.nA_i = mul2(dup(-2.f), u.A_r);
    d.B_r = u.B_i;
    d.B_i = mul2(dup(-1.f), u.B_r);
    d.nB_i = u.B_r;
    d.C_r = u.nC_i;
    d.C_i = u.C_r;
    d.nC_i = mul2(dup(-1.f), u.C_r);
    return d;
}

// Forward storing the trajectory.
template <int RP, int L>
__global__ void __launch_bounds__(128) complex_forward_traj_kernel(const ComplexAdjointArgs a) {
    constexpr int R = 2 * RP;
    constexpr int VPW = 32 / L;
    __shared__ Op s_ops[kComplexOpChunk];
    __shared__ float2 s_ph[kComplexOpChunk];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int q = lane % L;
    const int slot = lane / L;
    const int64_t warp_global = int64_t(blockIdx.x) * (blockDim.x >> 5) + warp;
    const int64_t atom = warp_global * VPW + slot;
    const int64_t train = blockIdx.y;
    const bool active = slot < VPW && atom < a.atoms;
    const int64_t ac = active ? atom : 0;
    const float r1 = 1000.f / a.t1[ac];
    const float r2 = 1000.f / a.t2[ac];
    const float m0 = a.m0 ? a.m0[ac] : 1.f;
    const float b1 = a.b1 ? a.b1[ac] : 1.f;
    const float eff = a.inv ? a.inv[ac] : 1.f;
    const float b1_phase = a.b1_phase ? a.b1_phase[ac] : 0.f;
    const float b0 = a.b0 ? a.b0[ac] : 0.f;
    const bool kill = L * R > a.states;
    const int kill_r = a.states - q * R;

    float2 X[6][RP];  // Pr, Pi, Mr, Mi, Zr, Zi
#pragma unroll
    for (int p = 0; p < 6; ++p)
#pragma unroll
        for (int k = 0; k < RP; ++k) X[p][k] = dup(0.f);
    if (q == 0) X[4][0].x = 1.f;

    const Op* ops = a.ops + train * a.n_ops;
    const float2* phase = a.phase + train * a.n_ops;
    const int64_t row = train * a.atoms + atom;
    const int64_t n_warps = (a.atoms + VPW - 1) / VPW;
    const int64_t op_stride = 6 * 32 * RP;
    float2* lane_traj = warp_global < n_warps
                            ? a.traj + (train * n_warps + warp_global) * a.n_ops * op_stride + lane * RP
                            : nullptr;

    // Each op's transcendentals are the same for the L lanes of a voxel:
    // lane q evaluates them for one of the next L ops and the lanes exchange
    // them by shuffle.
    const int first_lane = lane - q;
    const bool off_axis = a.b0 != nullptr;
    OpTrig mine;

    for (int base = 0; base < a.n_ops; base += kComplexOpChunk) {
        const int count = min(kComplexOpChunk, a.n_ops - base);
        __syncthreads();
        for (int i = threadIdx.x; i < count; i += blockDim.x) {
            s_ops[i] = ops[base + i];
            s_ph[i] = phase[base + i];
        }
        __syncthreads();
        for (int i = 0; i < count; ++i) {
            const Op op = s_ops[i];
            const uint32_t code = op.code;
            const int src = first_lane + i % L;
            if constexpr (L > 1) {
                if (i % L == 0) {
                    const int j = i + q;
                    mine = j < count ? op_trig(s_ops[j], s_ph[j], r1, r2, b1, b1_phase, b0, off_axis)
                                     : OpTrig{};
                }
            } else {
                mine = op_trig(op, s_ph[i], r1, r2, b1, b1_phase, b0, off_axis);
            }
            // This op's value of one field (shuffled where it is used, so the
            // fields are live only there; every lane takes part).
            auto tv = [&](float v) { return L > 1 ? __shfl_sync(0xffffffffu, v, src) : v; };
            if (lane_traj) {
                float2* dst = lane_traj + int64_t(base + i) * op_stride;
#pragma unroll
                for (int p = 0; p < 6; ++p)
#pragma unroll
                    for (int k = 0; k < RP; ++k) dst[p * 32 * RP + k] = X[p][k];
            }
            if (code & OP_RELAX) {
                const float e1 = tv(mine.e1), tr = tv(mine.tr), ti = tv(mine.ti);
                const float2 T = dup(tr), Ti = dup(ti), nTi = dup(-ti), E1 = dup(e1);
#pragma unroll
                for (int k = 0; k < RP; ++k) {
                    const float2 pr = X[0][k], pi = X[1][k], mr = X[2][k], mi = X[3][k];
                    X[0][k] = fma2(nTi, pi, mul2(T, pr));
                    X[1][k] = fma2(Ti, pr, mul2(T, pi));
                    X[2][k] = fma2(Ti, mi, mul2(T, mr));
                    X[3][k] = fma2(nTi, mr, mul2(T, mi));
                    X[4][k] = mul2(X[4][k], E1);
                    X[5][k] = mul2(X[5][k], E1);
                }
                if (q == 0) X[4][0].x += 1.f - e1;
            }
            for (int s = 0; s < op_shift1(code); ++s)
                shift_complex<RP, L>(X[0], X[1], X[2], X[3], q, kill, kill_r);
            const int rf = op_rf(code);
            if (rf == RF_ROTATE) {
                const float sa = tv(mine.sa), ca = tv(mine.ca), sp = tv(mine.sp), cp = tv(mine.cp);
                const float c2 = cp * cp - sp * sp, s2 = 2.f * cp * sp;
                const Pulse u = pulse_of(0.5f * (1.f + ca), ca, 0.5f * (1.f - ca), sa, 0.5f * sa,
                                         c2, s2, cp, sp);
#pragma unroll
                for (int k = 0; k < RP; ++k)
                    apply(u, X[0][k], X[1][k], X[2][k], X[3][k], X[4][k], X[5][k], X[0][k],
                          X[1][k], X[2][k], X[3][k], X[4][k], X[5][k]);
            } else if (rf == RF_INVERT) {
                const float2 f = dup(-eff);
#pragma unroll
                for (int k = 0; k < RP; ++k) {
                    X[4][k] = mul2(X[4][k], f);
                    X[5][k] = mul2(X[5][k], f);
                }
            }
            for (int s = 0; s < op_shift2(code); ++s)
                shift_complex<RP, L>(X[0], X[1], X[2], X[3], q, kill, kill_r);
            if (code & OP_SPOIL1) {
#pragma unroll
                for (int k = 0; k < RP; ++k) X[0][k] = X[1][k] = X[2][k] = X[3][k] = dup(0.f);
            }
            float sr = 0.f, cr = 1.f;
            if (code & OP_RECORD) {
                sr = tv(mine.sr);
                cr = tv(mine.cr);
            }
            if ((code & OP_RECORD) && q == 0 && active) {
                const float xr = X[0][0].x, xi = X[1][0].x;
                a.traj_rec[(train * a.outputs + op.record) * a.atoms + atom] = make_float2(xr, xi);
                if (a.out_a)
                    put(a.layout, a.out_a, a.out_b, row * a.outputs + op.record,
                        m0 * (xr * cr + xi * sr), m0 * (xi * cr - xr * sr));
            }
            for (int s = 0; s < op_shift3(code); ++s)
                shift_complex<RP, L>(X[0], X[1], X[2], X[3], q, kill, kill_r);
            if (code & OP_SPOIL2) {
#pragma unroll
                for (int k = 0; k < RP; ++k) X[0][k] = X[1][k] = X[2][k] = X[3][k] = dup(0.f);
            }
        }
    }
}

// <y, x> summed over a lane's pairs: the real inner product of two planes.
template <int RP>
__device__ __forceinline__ float2 dot_acc(const float2 (&y)[RP], const float2 (&x)[RP], float2 acc) {
#pragma unroll
    for (int k = 0; k < RP; ++k) acc = fma2(y[k], x[k], acc);
    return acc;
}

// The reverse sweep. Dynamic shared memory: the entry-state ring
// [D][6][T][RP] float2, then the ops [n_ops] and their phases [n_ops].
// Two orders per lane (the default shapes) hold the reverse step in 96
// registers, ten blocks per SM; four orders per lane take what they need.
template <int RP, int L>
__global__ void __launch_bounds__(32 * kCxWarps, RP == 1 ? 10 : 1)
    complex_adjoint_kernel(const ComplexAdjointArgs a) {
    extern __shared__ __align__(16) unsigned char s_raw[];
    constexpr int W = kCxWarps;
    constexpr int T = 32 * W;
    constexpr int R = 2 * RP;
    constexpr int VPW = 32 / L;
    constexpr int D = kCxRing;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int q = lane % L;
    const int slot = lane / L;
    const int64_t warp_global = int64_t(blockIdx.x) * W + warp;
    const int64_t atom = warp_global * VPW + slot;
    const int64_t train = blockIdx.y;
    const bool active = slot < VPW && atom < a.atoms;
    const int64_t ac = active ? atom : 0;
    const bool lane0 = active && q == 0;
    const int n_ops = a.n_ops;
    const int64_t n = a.atoms;
    const int64_t row = train * n + atom;
    const float t1 = a.t1[ac], t2 = a.t2[ac];
    const float r1 = 1000.f / t1, r2 = 1000.f / t2;
    const float w1 = 1000.f / (t1 * t1), w2 = 1000.f / (t2 * t2);
    const float m0 = a.m0 ? a.m0[ac] : 1.f;
    const float b1 = a.b1 ? a.b1[ac] : 1.f;
    const float eff = a.inv ? a.inv[ac] : 1.f;
    const float b1_phase = a.b1_phase ? a.b1_phase[ac] : 0.f;
    const float b0 = a.b0 ? a.b0[ac] : 0.f;
    const bool kill = L * R > a.states;
    const int kill_r = a.states - q * R;
    constexpr float kTwoPi = 6.28318530717958647692f;

    float2* s_ring = reinterpret_cast<float2*>(s_raw);           // [D][6][T][RP]
    Op* s_ops = reinterpret_cast<Op*>(s_ring + D * 6 * T * RP);  // [n_ops]
    float2* s_ph = reinterpret_cast<float2*>(s_ops + n_ops);     // [n_ops]
    {
        const Op* ops = a.ops + train * n_ops;
        const float2* ph = a.phase + train * n_ops;
        for (int i = threadIdx.x; i < n_ops; i += T) {
            s_ops[i] = ops[i];
            s_ph[i] = ph[i];
        }
        __syncthreads();
    }

    const int64_t n_warps = (n + VPW - 1) / VPW;
    const int64_t op_stride = 6 * 32 * RP;
    const float2* lane_traj =
        a.traj + (train * n_warps + (warp_global < n_warps ? warp_global : 0)) * n_ops * op_stride +
        lane * RP;
    const unsigned ring_base =
        static_cast<unsigned>(__cvta_generic_to_shared(s_ring + threadIdx.x * RP));
    auto fetch = [&](int o, int rs) {
        const float2* src = lane_traj + o * op_stride;
        const unsigned dst = ring_base + unsigned(rs * 6 * T * RP) * 8u;
#pragma unroll
        for (int p = 0; p < 6; ++p) {
            if constexpr (RP == 2) {
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(
                                 dst + unsigned(p * T * RP) * 8u),
                             "l"(src + p * 32 * RP)
                             : "memory");
            } else {
#pragma unroll
                for (int k = 0; k < RP; ++k)
                    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(
                                     dst + unsigned(p * T * RP + k) * 8u),
                                 "l"(src + p * 32 * RP + k)
                                 : "memory");
            }
        }
    };

    // Seeds: planes (re plane, im plane) or interleaved complex.
    const bool planes = a.seed_layout == TSG_LAYOUT_PLANES;
    const float2* rec_col = a.traj_rec + train * int64_t(a.outputs) * n + ac;

    float2 B[6][RP];  // cotangents Pr, Pi, Mr, Mi, Zr, Zi
#pragma unroll
    for (int p = 0; p < 6; ++p)
#pragma unroll
        for (int k = 0; k < RP; ++k) B[p][k] = dup(0.f);
    float g_t1 = 0.f, g_t2 = 0.f, g_m0 = 0.f, g_b1 = 0.f, g_inv = 0.f, g_b1p = 0.f, g_b0 = 0.f;

#pragma unroll
    for (int j = 1; j < D; ++j) {
        if (n_ops - j >= 0) fetch(n_ops - j, j - 1);
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    }
    float2* event_out = a.event_partial + (train * a.warps_per_train + warp_global) * int64_t(n_ops) * 2;
    int use_slot = 0, fill_slot = D - 1;
    // Each op's transcendentals, evaluated once per voxel: lane q takes one
    // of the next L ops of the reverse sweep (op o - q) and the lanes
    // exchange them by shuffle.
    const int first_lane = lane - q;
    const bool off_axis = a.b0 != nullptr;
    OpTrig mine;

    for (int o = n_ops - 1; o >= 0; --o) {
        if (o - (D - 1) >= 0) fetch(o - (D - 1), fill_slot);
        asm volatile("cp.async.commit_group;\n" ::: "memory");
        fill_slot = fill_slot + 1 == D ? 0 : fill_slot + 1;
        const Op op = s_ops[o];
        const float2 ph = s_ph[o];
        const uint32_t code = op.code;
        const int g = (n_ops - 1 - o) % L;
        const int src = first_lane + g;
        if constexpr (L > 1) {
            if (g == 0) {
                const int j = o - q;
                mine = j >= 0 ? op_trig(s_ops[j], s_ph[j], r1, r2, b1, b1_phase, b0, off_axis)
                              : OpTrig{};
            }
        } else {
            mine = op_trig(op, ph, r1, r2, b1, b1_phase, b0, off_axis);
        }
        // This op's value of one field (shuffled where it is used, so the
        // fields are live only there; every lane takes part).
        auto tv = [&](float v) { return L > 1 ? __shfl_sync(0xffffffffu, v, src) : v; };
        asm volatile("cp.async.wait_group %0;\n" ::"n"(D - 1) : "memory");
        const float2* ring = s_ring + use_slot * (6 * T * RP) + threadIdx.x * RP;
        use_slot = use_slot + 1 == D ? 0 : use_slot + 1;
        float2 X[6][RP];
#pragma unroll
        for (int p = 0; p < 6; ++p)
#pragma unroll
            for (int k = 0; k < RP; ++k) X[p][k] = ring[p * T * RP + k];

        // Replay the relaxation (and the turn) and the pre-shift.
        const bool relax = (code & OP_RELAX) != 0;
        float e1 = 1.f, tr = 1.f, ti = 0.f;
        if (relax) {
            e1 = tv(mine.e1);
            tr = tv(mine.tr);
            ti = tv(mine.ti);
            const float2 Tr = dup(tr), Ti = dup(ti), nTi = dup(-ti), E1 = dup(e1);
#pragma unroll
            for (int k = 0; k < RP; ++k) {
                const float2 pr = X[0][k], pi = X[1][k], mr = X[2][k], mi = X[3][k];
                X[0][k] = fma2(nTi, pi, mul2(Tr, pr));
                X[1][k] = fma2(Ti, pr, mul2(Tr, pi));
                X[2][k] = fma2(Ti, mi, mul2(Tr, mr));
                X[3][k] = fma2(nTi, mr, mul2(Tr, mi));
                X[4][k] = mul2(X[4][k], E1);
                X[5][k] = mul2(X[5][k], E1);
            }
            if (q == 0) X[4][0].x += 1.f - e1;
        }
        for (int s = 0; s < op_shift1(code); ++s)
            shift_complex<RP, L>(X[0], X[1], X[2], X[3], q, kill, kill_r);

        // The op's micro-steps after the pulse, reversed.
        if (code & OP_SPOIL2) {
#pragma unroll
            for (int k = 0; k < RP; ++k) B[0][k] = B[1][k] = B[2][k] = B[3][k] = dup(0.f);
        }
        for (int s = 0; s < op_shift3(code); ++s)
            shift_complex_adjoint<RP, L>(B[0], B[1], B[2], B[3], q, kill, kill_r);
        float e_rec = 0.f;  // this lane's d/d(receiver phase)
        float sr = 0.f, cr = 1.f;
        if (code & OP_RECORD) {
            sr = tv(mine.sr);
            cr = tv(mine.cr);
        }
        if ((code & OP_RECORD) && lane0) {
            const int64_t r = op.record;
            const int64_t idx = row * a.outputs + r;
            float gr, gi;
            if (planes) {
                gr = a.seed_a[idx];
                gi = a.seed_b[idx];
            } else {
                const float2 gs = reinterpret_cast<const float2*>(a.seed_a)[idx];
                gr = gs.x;
                gi = gs.y;
            }
            const float2 x0 = rec_col[r * n];
            // d = e^{-i phi_r}: x0 d, and v = m0 x0 d.
            const float fr = x0.x * cr + x0.y * sr, fi = x0.y * cr - x0.x * sr;
            g_m0 = fmaf(gr, fr, fmaf(gi, fi, g_m0));
            // dv/dphi_r = -i v: Re(conj(g) (-i v)) = m0 (gr fi - gi fr).
            e_rec = m0 * (gr * fi - gi * fr);
            // F+[0]_bar += m0 conj(d) g = m0 e^{i phi_r} g.
            B[0][0].x += m0 * (cr * gr - sr * gi);
            B[1][0].x += m0 * (cr * gi + sr * gr);
        }
        if (code & OP_SPOIL1) {
#pragma unroll
            for (int k = 0; k < RP; ++k) B[0][k] = B[1][k] = B[2][k] = B[3][k] = dup(0.f);
        }
        for (int s = 0; s < op_shift2(code); ++s)
            shift_complex_adjoint<RP, L>(B[0], B[1], B[2], B[3], q, kill, kill_r);

        float e_flip = 0.f, e_rf = 0.f;
        const int rf = op_rf(code);
        if (rf == RF_ROTATE) {
            const float sa = tv(mine.sa), ca = tv(mine.ca), sp = tv(mine.sp), cp = tv(mine.cp);
            const float c2 = cp * cp - sp * sp, s2 = 2.f * cp * sp;
            const Pulse u = pulse_of(0.5f * (1.f + ca), ca, 0.5f * (1.f - ca), sa, 0.5f * sa, c2,
                                     s2, cp, sp);
            const Pulse da = pulse_of(-0.5f * sa, -sa, 0.5f * sa, ca, 0.5f * ca, c2, s2, cp, sp);
            const Pulse dp = phase_derivative(u);
            const Pulse uh = hermitian(u);
            float2 ga = dup(0.f), gp = dup(0.f);
#pragma unroll
            for (int k = 0; k < RP; ++k) {
                float2 v[6];
                apply(da, X[0][k], X[1][k], X[2][k], X[3][k], X[4][k], X[5][k], v[0], v[1], v[2],
                      v[3], v[4], v[5]);
#pragma unroll
                for (int p = 0; p < 6; ++p) ga = fma2(B[p][k], v[p], ga);
                apply(dp, X[0][k], X[1][k], X[2][k], X[3][k], X[4][k], X[5][k], v[0], v[1], v[2],
                      v[3], v[4], v[5]);
#pragma unroll
                for (int p = 0; p < 6; ++p) gp = fma2(B[p][k], v[p], gp);
                apply(uh, B[0][k], B[1][k], B[2][k], B[3][k], B[4][k], B[5][k], B[0][k], B[1][k],
                      B[2][k], B[3][k], B[4][k], B[5][k]);
            }
            const float gsa = ga.x + ga.y, gsp = gp.x + gp.y;
            e_flip = gsa * b1;
            g_b1 = fmaf(gsa, op.flip, g_b1);
            e_rf = gsp;
            g_b1p += gsp;
        } else if (rf == RF_INVERT) {
            const float2 f = dup(-eff);
            float2 acc = dup(0.f);
            acc = dot_acc<RP>(B[4], X[4], acc);
            acc = dot_acc<RP>(B[5], X[5], acc);
            g_inv -= acc.x + acc.y;
#pragma unroll
            for (int k = 0; k < RP; ++k) {
                B[4][k] = mul2(B[4][k], f);
                B[5][k] = mul2(B[5][k], f);
            }
        }
        float e_dt = 0.f;
        if (relax) {
            // At the pre-pulse point: dL/dlog e2, dL/doff, dL/dlog e1.
            float2 q2 = dup(0.f), qo = dup(0.f), q1 = dup(0.f);
            q2 = dot_acc<RP>(B[0], X[0], q2);
            q2 = dot_acc<RP>(B[1], X[1], q2);
            q2 = dot_acc<RP>(B[2], X[2], q2);
            q2 = dot_acc<RP>(B[3], X[3], q2);
#pragma unroll
            for (int k = 0; k < RP; ++k) {
                // <pb, i p> = -pbr pi + pbi pr; <mb, -i m> = mbr mi - mbi mr.
                qo = fma2(B[1][k], X[0][k], fma2(mul2(dup(-1.f), B[0][k]), X[1][k], qo));
                qo = fma2(B[2][k], X[3][k], fma2(mul2(dup(-1.f), B[3][k]), X[2][k], qo));
            }
            q1 = dot_acc<RP>(B[4], X[4], q1);
            q1 = dot_acc<RP>(B[5], X[5], q1);
            const float G2 = q2.x + q2.y, Go = qo.x + qo.y;
            const float G1 = q1.x + q1.y - (q == 0 ? B[4][0].x : 0.f);
            g_t2 = fmaf(G2, op.dt * w2, g_t2);
            g_t1 = fmaf(G1, op.dt * w1, g_t1);
            g_b0 = fmaf(Go, -kTwoPi * op.dt, g_b0);
            e_dt = -r2 * G2 - r1 * G1 - kTwoPi * b0 * Go;
        }
        for (int s = 0; s < op_shift1(code); ++s)
            shift_complex_adjoint<RP, L>(B[0], B[1], B[2], B[3], q, kill, kill_r);
        if (relax) {
            // F+_bar *= conj(T), F-_bar *= T, Z_bar *= e1.
            const float2 Tr = dup(tr), Ti = dup(ti), nTi = dup(-ti), E1 = dup(e1);
#pragma unroll
            for (int k = 0; k < RP; ++k) {
                const float2 pr = B[0][k], pi = B[1][k], mr = B[2][k], mi = B[3][k];
                B[0][k] = fma2(Ti, pi, mul2(Tr, pr));
                B[1][k] = fma2(nTi, pr, mul2(Tr, pi));
                B[2][k] = fma2(nTi, mi, mul2(Tr, mr));
                B[3][k] = fma2(Ti, mr, mul2(Tr, mi));
                B[4][k] = mul2(B[4][k], E1);
                B[5][k] = mul2(B[5][k], E1);
            }
        }
        // The op's event partials summed over the warp (fixed butterfly).
        float ev[4] = {active ? e_flip : 0.f, active ? e_dt : 0.f, active ? e_rf : 0.f,
                       active ? e_rec : 0.f};
#pragma unroll
        for (int off = 16; off > 0; off >>= 1)
#pragma unroll
            for (int e = 0; e < 4; ++e) ev[e] += __shfl_xor_sync(0xffffffffu, ev[e], off);
        if (lane == 0) {
            event_out[int64_t(o) * 2] = make_float2(ev[0], ev[1]);
            event_out[int64_t(o) * 2 + 1] = make_float2(ev[2], ev[3]);
        }
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    float out[7] = {g_t1, g_t2, g_m0, g_b1, g_inv, g_b1p, g_b0};
#pragma unroll
    for (int j = 0; j < 7; ++j) {
        const float x = active ? out[j] : 0.f;
        float sum = 0.f;
#pragma unroll
        for (int l = 0; l < L; ++l) sum += __shfl_sync(0xffffffffu, x, lane - q + l);
        out[j] = sum;
    }
    if (lane0) {
        float* dst = a.tissue_partial + row * 7;
#pragma unroll
        for (int j = 0; j < 7; ++j) dst[j] = out[j];
    }
}

// Sums the per-warp event partials (one block per op and train, a fixed
// tree) and scatters them: flip and duration to the op's RF and dt events,
// the pulse phase to its RF event, the receiver phase to its record event.
__global__ void __launch_bounds__(kEventReduceThreads)
    reduce_complex_events(const float2* partial, int64_t warps, int64_t n_ops, int64_t events,
                          const OpSource* src, float* g_flip, float* g_dt, float* g_phase) {
    __shared__ float4 s_sum[kEventReduceThreads];
    const int64_t op = blockIdx.x;
    const int64_t t = blockIdx.y;
    const float2* p = partial + (t * warps * n_ops + op) * 2;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int64_t w = threadIdx.x; w < warps; w += kEventReduceThreads) {
        const float2 x = p[w * n_ops * 2], y = p[w * n_ops * 2 + 1];
        acc.x += x.x;
        acc.y += x.y;
        acc.z += y.x;
        acc.w += y.y;
    }
    s_sum[threadIdx.x] = acc;
    __syncthreads();
    for (int half = kEventReduceThreads / 2; half > 0; half >>= 1) {
        if (threadIdx.x < half) {
            float4& d = s_sum[threadIdx.x];
            const float4 e = s_sum[threadIdx.x + half];
            d.x += e.x;
            d.y += e.y;
            d.z += e.z;
            d.w += e.w;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const float4 c = s_sum[0];
        const OpSource s = src[t * n_ops + op];
        if (s.rf_event >= 0) {
            if (g_flip) g_flip[t * events + s.rf_event] += c.x;
            if (g_phase) g_phase[t * events + s.rf_event] += c.z;
        }
        if (s.dt_event >= 0 && g_dt) g_dt[t * events + s.dt_event] += c.y;
        if (s.rec_event >= 0 && g_phase) g_phase[t * events + s.rec_event] += c.w;
    }
}

// The seven per-atom gradient slots (t1, t2, m0, b1, inversion, b1 phase,
// b0), passed by value.
struct TissueSlots7 {
    float* p[7];
};

// Per atom, the trains' tissue partials in train order, added into the
// gradients.
__global__ void reduce_complex_tissue(const float* partial, int64_t atoms, int64_t trains,
                                      TissueSlots7 out) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= atoms) return;
    for (int j = 0; j < 7; ++j) {
        float sum = 0.f;
        for (int64_t t = 0; t < trains; ++t) sum += partial[(t * atoms + i) * 7 + j];
        if (out.p[j]) out.p[j][i] += sum;
    }
}

struct CxEntry {
    int orders_per_lane;
    int lanes_per_voxel;
    void (*forward)(const ComplexAdjointArgs&, dim3, dim3, cudaStream_t);
    void (*reverse)(const ComplexAdjointArgs&, dim3, dim3, size_t, cudaStream_t);
    const void* reverse_fn;
};

template <int RP, int L>
void launch_cx_forward(const ComplexAdjointArgs& a, dim3 g, dim3 b, cudaStream_t s) {
    complex_forward_traj_kernel<RP, L><<<g, b, 0, s>>>(a);
}
template <int RP, int L>
void launch_cx_reverse(const ComplexAdjointArgs& a, dim3 g, dim3 b, size_t smem, cudaStream_t s) {
    complex_adjoint_kernel<RP, L><<<g, b, smem, s>>>(a);
}

#define TSG_CX_ENTRY(R, L)                                                           \
    {R, L, &launch_cx_forward<(R) / 2, L>, &launch_cx_reverse<(R) / 2, L>,           \
     reinterpret_cast<const void*>(&complex_adjoint_kernel<(R) / 2, L>)}

const CxEntry kCx[] = {
    TSG_CX_ENTRY(2, 2),  TSG_CX_ENTRY(2, 4),  TSG_CX_ENTRY(2, 5),  TSG_CX_ENTRY(2, 8),
    TSG_CX_ENTRY(2, 10), TSG_CX_ENTRY(2, 16), TSG_CX_ENTRY(2, 32), TSG_CX_ENTRY(4, 1),
    TSG_CX_ENTRY(4, 2),  TSG_CX_ENTRY(4, 4),  TSG_CX_ENTRY(4, 5),  TSG_CX_ENTRY(4, 8),
    TSG_CX_ENTRY(4, 16),
};

struct CxPlan {
    const CxEntry* entry = nullptr;
    int64_t blocks = 0;
    int64_t warps_per_train = 0;
    int64_t state_bytes = 0;
    int64_t trajectory_bytes = 0;
    int64_t event_bytes = 0;
    int64_t workspace_bytes = 0;
    size_t smem = 0;
};

int cx_plan(const tsg_program* prog, int64_t atoms, int64_t states, const tsg_launch* want,
            CxPlan* plan) {
    if (!prog) return fail(TSG_ERR_ARGUMENT, "null program");
    if (atoms < 0 || states < 1) return fail(TSG_ERR_ARGUMENT, "invalid EPG buffer dimensions");
    if (states > 64) return fail(TSG_ERR_CAPACITY, "the complex adjoint takes at most 64 states");
    if (!prog->d_phase && prog->host.ops > 0)
        return fail(TSG_ERR_ARGUMENT, "the complex path needs a program built with event phases");
    const CxEntry* best = nullptr;
    for (const CxEntry& e : kCx) {
        if (want && want->lanes_per_voxel > 0 && e.lanes_per_voxel != want->lanes_per_voxel) continue;
        if (want && want->orders_per_lane > 0 && e.orders_per_lane != want->orders_per_lane) continue;
        if (e.lanes_per_voxel * e.orders_per_lane < states) continue;
        // Two orders per lane on the fewest lanes; four where two would need
        // more than 32 lanes.
        if (!best || e.orders_per_lane < best->orders_per_lane ||
            (e.orders_per_lane == best->orders_per_lane && e.lanes_per_voxel < best->lanes_per_voxel))
            best = &e;
    }
    if (!best) return fail(TSG_ERR_UNSUPPORTED, "no complex adjoint kernel for this state count / launch shape");
    plan->entry = best;
    const int64_t ops = prog->host.ops, trains = prog->host.trains;
    const int vpw = 32 / best->lanes_per_voxel;
    const int64_t n_warps = (atoms + vpw - 1) / vpw;
    const int vpb = kCxWarps * vpw;
    plan->blocks = (atoms + vpb - 1) / vpb;
    plan->warps_per_train = plan->blocks * kCxWarps;
    plan->state_bytes = trains * n_warps * ops * 6 * 32 * int64_t(best->orders_per_lane / 2) * 8;
    plan->trajectory_bytes =
        align256(plan->state_bytes) + trains * prog->host.outputs * atoms * int64_t(sizeof(float2));
    plan->event_bytes = align256(trains * plan->warps_per_train * ops * 2 * int64_t(sizeof(float2)));
    plan->workspace_bytes = plan->event_bytes + trains * atoms * 7 * int64_t(sizeof(float));
    plan->smem = size_t(kCxRing) * 6 * 32 * kCxWarps * size_t(best->orders_per_lane / 2) * 8 +
                 size_t(ops) * (sizeof(Op) + sizeof(float2));
    if (plan->smem > 220 * 1024)
        return fail(TSG_ERR_CAPACITY, "the program does not fit in shared memory for the reverse sweep");
    if (plan->blocks > 0x7fffffffLL || trains > 65535) return fail(TSG_ERR_CAPACITY, "launch too large");
    return TSG_OK;
}

ComplexAdjointArgs cx_args(const tsg_program* prog, const tsg_tissue* tissue,
                           const tsg_offaxis* off, int64_t atoms, int64_t states) {
    ComplexAdjointArgs a{};
    a.ops = prog->d_ops;
    a.phase = prog->d_phase;
    a.n_ops = int(prog->host.ops);
    a.atoms = atoms;
    a.states = int(states);
    a.outputs = int(prog->host.outputs);
    a.t1 = tissue->t1_ms;
    a.t2 = tissue->t2_ms;
    a.m0 = tissue->m0;
    a.b1 = tissue->b1;
    a.inv = tissue->inversion;
    a.b1_phase = off ? off->b1_phase_rad : nullptr;
    a.b0 = off ? off->b0_hz : nullptr;
    return a;
}

int cx_check(const tsg_program* prog, const tsg_tissue* tissue, int64_t atoms) {
    if (!prog) return fail(TSG_ERR_ARGUMENT, "null program");
    if (!tissue || (atoms > 0 && (!tissue->t1_ms || !tissue->t2_ms)))
        return fail(TSG_ERR_ARGUMENT, "t1 and t2 are required");
    return TSG_OK;
}

}  // namespace

}  // namespace tsg

using namespace tsg;

extern "C" int tsg_epg_complex_adjoint_plan(const tsg_program* program, int64_t atom_count,
                                            int64_t state_count, const tsg_launch* launch,
                                            int64_t* trajectory_bytes, int64_t* workspace_bytes) {
    CxPlan plan;
    int rc = cx_plan(program, atom_count, state_count, launch, &plan);
    if (rc) return rc;
    if (trajectory_bytes) *trajectory_bytes = plan.trajectory_bytes;
    if (workspace_bytes) *workspace_bytes = plan.workspace_bytes;
    return TSG_OK;
}

extern "C" int tsg_epg_forward_complex_trajectory(const tsg_program* program,
                                                  const tsg_tissue* tissue,
                                                  const tsg_offaxis* offaxis, int64_t atom_count,
                                                  int64_t state_count, int layout, float* out_a,
                                                  float* out_b, void* trajectory,
                                                  const tsg_launch* launch, void* stream) {
    int rc = cx_check(program, tissue, atom_count);
    if (rc) return rc;
    CxPlan plan;
    rc = cx_plan(program, atom_count, state_count, launch, &plan);
    if (rc) return rc;
    if (layout != TSG_LAYOUT_PLANES && layout != TSG_LAYOUT_COMPLEX_IJ && layout != TSG_LAYOUT_COMPLEX)
        return fail(TSG_ERR_ARGUMENT, "unknown output layout");
    if (layout == TSG_LAYOUT_PLANES && out_a && !out_b)
        return fail(TSG_ERR_ARGUMENT, "the planes layout writes both planes");
    if (atom_count == 0 || program->host.ops == 0) return TSG_OK;
    if (!trajectory) return fail(TSG_ERR_ARGUMENT, "null trajectory");
    ComplexAdjointArgs a = cx_args(program, tissue, offaxis, atom_count, state_count);
    a.layout = layout;
    a.out_a = out_a;
    a.out_b = out_b;
    a.traj = static_cast<float2*>(trajectory);
    a.traj_rec = reinterpret_cast<float2*>(static_cast<char*>(trajectory) + align256(plan.state_bytes));
    const int vpb = 4 * (32 / plan.entry->lanes_per_voxel);
    const int64_t blocks = (atom_count + vpb - 1) / vpb;
    if (blocks > 0x7fffffffLL) return fail(TSG_ERR_CAPACITY, "too many voxels for one launch");
    plan.entry->forward(a, dim3(unsigned(blocks), unsigned(program->host.trains)), dim3(128),
                        static_cast<cudaStream_t>(stream));
    TSG_CUDA(cudaGetLastError());
    return TSG_OK;
}

extern "C" int tsg_epg_adjoint_complex(const tsg_program* program, const tsg_tissue* tissue,
                                       const tsg_offaxis* offaxis, int64_t atom_count,
                                       int64_t state_count, const float* seed_a,
                                       const float* seed_b, int seed_layout,
                                       const void* trajectory, const tsg_gradients* gradients,
                                       const tsg_offaxis_gradients* offaxis_gradients,
                                       void* workspace, int64_t workspace_bytes,
                                       const tsg_launch* launch, void* stream) {
    int rc = cx_check(program, tissue, atom_count);
    if (rc) return rc;
    CxPlan plan;
    rc = cx_plan(program, atom_count, state_count, launch, &plan);
    if (rc) return rc;
    if (atom_count == 0 || program->host.ops == 0) return TSG_OK;
    if (!trajectory || !workspace || !seed_a) return fail(TSG_ERR_ARGUMENT, "null trajectory, workspace or seed");
    if (seed_layout != TSG_LAYOUT_PLANES && seed_layout != TSG_LAYOUT_COMPLEX)
        return fail(TSG_ERR_ARGUMENT, "the complex seed is planes or interleaved complex");
    if (seed_layout == TSG_LAYOUT_PLANES && !seed_b) return fail(TSG_ERR_ARGUMENT, "null seed plane");
    if (workspace_bytes < plan.workspace_bytes) return fail(TSG_ERR_ARGUMENT, "workspace too small");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    ComplexAdjointArgs a = cx_args(program, tissue, offaxis, atom_count, state_count);
    a.traj = const_cast<float2*>(static_cast<const float2*>(trajectory));
    a.traj_rec = reinterpret_cast<float2*>(const_cast<char*>(static_cast<const char*>(trajectory)) +
                                           align256(plan.state_bytes));
    a.seed_a = seed_a;
    a.seed_b = seed_b;
    a.seed_layout = seed_layout;
    char* ws = static_cast<char*>(workspace);
    a.event_partial = reinterpret_cast<float2*>(ws);
    a.tissue_partial = reinterpret_cast<float*>(ws + plan.event_bytes);
    a.warps_per_train = plan.warps_per_train;
    if (plan.smem > 48 * 1024)
        TSG_CUDA(cudaFuncSetAttribute(plan.entry->reverse_fn,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, int(plan.smem)));
    plan.entry->reverse(a, dim3(unsigned(plan.blocks), unsigned(program->host.trains)),
                        dim3(32 * kCxWarps), plan.smem, s);
    TSG_CUDA(cudaGetLastError());
    const int64_t ops = program->host.ops;
    float* g_phase = offaxis_gradients ? offaxis_gradients->phase_rad : nullptr;
    reduce_complex_events<<<dim3(unsigned(ops), unsigned(program->host.trains)),
                            kEventReduceThreads, 0, s>>>(
        a.event_partial, plan.warps_per_train, ops, program->host.events, program->d_src,
        gradients ? gradients->flip_rad : nullptr, gradients ? gradients->duration_s : nullptr,
        g_phase);
    TSG_CUDA(cudaGetLastError());
    TissueSlots7 slots{};
    if (gradients) {
        slots.p[0] = gradients->t1_ms;
        slots.p[1] = gradients->t2_ms;
        slots.p[2] = gradients->m0;
        slots.p[3] = gradients->b1;
        slots.p[4] = gradients->inversion;
    }
    if (offaxis_gradients) {
        slots.p[5] = offaxis_gradients->b1_phase_rad;
        slots.p[6] = offaxis_gradients->b0_hz;
    }
    reduce_complex_tissue<<<unsigned((atom_count + 127) / 128), 128, 0, s>>>(
        a.tissue_partial, atom_count, program->host.trains, slots);
    TSG_CUDA(cudaGetLastError());
    return TSG_OK;
}
