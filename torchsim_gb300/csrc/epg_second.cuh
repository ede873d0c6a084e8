// Second order: the adjoint of the tangent sweep, for K directions at once.
//
// The reference differentiates its first-order adjoint along ONE direction
// in dual numbers (forward over reverse, simulate_real_vjp_jvp_range,
// src/torchsim/_epg_cpu.cpp:7028-7330), and a design cost over a K-column
// Jacobian pays K such calls (sequence/_accelerators.py:1780-1800, one per
// column of model/_signal.py:255-268). Here the same derivatives come from
// the reverse sweep of the K-direction tangent system, in one pass:
//
//   forward   x' = A(p) x + b,   t_k' = A t_k + (dA/dp . d_k) x + db . d_k,
//             samples s = m0 F+[0](x),  j_k = m0 F+[0](t_k) + dm0_k F+[0](x)
//   loss      L = <g0, s> + sum_k <g_k, j_k>
//   reverse   mu_k  <- A^T mu_k + (record of g_k)
//             lam   <- A^T lam + sum_k (dA . d_k)^T mu_k + (record of g0, g_k)
//
// mu_k is the reference's dual value (the adjoint of seed g_k) and lam its
// tangent summed over the directions. The gradient of L with respect to the
// directions (J^T g_k, the reference's "value" side) and with respect to the
// inputs (its "curvature" side, plus J^T g0) follow per micro-step:
//
//   rotation by a = flip*b1, a'_k = dflip_k*b1 + flip*db1_k, with the pre-RF
//   state x, t_k and the post-RF cotangents lam, mu_k:
//     G_k = mu_k . R'x            (dL/da'_k)
//     dL/da = lam . R'x + sum_k (mu_k . R't_k + a'_k mu_k . R''x)
//   relaxation E = exp(-r dt), eps_k = E'_k / E = -(r'_k dt + r ddt_k),
//   with the pre-RF states and cotangents (a shift between relaxation and
//   pulse leaves the inner products unchanged):
//     Q = lam . (x - e0) + sum_k mu_k . t_k,   C_k = mu_k . (x - e0)
//     dL/dr += -dt Q - sum_k C_k ddt_k,  dL/dr'_k += -dt C_k,
//     dL/ddt += -r Q - sum_k C_k r'_k,   dL/dddt_k += -r C_k
//   (per plane pair: transverse with r2, longitudinal with r1 and the
//   recovery e0 at order 0), and r = 1000/T, r' = -1000 T'/T^2 chain to T.
//
// The forward stores every op's entry state of x and of each t_k (the
// trajectory, one tile per warp: per op, state and plane the warp's 32 lanes'
// order pairs are 32 * RP consecutive float2, so every store and every load
// is a whole, aligned line) and every recorded F+[0]; the reverse
// streams them back through a cp.async ring, so nothing is re-run but each
// op's relaxation and pre-shift. Per-event partials are summed over the warp
// with a fixed butterfly of shuffles after each op; tissue gradients are
// summed over a voxel's lanes with shuffles. No atomics: results are
// deterministic.
#pragma once
#include "epg_adjoint.cuh"

namespace tsg {

constexpr int kSecondMaxK = 3;
constexpr int kSecondRing = 2;
constexpr int kSecondWarps = 2;

struct SecondArgs {
    const Op* ops;
    const float2* op_dir;  // [K][train][ops] (d dt, d flip), or null (zero)
    int n_ops;
    int64_t atoms;
    int states;
    int outputs;
    const float* t1;
    const float* t2;
    const float* m0;
    const float* b1;
    const float* inv;
    // Per direction: tangents of t1, t2, m0, b1, inversion (nullable: zero).
    const float* dir[kSecondMaxK][5];
    // Forward outputs (nullable): signal (train, atom, output) and the K
    // derivatives, then with `with_m0` the derivative along M0 (F+[0]
    // itself): (train, atom, K + with_m0, output).
    int layout;
    int with_m0;
    float* sig_a;
    float* sig_b;
    float* jac_a;
    float* jac_b;
    // Trajectory: [train][warp][op][state][plane][lane][RP] float2 (state
    // 0 = x, k + 1 = t_k; warp = atom / (32 / lanes_per_voxel)), and the
    // recorded F+[0] of each state, [train][output][state][atom].
    float2* traj;
    float* traj_rec;
    // Reverse: cotangents of the signal (nullable) and of the derivatives
    // (laid out as the forward writes them).
    const float* seed0;
    const float* seed;
    int seed_layout;
    // Per (train, atom): curvature t1, t2, m0, b1, inversion, then per
    // direction the values t1, t2, m0, b1, inversion.
    float* tissue_partial;
    // Per (train, warp, op): the curvature (flip, duration), then for K == 1
    // the values (flip, duration).
    float2* event_partial;
    int64_t warps_per_train;
};

// Warps (trajectory tiles) per train for lanes_per_voxel lanes a voxel.
inline int64_t second_warps(int64_t atoms, int lanes_per_voxel) {
    const int64_t vpw = 32 / lanes_per_voxel;
    return (atoms + vpw - 1) / vpw;
}

inline int64_t second_trajectory_floats(int64_t trains, int64_t atoms, int64_t ops,
                                        int lanes_per_voxel, int orders_per_lane, int k) {
    return trains * second_warps(atoms, lanes_per_voxel) * ops * (k + 1) * 3 * 32 *
           int64_t(orders_per_lane);
}

inline int64_t second_record_floats(int64_t trains, int64_t atoms, int64_t outputs, int k) {
    return trains * outputs * (k + 1) * atoms;
}

namespace second_detail {

// One recorded sample in the given output layout (TSG_LAYOUT_*).
__device__ __forceinline__ void store_sample(int layout, float* a, float* b, int64_t idx, float v) {
    if (layout == TSG_LAYOUT_PLANES) {
        if (a) a[idx] = 0.f;
        b[idx] = v;
    } else if (layout == TSG_LAYOUT_COMPLEX) {
        reinterpret_cast<float2*>(a)[idx] = make_float2(0.f, v);
    } else {
        reinterpret_cast<float2*>(a)[idx] = make_float2(-v, 0.f);
    }
}

// A one-hot direction set (HOT != 0): direction k is the unit tangent of
// one property, (HOT >> 2k) & 3 = 1 T1, 2 T2, 3 B1, with no event
// directions; its zero terms are left out at compile time. HOT == 0: general
// directions.
__host__ __device__ constexpr int hot_dir(int hot, int k) { return (hot >> (2 * k)) & 3; }

// The voxel constants both sweeps use.
template <int K>
struct Voxel {
    float t1, t2, m0, b1, eff, r1, r2, w1, w2;
    float dt1[K], dt2[K], dm0[K], db1[K], deff[K];
};

template <int K, int HOT>
__device__ __forceinline__ Voxel<K> load_voxel(const SecondArgs& a, int64_t ac) {
    Voxel<K> v;
    v.t1 = a.t1[ac];
    v.t2 = a.t2[ac];
    v.m0 = a.m0 ? a.m0[ac] : 1.f;
    v.b1 = a.b1 ? a.b1[ac] : 1.f;
    v.eff = a.inv ? a.inv[ac] : 1.f;
    v.r1 = 1000.f / v.t1;
    v.r2 = 1000.f / v.t2;
    v.w1 = 1000.f / (v.t1 * v.t1);
    v.w2 = 1000.f / (v.t2 * v.t2);
#pragma unroll
    for (int k = 0; k < K; ++k) {
        if (HOT) {
            v.dt1[k] = hot_dir(HOT, k) == 1 ? 1.f : 0.f;
            v.dt2[k] = hot_dir(HOT, k) == 2 ? 1.f : 0.f;
            v.db1[k] = hot_dir(HOT, k) == 3 ? 1.f : 0.f;
            v.dm0[k] = v.deff[k] = 0.f;
            continue;
        }
        v.dt1[k] = a.dir[k][0] ? a.dir[k][0][ac] : 0.f;
        v.dt2[k] = a.dir[k][1] ? a.dir[k][1][ac] : 0.f;
        // m0, b1 and the inversion efficiency carry a direction only where
        // the property itself is given (the reference's feature flags).
        v.dm0[k] = (a.m0 && a.dir[k][2]) ? a.dir[k][2][ac] : 0.f;
        v.db1[k] = (a.b1 && a.dir[k][3]) ? a.dir[k][3][ac] : 0.f;
        v.deff[k] = (a.inv && a.dir[k][4]) ? a.dir[k][4][ac] : 0.f;
    }
    return v;
}

// Relaxation of x and the tangents over one op: t_k <- E (t_k + eps_k (x -
// e0)), x <- E x + (1 - E1) e0, e0 the recovery target (Z at order 0, held
// by lane 0's first slot).
template <int RP, int K, int HOT>
__device__ __forceinline__ void relax_all(float2 (&P)[K + 1][RP], float2 (&M)[K + 1][RP],
                                          float2 (&Z)[K + 1][RP], float e1, float e2,
                                          const float (&eps1)[K], const float (&eps2)[K], int q) {
    const float2 E1 = dup(e1), E2 = dup(e2);
    const float z0 = Z[0][0].x - (q == 0 ? 1.f : 0.f);
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const float2 a1 = dup(eps1[k]), a2 = dup(eps2[k]);
        const bool e2k = !HOT || hot_dir(HOT, k) == 2;
        const bool e1k = !HOT || hot_dir(HOT, k) == 1;
#pragma unroll
        for (int kk = 0; kk < RP; ++kk) {
            if (e2k) {
                P[k + 1][kk] = mul2(E2, fma2(a2, P[0][kk], P[k + 1][kk]));
                M[k + 1][kk] = mul2(E2, fma2(a2, M[0][kk], M[k + 1][kk]));
            } else {
                P[k + 1][kk] = mul2(E2, P[k + 1][kk]);
                M[k + 1][kk] = mul2(E2, M[k + 1][kk]);
            }
            if (e1k) {
                float2 zx = Z[0][kk];
                if (kk == 0) zx.x = z0;
                Z[k + 1][kk] = mul2(E1, fma2(a1, zx, Z[k + 1][kk]));
            } else {
                Z[k + 1][kk] = mul2(E1, Z[k + 1][kk]);
            }
        }
    }
#pragma unroll
    for (int kk = 0; kk < RP; ++kk) {
        P[0][kk] = mul2(P[0][kk], E2);
        M[0][kk] = mul2(M[0][kk], E2);
        Z[0][kk] = mul2(Z[0][kk], E1);
    }
    if (q == 0) Z[0][0].x += 1.f - e1;
}

template <int RP, int L, int K>
__device__ __forceinline__ void shift_all(float2 (&P)[K + 1][RP], float2 (&M)[K + 1][RP], int q,
                                          bool kill, int kill_r) {
#pragma unroll
    for (int s = 0; s <= K; ++s) shift_fwd<RP, L>(P[s], M[s], q, kill, kill_r);
}

template <int RP, int L, int K>
__device__ __forceinline__ void shift_adjoint_all(float2 (&P)[K + 1][RP], float2 (&M)[K + 1][RP],
                                                  int q, bool kill, int kill_r) {
#pragma unroll
    for (int s = 0; s <= K; ++s) shift_adjoint<RP, L>(P[s], M[s], q, kill, kill_r);
}

template <int RP, int K>
__device__ __forceinline__ void spoil_all(float2 (&P)[K + 1][RP], float2 (&M)[K + 1][RP]) {
#pragma unroll
    for (int s = 0; s <= K; ++s)
#pragma unroll
        for (int kk = 0; kk < RP; ++kk) P[s][kk] = M[s][kk] = dup(0.f);
}

// One op's per-direction scalars: eps1_k, eps2_k (relaxation) and a'_k
// (rotation); ddt_k and dflip_k from the op's directions.
template <int K, int HOT>
__device__ __forceinline__ void op_directions(const SecondArgs& a, const float2* dirs, int64_t n,
                                              int o, const Op& op, const Voxel<K>& v,
                                              float (&ddt)[K], float (&eps1)[K], float (&eps2)[K],
                                              float (&dal)[K], float (&dfl)[K]) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
        if (HOT) {
            ddt[k] = dfl[k] = 0.f;
            eps1[k] = hot_dir(HOT, k) == 1 ? v.w1 * op.dt : 0.f;
            eps2[k] = hot_dir(HOT, k) == 2 ? v.w2 * op.dt : 0.f;
            dal[k] = hot_dir(HOT, k) == 3 ? op.flip : 0.f;
            continue;
        }
        const float2 d = dirs ? dirs[k * n + o] : make_float2(0.f, 0.f);
        ddt[k] = d.x;
        dfl[k] = d.y;
        eps1[k] = v.w1 * v.dt1[k] * op.dt - v.r1 * d.x;
        eps2[k] = v.w2 * v.dt2[k] * op.dt - v.r2 * d.x;
        dal[k] = d.y * v.b1 + op.flip * v.db1[k];
    }
}

}  // namespace second_detail

using namespace second_detail;

// ---- forward: x and K tangents, storing the trajectory ---------------------

// Static shared memory: a chunk of ops and of each direction's per-op
// (d dt, d flip).
template <int RP, int L, int K, int HOT>
__global__ void __launch_bounds__(128) second_forward_kernel(const SecondArgs a) {
    constexpr int R = 2 * RP;
    constexpr int VPW = 32 / L;
    constexpr int NS = K + 1;
    __shared__ Op s_ops[kOpChunk];
    __shared__ float2 s_dir[K][kOpChunk];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int q = lane % L;
    const int slot = lane / L;
    const int64_t atom = (int64_t(blockIdx.x) * (blockDim.x >> 5) + warp) * VPW + slot;
    const int64_t train = blockIdx.y;
    const bool active = slot < VPW && atom < a.atoms;
    const int64_t ac = active ? atom : 0;
    const int S = a.states;
    const bool kill = L * R > S;
    const int kill_r = S - q * R;
    const Voxel<K> v = load_voxel<K, HOT>(a, ac);

    float2 P[NS][RP], M[NS][RP], Z[NS][RP];
#pragma unroll
    for (int s = 0; s < NS; ++s)
#pragma unroll
        for (int kk = 0; kk < RP; ++kk) P[s][kk] = M[s][kk] = Z[s][kk] = dup(0.f);
    if (q == 0) Z[0][0].x = 1.f;

    const Op* ops = a.ops + train * a.n_ops;
    const int64_t n_all = int64_t(gridDim.y) * a.n_ops;  // ops of all trains, per direction
    const float2* dirs = a.op_dir ? a.op_dir + train * a.n_ops : nullptr;
    const int64_t row = train * a.atoms + atom;
    // This warp's tile; lanes of a warp past the last voxel store nothing.
    const int64_t n_warps = (a.atoms + VPW - 1) / VPW;
    const int64_t warp_global = int64_t(blockIdx.x) * (blockDim.x >> 5) + warp;
    const int64_t op_stride = int64_t(NS) * 3 * 32 * RP;
    float2* lane_traj = (a.traj && warp_global < n_warps)
                            ? a.traj + (train * n_warps + warp_global) * a.n_ops * op_stride +
                                  lane * RP
                            : nullptr;
    const bool lane0 = active && q == 0;
    // Distributed records: with 2K + 3 lanes per voxel or more, lane q of
    // the voxel writes one output of a record from a pointer set up once
    // (q = 0 the signal, 1..K the derivative columns, K + 1 the M0 column,
    // K + 2 + s state s's recorded F+[0] for the reverse), the values coming
    // from lane 0 by shuffle: one store instruction per record instead of up
    // to 2K + 3 serial ones in lane 0.
    constexpr bool DIST = L >= 2 * K + 3;
    float* row_a = nullptr;    // this lane's output row: plane a, or the complex row
    float* row_b = nullptr;    // plane b of the planes layout
    float* rec_row = nullptr;  // this lane's recorded-F+[0] row of the trajectory
    if constexpr (DIST) {
        if (active) {
            float* ba = nullptr;
            float* bb = nullptr;
            int64_t off = 0;
            const int jc = K + a.with_m0;
            if (q == 0) {
                if (a.sig_a != nullptr || a.sig_b != nullptr) {
                    ba = a.sig_a;
                    bb = a.sig_b;
                    off = row * a.outputs;
                }
            } else if (q <= K || (q == K + 1 && a.with_m0)) {
                if (a.jac_a != nullptr || a.jac_b != nullptr) {
                    ba = a.jac_a;
                    bb = a.jac_b;
                    off = (row * jc + (q - 1)) * a.outputs;
                }
            } else if (q >= K + 2 && q < K + 2 + NS && a.traj_rec != nullptr) {
                rec_row = a.traj_rec + (train * a.outputs * NS + (q - K - 2)) * a.atoms + atom;
            }
            if (a.layout == TSG_LAYOUT_PLANES) {
                row_a = ba ? ba + off : nullptr;
                row_b = bb ? bb + off : nullptr;
            } else if (ba) {
                row_a = reinterpret_cast<float*>(reinterpret_cast<float2*>(ba) + off);
            }
        }
    }

    for (int base = 0; base < a.n_ops; base += kOpChunk) {
        const int count = min(kOpChunk, a.n_ops - base);
        __syncthreads();
        for (int i = threadIdx.x; i < count; i += blockDim.x) {
            s_ops[i] = ops[base + i];
#pragma unroll
            for (int k = 0; k < K; ++k)
                s_dir[k][i] = dirs ? dirs[k * n_all + base + i] : make_float2(0.f, 0.f);
        }
        __syncthreads();
        for (int i = 0; i < count; ++i) {
            const Op op = s_ops[i];
            const uint32_t code = op.code;
            if (lane_traj) {
                float2* dst = lane_traj + int64_t(base + i) * op_stride;
#pragma unroll
                for (int s = 0; s < NS; ++s)
#pragma unroll
                    for (int kk = 0; kk < RP; ++kk) {
                        dst[(s * 3 + 0) * 32 * RP + kk] = P[s][kk];
                        dst[(s * 3 + 1) * 32 * RP + kk] = M[s][kk];
                        dst[(s * 3 + 2) * 32 * RP + kk] = Z[s][kk];
                    }
            }
            float ddt[K], eps1[K], eps2[K], dal[K], dfl[K];
            op_directions<K, HOT>(a, HOT ? nullptr : &s_dir[0][0], kOpChunk, i, op, v, ddt, eps1,
                                  eps2, dal, dfl);
            if (code & OP_RELAX)
                relax_all<RP, K, HOT>(P, M, Z, expf(-v.r1 * op.dt), expf(-v.r2 * op.dt), eps1,
                                      eps2, q);
            for (int s = 0; s < op_shift1(code); ++s) shift_all<RP, L, K>(P, M, q, kill, kill_r);
            const int rf = op_rf(code);
            if (rf == RF_ROTATE) {
                float si, co;
                sincosf(op.flip * v.b1, &si, &co);
                const float2 ch = dup(0.5f * (1.f + co)), sh = dup(0.5f * (1.f - co));
                const float2 hs = dup(0.5f * si), nhs = dup(-0.5f * si), hc = dup(0.5f * co);
                const float2 si2 = dup(si), nsi2 = dup(-si), co2 = dup(co);
                const float2 neg1 = dup(-1.f);
#pragma unroll
                for (int kk = 0; kk < RP; ++kk) {
                    const float2 p = P[0][kk], m = M[0][kk], z = Z[0][kk];
                    const float2 w = fma2(neg1, m, p);
                    // R'x: (-hs w - co z, hs w + co z, hc w - si z).
                    const float2 dM = fma2(hs, w, mul2(co2, z));
                    const float2 dZ = fma2(hc, w, mul2(nsi2, z));
#pragma unroll
                    for (int k = 0; k < K; ++k) {
                        const float2 tp = P[k + 1][kk], tm = M[k + 1][kk], tz = Z[k + 1][kk];
                        if (!HOT || hot_dir(HOT, k) == 3) {
                            const float2 al = dup(dal[k]);
                            const float2 aM = mul2(al, dM);
                            P[k + 1][kk] = fma2(ch, tp, fma2(sh, tm, fma2(nsi2, tz, mul2(neg1, aM))));
                            M[k + 1][kk] = fma2(sh, tp, fma2(ch, tm, fma2(si2, tz, aM)));
                            Z[k + 1][kk] = fma2(hs, tp, fma2(nhs, tm, fma2(co2, tz, mul2(al, dZ))));
                        } else {
                            P[k + 1][kk] = fma2(ch, tp, fma2(sh, tm, mul2(nsi2, tz)));
                            M[k + 1][kk] = fma2(sh, tp, fma2(ch, tm, mul2(si2, tz)));
                            Z[k + 1][kk] = fma2(hs, tp, fma2(nhs, tm, mul2(co2, tz)));
                        }
                    }
                    P[0][kk] = fma2(ch, p, fma2(sh, m, mul2(nsi2, z)));
                    M[0][kk] = fma2(sh, p, fma2(ch, m, mul2(si2, z)));
                    Z[0][kk] = fma2(hs, w, mul2(co2, z));
                }
            } else if (rf == RF_INVERT) {
                const float2 f = dup(-v.eff);
#pragma unroll
                for (int kk = 0; kk < RP; ++kk) {
#pragma unroll
                    for (int k = 0; k < K; ++k)
                        Z[k + 1][kk] = HOT ? mul2(f, Z[k + 1][kk])
                                           : fma2(f, Z[k + 1][kk], mul2(dup(-v.deff[k]), Z[0][kk]));
                    Z[0][kk] = mul2(Z[0][kk], f);
                }
            }
            for (int s = 0; s < op_shift2(code); ++s) shift_all<RP, L, K>(P, M, q, kill, kill_r);
            if (code & OP_SPOIL1) spoil_all<RP, K>(P, M);
            if (DIST && (code & OP_RECORD)) {
                const int64_t rec = op.record;
                const int first = lane - q;
                const float p0 = __shfl_sync(0xffffffffu, P[0][0].x, first);
                float val = v.m0 * p0;  // q = 0: the signal
                float raw = p0;         // q = K + 2: state 0's recorded F+[0]
#pragma unroll
                for (int k = 0; k < K; ++k) {
                    const float d = __shfl_sync(0xffffffffu, P[k + 1][0].x, first);
                    if (q == k + 1) val = HOT ? v.m0 * d : fmaf(v.m0, d, v.dm0[k] * p0);
                    if (q == K + 3 + k) raw = d;
                }
                if (q == K + 1) val = p0;  // the M0 column
                if (a.layout == TSG_LAYOUT_PLANES) {
                    if (row_b != nullptr) {
                        if (row_a != nullptr) row_a[rec] = 0.f;
                        row_b[rec] = val;
                    }
                } else if (row_a != nullptr) {
                    reinterpret_cast<float2*>(row_a)[rec] = a.layout == TSG_LAYOUT_COMPLEX
                                                                ? make_float2(0.f, val)
                                                                : make_float2(-val, 0.f);
                }
                if (rec_row != nullptr) rec_row[rec * NS * a.atoms] = raw;
            } else if ((code & OP_RECORD) && lane0) {
                const int64_t rec = op.record;
                const float p0 = P[0][0].x;
                if (a.sig_a != nullptr || a.sig_b != nullptr)
                    store_sample(a.layout, a.sig_a, a.sig_b, row * a.outputs + rec, v.m0 * p0);
                if (a.jac_a != nullptr || a.jac_b != nullptr) {
                    const int jc = K + a.with_m0;
#pragma unroll
                    for (int k = 0; k < K; ++k)
                        store_sample(a.layout, a.jac_a, a.jac_b, (row * jc + k) * a.outputs + rec,
                                     HOT ? v.m0 * P[k + 1][0].x
                                         : fmaf(v.m0, P[k + 1][0].x, v.dm0[k] * p0));
                    if (a.with_m0)
                        store_sample(a.layout, a.jac_a, a.jac_b, (row * jc + K) * a.outputs + rec, p0);
                }
                if (a.traj_rec) {
                    float* dst = a.traj_rec + ((train * a.outputs + rec) * NS) * a.atoms + atom;
#pragma unroll
                    for (int s = 0; s < NS; ++s) dst[s * a.atoms] = P[s][0].x;
                }
            }
            for (int s = 0; s < op_shift3(code); ++s) shift_all<RP, L, K>(P, M, q, kill, kill_r);
            if (code & OP_SPOIL2) spoil_all<RP, K>(P, M);
        }
    }
}

// ---- reverse ---------------------------------------------------------------

// Dynamic shared memory: transcendentals [D][T] float4, entry states
// [D][NS][3][RP][T] float2, (seed, recorded F+[0]) [D][NS][T] float2, the
// M0 derivative's seed [D][T] float, ops [n_ops], per-direction op
// directions [K][n_ops] float2 (only with event directions).
template <int RP, int L, int K, int HOT>
__global__ void __launch_bounds__(32 * kSecondWarps) second_reverse_kernel(const SecondArgs a) {
    extern __shared__ __align__(16) unsigned char s_raw[];
    constexpr int W = kSecondWarps;
    constexpr int T = 32 * W;
    constexpr int R = 2 * RP;
    constexpr int VPW = 32 / L;
    constexpr int NS = K + 1;
    constexpr int D = kSecondRing;
    constexpr int NE2 = (K == 1 && !HOT) ? 2 : 1;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int q = lane % L;
    const int slot = lane / L;
    const int64_t warp_global = int64_t(blockIdx.x) * W + warp;
    const int64_t atom = warp_global * VPW + slot;
    const int64_t train = blockIdx.y;
    const bool active = slot < VPW && atom < a.atoms;
    const int64_t ac = active ? atom : 0;
    const int S = a.states;
    const int n_ops = a.n_ops;
    const bool kill = L * R > S;
    const int kill_r = S - q * R;
    const bool lane0 = active && q == 0;
    const int64_t n = a.atoms;
    const int64_t row = train * n + atom;
    const int vslot = warp * VPW + (slot < VPW ? slot : VPW - 1);

    // Per voxel slot (not per lane): the transcendentals, seeds and
    // recorded F+[0] one lane of the voxel fetches.
    constexpr int VPB = W * VPW;
    constexpr int VPB4 = (VPB + 3) & ~3;
    float2* s_ring = reinterpret_cast<float2*>(s_raw);                    // [D][NS*3][T][RP]
    float4* s_tring = reinterpret_cast<float4*>(s_ring + D * NS * 3 * RP * T);  // [L][VPB]
    float2* s_sring = reinterpret_cast<float2*>(s_tring + L * VPB);       // [D][NS][VPB]
    float* s_mring = reinterpret_cast<float*>(s_sring + D * NS * VPB);    // [D][VPB4]
    Op* s_ops = reinterpret_cast<Op*>(s_mring + D * VPB4);                 // [n_ops]
    float2* s_dir = reinterpret_cast<float2*>(s_ops + n_ops);              // [K][n_ops]

    const Voxel<K> v = load_voxel<K, HOT>(a, ac);
    {
        const Op* ops = a.ops + train * n_ops;
        for (int i = threadIdx.x; i < n_ops; i += T) s_ops[i] = ops[i];
        if (!HOT && a.op_dir) {
            const int64_t n_all = int64_t(gridDim.y) * n_ops;
            for (int i = threadIdx.x; i < K * n_ops; i += T) {
                const int k = i / n_ops, o = i - k * n_ops;
                s_dir[i] = a.op_dir[k * n_all + train * n_ops + o];
            }
        }
        __syncthreads();
    }

    // Cotangents: lam (state 0) and mu_k (state k + 1).
    float2 pb[NS][RP], mb[NS][RP], zb[NS][RP];
#pragma unroll
    for (int s = 0; s < NS; ++s)
#pragma unroll
        for (int kk = 0; kk < RP; ++kk) pb[s][kk] = mb[s][kk] = zb[s][kk] = dup(0.f);

    // Accumulated per lane: dL/dr1, dL/dr2, dL/dr1'_k, dL/dr2'_k; the
    // curvature of m0, b1, inversion; the values of m0, b1, inversion.
    float g_r1 = 0.f, g_r2 = 0.f, c_m0 = 0.f, c_b1 = 0.f, c_inv = 0.f;
    float g_rd1[K], g_rd2[K], v_m0[K], v_b1[K], v_inv[K];
#pragma unroll
    for (int k = 0; k < K; ++k) g_rd1[k] = g_rd2[k] = v_m0[k] = v_b1[k] = v_inv[k] = 0.f;

    const bool planes = a.seed_layout == TSG_LAYOUT_PLANES;
    const int seed_stride = planes ? 1 : 2;
    const float seed_sign = planes ? 1.f : -1.f;
    const float* seed0_row = a.seed0 ? a.seed0 + (active ? row : 0) * a.outputs * seed_stride
                                     : nullptr;
    const int jc = K + a.with_m0;
    const float* seed_row = a.seed + (active ? row : 0) * jc * a.outputs * seed_stride;
    const float* rec_col = a.traj_rec + train * a.outputs * NS * n + ac;

    // This warp's tile (a warp past the last voxel reads tile 0 and keeps
    // nothing of it).
    const int64_t n_warps = (n + VPW - 1) / VPW;
    const int64_t op_stride = int64_t(NS) * 3 * 32 * RP;
    const float2* lane_traj =
        a.traj + (train * n_warps + (warp_global < n_warps ? warp_global : 0)) * n_ops * op_stride +
        lane * RP;
    const unsigned ring_base =
        static_cast<unsigned>(__cvta_generic_to_shared(s_ring + threadIdx.x * RP));
    const unsigned sring_base = static_cast<unsigned>(__cvta_generic_to_shared(s_sring + vslot));
    const unsigned mring_base = static_cast<unsigned>(__cvta_generic_to_shared(s_mring + vslot));

    // Op o into ring slot rs: entry-state pairs of every state (zero past the
    // last pair), the seeds and recorded F+[0] (zero unless this lane
    // records), and the transcendentals.
    auto fetch = [&](int o, int rs) {
        const float2* src_op = lane_traj + o * op_stride;
        const unsigned dst_op = ring_base + unsigned(rs * NS * 3 * RP * T) * 8u;
#pragma unroll
        for (int sp = 0; sp < NS * 3; ++sp) {
            const float2* src = src_op + sp * 32 * RP;
            const unsigned dst = dst_op + unsigned(sp * T * RP) * 8u;
            if constexpr (RP == 2) {
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src)
                             : "memory");
            } else {
#pragma unroll
                for (int kk = 0; kk < RP; ++kk)
                    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(dst + 8u * kk),
                                 "l"(src + kk)
                                 : "memory");
            }
        }
        const Op op = s_ops[o];
        // Seeds and recorded F+[0]: lane 0 of each voxel slot copies them
        // (zeros unless the voxel is live and the op records).
        if (q == 0 && slot < VPW) {
            const bool rec = lane0 && (op.code & OP_RECORD);
            const int64_t r = rec ? op.record : 0;
            const unsigned sdst = sring_base + unsigned(rs * NS * VPB) * 8u;
            const bool have0 = rec && seed0_row != nullptr;
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(sdst),
                         "l"(have0 ? seed0_row + r * seed_stride : a.seed), "r"(have0 ? 4 : 0)
                         : "memory");
#pragma unroll
            for (int k = 0; k < K; ++k)
                asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(
                                 sdst + unsigned((k + 1) * VPB) * 8u),
                             "l"(seed_row + (k * a.outputs + r) * seed_stride), "r"(rec ? 4 : 0)
                             : "memory");
#pragma unroll
            for (int s = 0; s < NS; ++s)
                asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(
                                 sdst + unsigned(s * VPB) * 8u + 4u),
                             "l"(rec_col + (r * NS + s) * n), "r"(rec ? 4 : 0)
                             : "memory");
            const bool have_m = rec && a.with_m0;
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(
                             mring_base + unsigned(rs * VPB4) * 4u),
                         "l"(have_m ? seed_row + (K * a.outputs + r) * seed_stride : a.seed),
                         "r"(have_m ? 4 : 0)
                         : "memory");
        }
    };

#pragma unroll
    for (int j = 1; j < D; ++j) {
        if (n_ops - j >= 0) fetch(n_ops - j, j - 1);
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    }
    float2* event_out =
        a.event_partial + (train * a.warps_per_train + warp_global) * int64_t(n_ops) * NE2;
    const float2* dirs = a.op_dir ? s_dir : nullptr;
    int use_slot = 0, fill_slot = D - 1;
    const float2 neg1 = dup(-1.f);

    for (int o = n_ops - 1; o >= 0; --o) {
        if ((n_ops - 1 - o) % L == 0) {
            // Every L ops, the transcendentals of the next L: lane q of a
            // voxel evaluates op o - q, so one pass of the warp covers them
            // (slot (op % L) of each voxel; the slots' last readers are done).
            __syncwarp();
            const int oq = o - q;
            if (slot < VPW && oq >= 0) {
                const Op opq = s_ops[oq];
                float si = 0.f, co = 1.f;
                if (op_rf(opq.code) == RF_ROTATE) sincosf(opq.flip * v.b1, &si, &co);
                s_tring[(oq % L) * VPB + vslot] =
                    make_float4(si, co, expf(-v.r1 * opq.dt), expf(-v.r2 * opq.dt));
            }
        }
        // Orders the lanes' reads of the slot this fetch refills (used last
        // iteration) and the transcendentals written above.
        __syncwarp();
        if (o - (D - 1) >= 0) fetch(o - (D - 1), fill_slot);
        asm volatile("cp.async.commit_group;\n" ::: "memory");
        fill_slot = fill_slot + 1 == D ? 0 : fill_slot + 1;
        const Op op = s_ops[o];
        const uint32_t code = op.code;
        asm volatile("cp.async.wait_group %0;\n" ::"n"(D - 1) : "memory");
        const int cur = use_slot;
        use_slot = use_slot + 1 == D ? 0 : use_slot + 1;
        const float4 tr = s_tring[(o % L) * VPB + vslot];
        const float2* ring = s_ring + cur * (NS * 3 * RP * T) + threadIdx.x * RP;
        const float2* sr = s_sring + cur * (NS * VPB) + vslot;

        // The pre-RF states: entry states relaxed and pre-shifted.
        float2 P[NS][RP], M[NS][RP], Z[NS][RP];
#pragma unroll
        for (int s = 0; s < NS; ++s)
#pragma unroll
            for (int kk = 0; kk < RP; ++kk) {
                P[s][kk] = ring[(s * 3 + 0) * T * RP + kk];
                M[s][kk] = ring[(s * 3 + 1) * T * RP + kk];
                Z[s][kk] = ring[(s * 3 + 2) * T * RP + kk];
            }
        float ddt[K], eps1[K], eps2[K], dal[K], dfl[K];
        op_directions<K, HOT>(a, dirs, n_ops, o, op, v, ddt, eps1, eps2, dal, dfl);
        const bool relax = (code & OP_RELAX) != 0;
        if (relax) relax_all<RP, K, HOT>(P, M, Z, tr.z, tr.w, eps1, eps2, q);
        for (int s = 0; s < op_shift1(code); ++s) shift_all<RP, L, K>(P, M, q, kill, kill_r);

        // Reverse of the op's micro-steps after the pulse.
        if (code & OP_SPOIL2) spoil_all<RP, K>(pb, mb);
        for (int s = 0; s < op_shift3(code); ++s) shift_adjoint_all<RP, L, K>(pb, mb, q, kill, kill_r);
        if ((code & OP_RECORD) && lane0) {
            const float g0 = seed_sign * sr[0].x;
            const float x0 = sr[0].y;
            // The M0 derivative is F+[0] itself: its seed acts unscaled.
            const float g_m0col = s_mring[cur * VPB4 + vslot];
            float add0 = fmaf(g0, v.m0, seed_sign * g_m0col);
            c_m0 = fmaf(g0, x0, c_m0);
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const float gk = seed_sign * sr[(k + 1) * VPB].x;
                const float tk0 = sr[(k + 1) * VPB].y;
                if (!HOT) add0 = fmaf(gk, v.dm0[k], add0);
                pb[k + 1][0].x = fmaf(gk, v.m0, pb[k + 1][0].x);
                c_m0 = fmaf(gk, tk0, c_m0);
                if (!HOT) v_m0[k] = fmaf(gk, x0, v_m0[k]);
            }
            pb[0][0].x += add0;
        }
        if (code & OP_SPOIL1) spoil_all<RP, K>(pb, mb);
        for (int s = 0; s < op_shift2(code); ++s) shift_adjoint_all<RP, L, K>(pb, mb, q, kill, kill_r);

        float e_flip = 0.f, e_dt = 0.f;  // this lane's curvature of the op
        float ev_flip = 0.f, ev_dt = 0.f;  // value (K == 1)
        const int rf = op_rf(code);
        if (rf == RF_ROTATE) {
            const float si = tr.x, co = tr.y;
            const float2 ch = dup(0.5f * (1.f + co)), sh = dup(0.5f * (1.f - co));
            const float2 hs = dup(0.5f * si), nhs = dup(-0.5f * si), hc = dup(0.5f * co);
            const float2 si2 = dup(si), nsi2 = dup(-si), co2 = dup(co), nco2 = dup(-co);
            float2 ga = dup(0.f);  // dL/da, this lane's part
            float2 gk[K];          // G_k
#pragma unroll
            for (int k = 0; k < K; ++k) gk[k] = dup(0.f);
#pragma unroll
            for (int kk = 0; kk < RP; ++kk) {
                const float2 w = fma2(neg1, M[0][kk], P[0][kk]);
                const float2 z = Z[0][kk];
                // R'x as (a, b): rows P, M, Z are (-a, a, b); R''x as (c, e)
                // with rows (-c, c, e).
                const float2 ax = fma2(hs, w, mul2(co2, z));
                const float2 bx = fma2(hc, w, mul2(nsi2, z));
                const float2 ex = fma2(nhs, w, mul2(nco2, z));
                const float2 dl = fma2(neg1, pb[0][kk], mb[0][kk]);
                ga = fma2(dl, ax, fma2(zb[0][kk], bx, ga));
                float2 U = dup(0.f), V = dup(0.f);
#pragma unroll
                for (int k = 0; k < K; ++k) {
                    const float2 d = fma2(neg1, pb[k + 1][kk], mb[k + 1][kk]);
                    const float2 zbk = zb[k + 1][kk];
                    const float2 wt = fma2(neg1, M[k + 1][kk], P[k + 1][kk]);
                    const float2 zt = Z[k + 1][kk];
                    const float2 at = fma2(hs, wt, mul2(co2, zt));
                    const float2 bt = fma2(hc, wt, mul2(nsi2, zt));
                    // G_k = d.ax + zb.bx; H_k = d.at + zb.bt;
                    // I_k = d.(hc w - si z) + zb.(-hs w - co z) = d.bx + zb.ex.
                    gk[k] = fma2(d, ax, fma2(zbk, bx, gk[k]));
                    ga = fma2(d, at, fma2(zbk, bt, ga));
                    if (!HOT || hot_dir(HOT, k) == 3) {
                        const float2 al = dup(dal[k]);
                        ga = fma2(al, fma2(d, bx, mul2(zbk, ex)), ga);
                        // (R'^T mu_k): P (hs d + hc zb), M -(..), Z (co d - si zb).
                        U = fma2(al, fma2(hs, d, mul2(hc, zbk)), U);
                        V = fma2(al, fma2(co2, d, mul2(nsi2, zbk)), V);
                    }
                    // mu_k <- R^T mu_k.
                    const float2 p_ = pb[k + 1][kk], m_ = mb[k + 1][kk];
                    pb[k + 1][kk] = fma2(ch, p_, fma2(sh, m_, mul2(hs, zbk)));
                    mb[k + 1][kk] = fma2(sh, p_, fma2(ch, m_, mul2(nhs, zbk)));
                    zb[k + 1][kk] = fma2(si2, d, mul2(co2, zbk));
                }
                const float2 p_ = pb[0][kk], m_ = mb[0][kk], z_ = zb[0][kk];
                pb[0][kk] = fma2(ch, p_, fma2(sh, m_, fma2(hs, z_, U)));
                mb[0][kk] = fma2(sh, p_, fma2(ch, m_, fma2(nhs, z_, mul2(neg1, U))));
                zb[0][kk] = fma2(si2, dl, fma2(co2, z_, V));
            }
            const float gsum = ga.x + ga.y;
            float gf = gsum * v.b1, gb = gsum * op.flip;
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const float g = gk[k].x + gk[k].y;
                if (HOT) {
                    if (hot_dir(HOT, k) == 3) gf += g;
                    continue;
                }
                gf = fmaf(g, v.db1[k], gf);
                gb = fmaf(g, dfl[k], gb);
                v_b1[k] = fmaf(g, op.flip, v_b1[k]);
                if (K == 1) ev_flip = g * v.b1;
            }
            e_flip = gf;
            c_b1 += gb;
        } else if (rf == RF_INVERT) {
            const float2 f = dup(-v.eff);
            float2 acc = dup(0.f);
            float2 vk[K];
#pragma unroll
            for (int k = 0; k < K; ++k) vk[k] = dup(0.f);
#pragma unroll
            for (int kk = 0; kk < RP; ++kk) {
                acc = fma2(zb[0][kk], Z[0][kk], acc);
                float2 nz = mul2(zb[0][kk], f);
#pragma unroll
                for (int k = 0; k < K; ++k) {
                    const float2 zbk = zb[k + 1][kk];
                    acc = fma2(zbk, Z[k + 1][kk], acc);
                    if (!HOT) {
                        vk[k] = fma2(zbk, Z[0][kk], vk[k]);
                        nz = fma2(dup(-v.deff[k]), zbk, nz);
                    }
                    zb[k + 1][kk] = mul2(zbk, f);
                }
                zb[0][kk] = nz;
            }
            c_inv -= acc.x + acc.y;
            if (!HOT)
#pragma unroll
                for (int k = 0; k < K; ++k) v_inv[k] -= vk[k].x + vk[k].y;
        }
        if (relax) {
            // Q2, Q1 and C2_k, C1_k at the pre-RF point.
            float2 q2 = dup(0.f), q1 = dup(0.f);
            float zx0 = 0.f;  // the recovery target's part of lam.(x - e0)
#pragma unroll
            for (int kk = 0; kk < RP; ++kk) {
                q2 = fma2(pb[0][kk], P[0][kk], fma2(mb[0][kk], M[0][kk], q2));
                q1 = fma2(zb[0][kk], Z[0][kk], q1);
            }
            if (q == 0) zx0 = zb[0][0].x;
            float Q2 = q2.x + q2.y, Q1 = q1.x + q1.y - zx0;
            float dtc = 0.f;
#pragma unroll
            for (int k = 0; k < K; ++k) {
                // C2_k and C1_k: a one-hot direction needs only its own.
                const bool n2 = !HOT || hot_dir(HOT, k) == 2;
                const bool n1 = !HOT || hot_dir(HOT, k) == 1;
                float2 c2 = dup(0.f), c1 = dup(0.f), t2 = dup(0.f), t1 = dup(0.f);
#pragma unroll
                for (int kk = 0; kk < RP; ++kk) {
                    if (n2) c2 = fma2(pb[k + 1][kk], P[0][kk], fma2(mb[k + 1][kk], M[0][kk], c2));
                    if (n1) c1 = fma2(zb[k + 1][kk], Z[0][kk], c1);
                    t2 = fma2(pb[k + 1][kk], P[k + 1][kk], fma2(mb[k + 1][kk], M[k + 1][kk], t2));
                    t1 = fma2(zb[k + 1][kk], Z[k + 1][kk], t1);
                }
                Q2 += t2.x + t2.y;
                Q1 += t1.x + t1.y;
                const float C2 = n2 ? c2.x + c2.y : 0.f;
                const float C1 = n1 ? c1.x + c1.y - (q == 0 ? zb[k + 1][0].x : 0.f) : 0.f;
                if (HOT) {
                    // r'_k = -w for the unit tangent of T1 (or T2).
                    if (n2) {
                        g_rd2[k] = fmaf(-op.dt, C2, g_rd2[k]);
                        dtc = fmaf(C2, v.w2, dtc);
                    }
                    if (n1) {
                        g_rd1[k] = fmaf(-op.dt, C1, g_rd1[k]);
                        dtc = fmaf(C1, v.w1, dtc);
                    }
                    continue;
                }
                g_r2 = fmaf(-C2, ddt[k], g_r2);
                g_r1 = fmaf(-C1, ddt[k], g_r1);
                g_rd2[k] = fmaf(-op.dt, C2, g_rd2[k]);
                g_rd1[k] = fmaf(-op.dt, C1, g_rd1[k]);
                // r'_k = -w T'_k.
                dtc = fmaf(C2, v.w2 * v.dt2[k], fmaf(C1, v.w1 * v.dt1[k], dtc));
                if (K == 1) ev_dt = -v.r2 * C2 - v.r1 * C1;
            }
            g_r2 = fmaf(-op.dt, Q2, g_r2);
            g_r1 = fmaf(-op.dt, Q1, g_r1);
            e_dt = -v.r2 * Q2 - v.r1 * Q1 + dtc;
        }
        for (int s = 0; s < op_shift1(code); ++s) shift_adjoint_all<RP, L, K>(pb, mb, q, kill, kill_r);
        if (relax) {
            const float2 E1 = dup(tr.z), E2 = dup(tr.w);
#pragma unroll
            for (int kk = 0; kk < RP; ++kk) {
                float2 lp = mul2(pb[0][kk], E2), lm = mul2(mb[0][kk], E2), lz = mul2(zb[0][kk], E1);
#pragma unroll
                for (int k = 0; k < K; ++k) {
                    pb[k + 1][kk] = mul2(pb[k + 1][kk], E2);
                    mb[k + 1][kk] = mul2(mb[k + 1][kk], E2);
                    zb[k + 1][kk] = mul2(zb[k + 1][kk], E1);
                    if (!HOT || hot_dir(HOT, k) == 2) {
                        lp = fma2(dup(eps2[k]), pb[k + 1][kk], lp);
                        lm = fma2(dup(eps2[k]), mb[k + 1][kk], lm);
                    }
                    if (!HOT || hot_dir(HOT, k) == 1) lz = fma2(dup(eps1[k]), zb[k + 1][kk], lz);
                }
                pb[0][kk] = lp;
                mb[0][kk] = lm;
                zb[0][kk] = lz;
            }
        }
        // The op's event partials summed over the warp (a fixed butterfly;
        // nothing on the state recursion waits for it).
        float ev[2 * NE2] = {active ? e_flip : 0.f, active ? e_dt : 0.f};
        if constexpr (NE2 == 2) {
            ev[2] = active ? ev_flip : 0.f;
            ev[3] = active ? ev_dt : 0.f;
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1)
#pragma unroll
            for (int e = 0; e < 2 * NE2; ++e) ev[e] += __shfl_xor_sync(0xffffffffu, ev[e], off);
        if (lane == 0) {
#pragma unroll
            for (int e = 0; e < NE2; ++e)
                event_out[int64_t(o) * NE2 + e] = make_float2(ev[2 * e], ev[2 * e + 1]);
        }
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");

    // Tissue: r = 1000/T, r'_k = -1000 T'_k/T^2, summed over the voxel's lanes.
    // One-hot directions write the curvature only.
    constexpr int NV = HOT ? 5 : 5 * (1 + K);
    float out[NV];
    {
        float gt1 = -v.w1 * g_r1, gt2 = -v.w2 * g_r2;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            if (HOT) {
                if (hot_dir(HOT, k) == 1) gt1 = fmaf(g_rd1[k], 2.f * v.w1 / v.t1, gt1);
                if (hot_dir(HOT, k) == 2) gt2 = fmaf(g_rd2[k], 2.f * v.w2 / v.t2, gt2);
                continue;
            }
            gt1 = fmaf(g_rd1[k], 2.f * v.w1 * v.dt1[k] / v.t1, gt1);
            gt2 = fmaf(g_rd2[k], 2.f * v.w2 * v.dt2[k] / v.t2, gt2);
        }
        out[0] = gt1;
        out[1] = gt2;
        out[2] = c_m0;
        out[3] = c_b1;
        out[4] = c_inv;
        if constexpr (!HOT) {
#pragma unroll
            for (int k = 0; k < K; ++k) {
                out[5 + 5 * k + 0] = -v.w1 * g_rd1[k];
                out[5 + 5 * k + 1] = -v.w2 * g_rd2[k];
                out[5 + 5 * k + 2] = v_m0[k];
                out[5 + 5 * k + 3] = v_b1[k];
                out[5 + 5 * k + 4] = v_inv[k];
            }
        }
    }
#pragma unroll
    for (int j = 0; j < NV; ++j) {
        const float x = active ? out[j] : 0.f;
        float sum = 0.f;
#pragma unroll
        for (int l = 0; l < L; ++l) sum += __shfl_sync(0xffffffffu, x, lane - q + l);
        out[j] = sum;
    }
    if (lane0) {
        float* dst = a.tissue_partial + row * NV;
#pragma unroll
        for (int j = 0; j < NV; ++j) dst[j] = out[j];
    }
}

template <int RP, int L, int K, int HOT>
void launch_second_forward(const SecondArgs& a, dim3 grid, dim3 block, size_t smem,
                           cudaStream_t s) {
    second_forward_kernel<RP, L, K, HOT><<<grid, block, smem, s>>>(a);
}

template <int RP, int L, int K, int HOT>
void launch_second_reverse(const SecondArgs& a, dim3 grid, dim3 block, size_t smem,
                           cudaStream_t s) {
    second_reverse_kernel<RP, L, K, HOT><<<grid, block, smem, s>>>(a);
}

// One (orders per lane, lanes per voxel) shape for K directions, general
// (hot == 0) or one-hot (the direction code of hot_dir).
struct SecondEntry {
    int orders_per_lane;
    int lanes_per_voxel;
    int directions;
    int hot;
    void (*forward)(const SecondArgs&, dim3, dim3, size_t, cudaStream_t);
    void (*reverse)(const SecondArgs&, dim3, dim3, size_t, cudaStream_t);
    const void* reverse_fn;
};

#define TSG_SECOND_ENTRY(R, L, K, HOT)                                                  \
    {R,                                                                                 \
     L,                                                                                 \
     K,                                                                                 \
     HOT,                                                                               \
     &launch_second_forward<(R) / 2, L, K, HOT>,                                        \
     &launch_second_reverse<(R) / 2, L, K, HOT>,                                        \
     reinterpret_cast<const void*>(&second_reverse_kernel<(R) / 2, L, K, HOT>)}

// The shapes instantiated per direction set: general directions take every
// shape, one-hot sets the ones measured useful.
#define TSG_SECOND_SHAPES_HOT(K, HOT)                                                     \
    TSG_SECOND_ENTRY(2, 4, K, HOT), TSG_SECOND_ENTRY(2, 5, K, HOT),                       \
        TSG_SECOND_ENTRY(2, 8, K, HOT), TSG_SECOND_ENTRY(2, 10, K, HOT),                  \
        TSG_SECOND_ENTRY(2, 16, K, HOT), TSG_SECOND_ENTRY(2, 32, K, HOT),                 \
        TSG_SECOND_ENTRY(4, 1, K, HOT), TSG_SECOND_ENTRY(4, 2, K, HOT),                   \
        TSG_SECOND_ENTRY(4, 4, K, HOT), TSG_SECOND_ENTRY(4, 5, K, HOT),                   \
        TSG_SECOND_ENTRY(4, 8, K, HOT)

// Every table of one translation unit.
const SecondEntry* second_table(int k, int hot, int* count);

}  // namespace tsg
