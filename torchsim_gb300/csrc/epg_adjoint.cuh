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
// Per-event gradients (flip, duration): each lane parks its per-op partials
// in shared memory; at the end of a segment the warp sums them over its lanes
// (lane j takes op j) and writes one partial per warp; a second kernel adds
// the warps up. Every sum runs in a fixed order, so the result does not depend
// on scheduling (no atomics), and no shuffle chain sits between two ops.
#pragma once
#include "tsg_internal.h"

namespace tsg {

namespace adjoint_detail {

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

// The same two shifts for one lane holding a voxel's R = 2 RP orders as
// strided pairs (pair k = orders k and k + RP): whole pairs move, and only
// the wrap between the halves (order RP - 1 <-> RP) and the ends move single
// values. `kill` clears order `kill_r` (= states) as the contiguous shifts do.
template <int RP>
__device__ __forceinline__ void shift_fwd_strided(float2 (&p)[RP], float2 (&m)[RP], bool kill,
                                                  int kill_r) {
    const float m_wrap = m[0].y;  // order RP moves down to RP - 1
    const float p_wrap = p[RP - 1].x;  // order RP - 1 moves up to RP
#pragma unroll
    for (int k = 0; k + 1 < RP; ++k) m[k] = m[k + 1];
    m[RP - 1] = make_float2(m_wrap, 0.f);
#pragma unroll
    for (int k = RP - 1; k > 0; --k) p[k] = p[k - 1];
    p[0] = make_float2(-m[0].x, p_wrap);
    if (kill) {
#pragma unroll
        for (int k = 0; k < RP; ++k) {
            if (k == kill_r) p[k].x = 0.f;
            if (k + RP == kill_r) p[k].y = 0.f;
        }
    }
}

template <int RP>
__device__ __forceinline__ void shift_adjoint_strided(float2 (&pb)[RP], float2 (&mb)[RP], bool kill,
                                                      int kill_r) {
    const float carry = -pb[0].x;
    const float pb_wrap = pb[0].y;      // order RP's cotangent moves down to RP - 1
    const float mb_wrap = mb[RP - 1].x;  // order RP - 1's moves up to RP
#pragma unroll
    for (int k = 0; k + 1 < RP; ++k) pb[k] = pb[k + 1];
    pb[RP - 1] = make_float2(pb_wrap, 0.f);
#pragma unroll
    for (int k = RP - 1; k > 0; --k) mb[k] = mb[k - 1];
    mb[0] = make_float2(0.f, mb_wrap);
    if constexpr (RP > 1) mb[1].x += carry;
    if (kill) {
#pragma unroll
        for (int k = 0; k < RP; ++k) {
            if (k == kill_r) mb[k].x = 0.f;
            if (k + RP == kill_r) mb[k].y = 0.f;
        }
    }
}

}  // namespace adjoint_detail

using namespace adjoint_detail;

// Per-voxel constants of the reverse sweep and its per-voxel gradients.
struct VoxelConsts {
    float m0, b1, eff, r1, r2, w1, w2;
};
struct TissueGrads {
    float t1 = 0.f, t2 = 0.f, m0 = 0.f, b1 = 0.f, inv = 0.f;
};

// The transposed micro-steps of one op, from its last spoil back to its
// relaxation. The op's pre-RF state is (ep * p_, ep * m_, ez * z_ + r0 at
// order 0): the staged pre-RF state itself (ep = ez = 1, r0 = 0), or an entry
// state whose relaxation is folded into the coefficients (ep = e2, ez = e1,
// r0 = 1 - e1) when no shift sits between the relaxation and the pulse.
// tr = (sin, cos, e1, e2); `seed` is the cotangent of the op's sample and
// `rec` the F+[0] it recorded (both used on the voxel's lane 0 only).
// Updates the cotangent (pb, mb, zb) and the voxel gradients; returns this
// lane's (dL/dflip, dL/dduration) of the op.
template <int RP, int L, bool STRIDED = false>
__device__ __forceinline__ float2 reverse_op(const Op& op, const float4& tr, const float2 (&p_)[RP],
                                             const float2 (&m_)[RP], const float2 (&z_)[RP],
                                             float ep, float ez, float r0, float2 (&pb)[RP],
                                             float2 (&mb)[RP], float2 (&zb)[RP], float seed,
                                             float rec, bool lane0, const VoxelConsts& v,
                                             TissueGrads& g, int q, bool kill, int kill_r) {
    const uint32_t code = op.code;
    const float2 neg1 = dup(-1.f);
    auto adjoint_shift = [&](float2 (&b_p)[RP], float2 (&b_m)[RP]) {
        if constexpr (STRIDED)
            shift_adjoint_strided<RP>(b_p, b_m, kill, kill_r);
        else
            shift_adjoint<RP, L>(b_p, b_m, q, kill, kill_r);
    };
    if (code & OP_SPOIL2) {
#pragma unroll
        for (int k = 0; k < RP; ++k) pb[k] = mb[k] = dup(0.f);
    }
    for (int s = 0; s < op_shift3(code); ++s) adjoint_shift(pb, mb);
    if ((code & OP_RECORD) && lane0) {
        pb[0].x = fmaf(seed, v.m0, pb[0].x);
        g.m0 = fmaf(seed, rec, g.m0);
    }
    if (code & OP_SPOIL1) {
#pragma unroll
        for (int k = 0; k < RP; ++k) pb[k] = mb[k] = dup(0.f);
    }
    for (int s = 0; s < op_shift2(code); ++s) adjoint_shift(pb, mb);
    const int rf = op_rf(code);
    // The recovery term r0 sits in z at order 0 (lane 0's first slot).
    const float r0q = q == 0 ? r0 : 0.f;
    float g_flip = 0.f;
    if (rf == RF_ROTATE) {
        const float si = tr.x, co = tr.y;
        const float2 ch = dup(0.5f * (1.f + co)), sh = dup(0.5f * (1.f - co));
        const float2 hs = dup(0.5f * si), nhs = dup(-0.5f * si);
        const float2 si2 = dup(si), co2 = dup(co);
        // d/dalpha terms on the pre-RF state, with its scale folded in.
        const float2 hs_w = dup(0.5f * si * ep), co_z = dup(co * ez);
        const float2 hc_w = dup(0.5f * co * ep), nsi_z = dup(-si * ez);
        float2 ga0 = dup(0.f), ga1 = dup(0.f);
        // Order 0's recovery: d0 * co * r0 - zb0 * si * r0.
        const float fix = r0q * (co * (mb[0].x - pb[0].x) - si * zb[0].x);
#pragma unroll
        for (int k = 0; k < RP; ++k) {
            const float2 w = fma2(neg1, m_[k], p_[k]);
            const float2 d = fma2(neg1, pb[k], mb[k]);
            ga0 = fma2(d, fma2(hs_w, w, mul2(co_z, z_[k])), ga0);
            ga1 = fma2(zb[k], fma2(hc_w, w, mul2(nsi_z, z_[k])), ga1);
            const float2 npb = fma2(ch, pb[k], fma2(sh, mb[k], mul2(hs, zb[k])));
            const float2 nmb = fma2(sh, pb[k], fma2(ch, mb[k], mul2(nhs, zb[k])));
            zb[k] = fma2(si2, d, mul2(co2, zb[k]));
            pb[k] = npb;
            mb[k] = nmb;
        }
        const float gsum = (ga0.x + ga1.x) + (ga0.y + ga1.y) + fix;
        g_flip = gsum * v.b1;
        g.b1 = fmaf(gsum, op.flip, g.b1);
    } else if (rf == RF_INVERT) {
        float2 acc = dup(0.f);
        const float zb0 = zb[0].x;
#pragma unroll
        for (int k = 0; k < RP; ++k) {
            acc = fma2(zb[k], z_[k], acc);
            zb[k] = mul2(zb[k], dup(-v.eff));
        }
        g.inv -= ez * (acc.x + acc.y) + r0q * zb0;
    }
    float g_dt = 0.f;
    if (code & OP_RELAX) {
        float2 A2a = dup(0.f), A2b = dup(0.f), A1 = dup(0.f);
#pragma unroll
        for (int k = 0; k < RP; ++k) {
            A2a = fma2(pb[k], p_[k], A2a);
            A2b = fma2(mb[k], m_[k], A2b);
            A1 = fma2(zb[k], z_[k], A1);
        }
        const float a2 = ep * ((A2a.x + A2b.x) + (A2a.y + A2b.y));
        float a1 = ez * (A1.x + A1.y);
        if (q == 0) a1 += (r0 - 1.f) * zb[0].x;
        g.t2 = fmaf(a2, op.dt * v.w2, g.t2);
        g.t1 = fmaf(a1, op.dt * v.w1, g.t1);
        g_dt = -v.r2 * a2 - v.r1 * a1;
    }
    for (int s = 0; s < op_shift1(code); ++s) adjoint_shift(pb, mb);
    if (code & OP_RELAX) {
        const float2 E1 = dup(tr.z), E2 = dup(tr.w);
#pragma unroll
        for (int k = 0; k < RP; ++k) {
            pb[k] = mul2(pb[k], E2);
            mb[k] = mul2(mb[k], E2);
            zb[k] = mul2(zb[k], E1);
        }
    }
    return make_float2(g_flip, g_dt);
}

// The transcendentals of ops [0, cnt) of the staged chunk for this voxel:
// lane q of the voxel evaluates every L-th op.
template <int L, int VPW, int VPB>
__device__ __forceinline__ void stage_transcendentals(const Op* s_ops, float4* s_tr, int cnt, int q,
                                                      int slot, int vslot, float b1, float r1,
                                                      float r2) {
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
}

// Sums the lanes' event partials of ops [0, cnt) over the warp (lane j takes
// op j; fixed order) and writes them as the warp's partials.
__device__ __forceinline__ void reduce_chunk_events(const float2* warp_ev, int row_len, int cnt,
                                                    int lane, float2* out) {
    for (int i = lane; i < cnt; i += 32) {
        float2 acc[4] = {dup(0.f), dup(0.f), dup(0.f), dup(0.f)};
#pragma unroll
        for (int l = 0; l < 32; ++l) acc[l & 3] = __fadd2_rn(acc[l & 3], warp_ev[l * row_len + i]);
        out[i] = __fadd2_rn(__fadd2_rn(acc[0], acc[1]), __fadd2_rn(acc[2], acc[3]));
    }
}

// Adds a voxel's lanes' gradients together and writes the voxel's partial
// (T1, T2, M0, B1, inversion) for its train.
template <int L>
__device__ __forceinline__ void write_tissue_partial(const AdjointArgs& a, const TissueGrads& g,
                                                     int lane, int q, bool active, int64_t row) {
    float v[5] = {g.t1, g.t2, g.m0, g.b1, g.inv};
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

// Copies this lane's part of segment `seg`'s checkpoint (its orders of the
// three planes; zeros past `states`) into shared memory with cp.async, as
// one commit group. Each lane later reads back only what it copied, so a
// cp.async.wait_all of its own suffices.
template <int R, int T>
__device__ __forceinline__ void copy_checkpoint(float* s_ck, const AdjointArgs& a, int64_t train,
                                                int seg, int64_t atom, bool active, int q) {
    const int S = a.states;
    const int64_t n = a.atoms;
    const float* base =
        a.ckpt + (train * a.ckpt_count + seg) * (3 * int64_t(S)) * n + (active ? atom : 0);
    for (int plane = 0; plane < 3; ++plane) {
        for (int j = 0; j < R; ++j) {
            const int o = q * R + j;
            const bool ok = active && o < S;
            const float* src = ok ? base + (int64_t(plane) * S + o) * n : a.ckpt;
            const unsigned dst = static_cast<unsigned>(
                __cvta_generic_to_shared(s_ck + (plane * R + j) * T + threadIdx.x));
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(dst), "l"(src),
                         "r"(ok ? 4 : 0)
                         : "memory");
        }
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}

// Dynamic shared memory: ops [C] (16 B each), then per op and voxel slot the
// transcendentals (sin, cos, e1, e2) [C][VPB] float4, then the pre-RF states
// [C][3][RP][T] float2, then the per-lane event partials [T][C | 1] float2
// (an odd row length keeps the lanes' rows on distinct banks), then the
// recorded F+[0] of each op [C][T] float, then the next segment's checkpoint
// [3][R][T] float (filled by cp.async while the current segment runs).
template <int RP, int L, int W>
__global__ void __launch_bounds__(32 * W) epg_adjoint_kernel(const AdjointArgs a) {
    extern __shared__ __align__(16) unsigned char s_raw[];
    constexpr int VPW = 32 / L;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int q = lane % L;
    const int slot = lane / L;
    // Threads and voxel slots per block are compile-time, so every
    // shared-memory address below is a base plus an immediate offset.
    constexpr int T = 32 * W;
    constexpr int VPB = W * VPW;
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
    const int C1 = C | 1;
    float2* s_ev = s_stage + size_t(C) * 3 * RP * T;
    float2* my_ev = s_ev + size_t(threadIdx.x) * C1;
    const float2* warp_ev = s_ev + size_t(warp) * 32 * C1;
    float* s_rec = reinterpret_cast<float*>(s_ev + size_t(T) * C1);
    float* s_ck = s_rec + size_t(C) * T;

    const float t1 = a.t1[ac];
    const float t2 = a.t2[ac];
    VoxelConsts vc;
    vc.m0 = a.m0 ? a.m0[ac] : 1.f;
    vc.b1 = a.b1 ? a.b1[ac] : 1.f;
    vc.eff = a.inv ? a.inv[ac] : 1.f;
    vc.r1 = 1000.f / t1;
    vc.r2 = 1000.f / t2;
    vc.w1 = 1000.f / (t1 * t1);
    vc.w2 = 1000.f / (t2 * t2);

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

    TissueGrads g;
    float2* event_out = a.event_partial + (train * a.warps_per_train + warp_global) * a.n_ops;

    // The cotangent of the sample op i records (lane 0 of a voxel holds F+[0]).
    // Planes: the imaginary plane's value; interleaved 1j*(i v) = -v: minus
    // the real part.
    const bool planes = a.seed_layout == TSG_LAYOUT_PLANES;
    const int seed_stride = planes ? 1 : 2;
    const float seed_sign = planes ? 1.f : -1.f;
    const float* seed_row = a.seed + (active ? row : 0) * a.outputs * seed_stride;
    const bool lane0 = q == 0 && active;
    auto seed_at = [&](int i) -> float {
        const Op op = s_ops[i];
        if (!(op.code & OP_RECORD) || !lane0) return 0.f;
        return seed_sign * seed_row[int64_t(op.record) * seed_stride];
    };

    const int n_seg = (a.n_ops + C - 1) / C;
    if (n_seg > 0) copy_checkpoint<R, T>(s_ck, a, train, n_seg - 1, atom, active, q);
    for (int seg = n_seg - 1; seg >= 0; --seg) {
        const int o0 = seg * C;
        const int o1 = min(o0 + C, a.n_ops);
        const int cnt = o1 - o0;
        __syncthreads();
        for (int i = threadIdx.x; i < cnt; i += T) s_ops[i] = ops[o0 + i];
        __syncthreads();
        stage_transcendentals<L, VPW, VPB>(s_ops, s_tr, cnt, q, slot, vslot, vc.b1, vc.r1, vc.r2);
        __syncwarp();
        // The state entering op o0, copied in while the previous segment ran.
        asm volatile("cp.async.wait_all;\n" ::: "memory");
#pragma unroll
        for (int k = 0; k < RP; ++k) {
            P[k] = make_float2(s_ck[(0 * R + 2 * k) * T + threadIdx.x],
                               s_ck[(0 * R + 2 * k + 1) * T + threadIdx.x]);
            M[k] = make_float2(s_ck[(1 * R + 2 * k) * T + threadIdx.x],
                               s_ck[(1 * R + 2 * k + 1) * T + threadIdx.x]);
            Z[k] = make_float2(s_ck[(2 * R + 2 * k) * T + threadIdx.x],
                               s_ck[(2 * R + 2 * k + 1) * T + threadIdx.x]);
        }
        // The last op's seed is loaded now; the re-run hides its latency.
        float cur_seed = seed_at(cnt - 1);
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
                for (int k = 0; k < RP; ++k) Z[k] = mul2(Z[k], dup(-vc.eff));
            }
            for (int s = 0; s < op_shift2(code); ++s) shift_fwd<RP, L>(P, M, q, kill, kill_r);
            if (code & OP_SPOIL1) {
#pragma unroll
                for (int k = 0; k < RP; ++k) P[k] = M[k] = dup(0.f);
            }
            if (code & OP_RECORD) s_rec[i * T + threadIdx.x] = P[0].x;
            for (int s = 0; s < op_shift3(code); ++s) shift_fwd<RP, L>(P, M, q, kill, kill_r);
            if (code & OP_SPOIL2) {
#pragma unroll
                for (int k = 0; k < RP; ++k) P[k] = M[k] = dup(0.f);
            }
        }
        // The next segment's checkpoint streams in during the reverse pass.
        if (seg > 0) copy_checkpoint<R, T>(s_ck, a, train, seg - 1, atom, active, q);
        // Reverse over the segment; each op loads the seed of the op before
        // it, one iteration ahead of its use.
        for (int i = cnt - 1; i >= 0; --i) {
            const Op op = s_ops[i];
            const float4 tr = s_tr[i * VPB + vslot];
            const float next_seed = i > 0 ? seed_at(i - 1) : 0.f;
            const float2* st = s_stage + size_t(i) * 3 * RP * T + threadIdx.x;
            float2 p_[RP], m_[RP], z_[RP];
#pragma unroll
            for (int k = 0; k < RP; ++k) {
                p_[k] = st[(0 * RP + k) * T];
                m_[k] = st[(1 * RP + k) * T];
                z_[k] = st[(2 * RP + k) * T];
            }
            const float2 ev = reverse_op<RP, L>(op, tr, p_, m_, z_, 1.f, 1.f, 0.f, pb, mb, zb,
                                                cur_seed, s_rec[i * T + threadIdx.x], lane0, vc, g,
                                                q, kill, kill_r);
            cur_seed = next_seed;
            my_ev[i] = active ? ev : dup(0.f);
        }
        // Event gradients of the segment's ops, summed over the warp's lanes.
        __syncwarp();
        reduce_chunk_events(warp_ev, C1, cnt, lane, event_out + o0);
    }
    write_tissue_partial<L>(a, g, lane, q, active, row);
}

// Trajectory mode: the forward stored every op's entry state (float2 pairs
// in tiles of 32 atoms, [train][atom / 32][op][plane][pair][atom % 32]) and
// every recorded F+[0] ([train][output][atom]), so nothing is re-run but each
// op's relaxation, which folds into the reverse step. The whole program sits
// in shared memory; the reverse sweep walks the ops from last to first, and
// kTrajRing - 1 ops ahead of use each lane copies (cp.async) its pairs of an
// op's entry state, its seed and recorded F+[0] into a ring of shared-memory
// slots and evaluates the op's transcendentals into the same slot, so no
// global load and no transcendental sits on the reverse chain. Within a tile
// a lane's pairs of one op sit at fixed offsets from one pointer, so each
// copy is a register plus an immediate.
//
// Dynamic shared memory: ops [n_ops], the entry-state ring [D][3][RP][T]
// float2, the (seed, F+[0]) ring [D][T] float2, the transcendental ring
// [D][T] float4, per-lane event partials [T][K + 1] float2.
template <int RP, int L, int W>
__global__ void __launch_bounds__(32 * W) epg_adjoint_trajectory_kernel(const AdjointArgs a) {
    extern __shared__ __align__(16) unsigned char s_raw[];
    constexpr int VPW = 32 / L;
    constexpr int T = 32 * W;
    constexpr int K = kTrajChunk;
    constexpr int D = kTrajRing;
    constexpr int R = 2 * RP;
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
    const int NP = (S + 1) >> 1;
    const int n_ops = a.n_ops;

    float4* s_tring = reinterpret_cast<float4*>(s_raw);                 // [D][T]
    float2* s_ring = reinterpret_cast<float2*>(s_tring + D * T);        // [D][3][RP][T]
    float2* s_sring = s_ring + D * 3 * RP * T;                           // [D][T]
    float2* s_ev = s_sring + D * T;                                      // [T][K + 1]
    Op* s_ops = reinterpret_cast<Op*>(s_ev + T * (K + 1));               // [n_ops]
    float2* my_ev = s_ev + threadIdx.x * (K + 1);
    const float2* warp_ev = s_ev + warp * 32 * (K + 1);

    const float t1 = a.t1[ac];
    const float t2 = a.t2[ac];
    VoxelConsts vc;
    vc.m0 = a.m0 ? a.m0[ac] : 1.f;
    vc.b1 = a.b1 ? a.b1[ac] : 1.f;
    vc.eff = a.inv ? a.inv[ac] : 1.f;
    vc.r1 = 1000.f / t1;
    vc.r2 = 1000.f / t2;
    vc.w1 = 1000.f / (t1 * t1);
    vc.w2 = 1000.f / (t2 * t2);

    const bool kill = L * R > S;
    const int kill_r = S - q * R;
    const int64_t row = train * a.atoms + atom;
    const int64_t n = a.atoms;

    {
        const Op* ops = a.ops + train * n_ops;
        for (int i = threadIdx.x; i < n_ops; i += T) s_ops[i] = ops[i];
        __syncthreads();
    }

    float2 pb[RP], mb[RP], zb[RP];
#pragma unroll
    for (int k = 0; k < RP; ++k) pb[k] = mb[k] = zb[k] = dup(0.f);
    TissueGrads g;
    float2* event_out = a.event_partial + (train * a.warps_per_train + warp_global) * n_ops;

    const bool planes = a.seed_layout == TSG_LAYOUT_PLANES;
    const int seed_stride = planes ? 1 : 2;
    const float seed_sign = planes ? 1.f : -1.f;
    const float* seed_row = a.seed + (active ? row : 0) * a.outputs * seed_stride;
    const float* rec_col = a.traj_rec + train * a.outputs * n + ac;
    const bool lane0 = q == 0 && active;

    // This lane's pairs of op o: lane_traj + o * op_stride + plane * NP * 32
    // + k * 32 (float2). Inactive lanes read atom 0's column.
    const int64_t tiles = (n + 31) >> 5;
    const int64_t op_stride = 3 * int64_t(NP) * 32;
    const float2* lane_traj = a.traj + (train * tiles + (ac >> 5)) * n_ops * op_stride +
                              (ac & 31) + q * RP * 32;
    const int plane_stride = NP * 32;
    const unsigned ring_base = static_cast<unsigned>(__cvta_generic_to_shared(s_ring + threadIdx.x));
    const unsigned sring_base =
        static_cast<unsigned>(__cvta_generic_to_shared(s_sring + threadIdx.x));
    // Op o into ring slot `rs`: entry-state pairs (zero past the last pair),
    // seed and F+[0] (zero unless this lane records), transcendentals.
    auto fetch = [&](int o, int rs) {
        const float2* src_op = lane_traj + o * op_stride;
        const unsigned dst_op = ring_base + unsigned(rs * 3 * RP * T) * 8u;
        if (!kill) {
#pragma unroll
            for (int plane = 0; plane < 3; ++plane) {
                const float2* src = src_op + plane * plane_stride;
#pragma unroll
                for (int k = 0; k < RP; ++k)
                    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(
                                     dst_op + unsigned((plane * RP + k) * T) * 8u),
                                 "l"(src + k * 32)
                                 : "memory");
            }
        } else {
#pragma unroll
            for (int plane = 0; plane < 3; ++plane) {
                const float2* src = src_op + plane * plane_stride;
#pragma unroll
                for (int k = 0; k < RP; ++k) {
                    const bool ok = q * RP + k < NP;
                    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(
                                     dst_op + unsigned((plane * RP + k) * T) * 8u),
                                 "l"(ok ? src + k * 32 : a.traj), "r"(ok ? 8 : 0)
                                 : "memory");
                }
            }
        }
        const Op op = s_ops[o];
        const bool rec = lane0 && (op.code & OP_RECORD);
        const int64_t r = rec ? op.record : 0;
        const unsigned sdst = sring_base + unsigned(rs * T) * 8u;
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(sdst),
                     "l"(seed_row + r * seed_stride), "r"(rec ? 4 : 0)
                     : "memory");
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(sdst + 4u),
                     "l"(rec_col + r * n), "r"(rec ? 4 : 0)
                     : "memory");
        float si, co;
        sincosf(op.flip * vc.b1, &si, &co);
        s_tring[rs * T + threadIdx.x] =
            make_float4(si, co, expf(-vc.r1 * op.dt), expf(-vc.r2 * op.dt));
    };

    // Op o sits in ring slot (n_ops - 1 - o) % D.
#pragma unroll
    for (int j = 1; j < D; ++j) {
        if (n_ops - j >= 0) fetch(n_ops - j, j - 1);
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    }
    int use_slot = 0;
    int fill_slot = D - 1;
    int group = 0;  // ops processed since the last event reduction
    // Not unrolled: one op's body (the reverse step, its shifts and the
    // ring's bookkeeping) is large, and a second copy of it overflows the
    // instruction cache (measured: 0.76 -> 0.57 ms on 16,384 voxels x 601
    // ops x 20 states when the unroll by two was removed).
#pragma unroll 1
    for (int o = n_ops - 1; o >= 0; --o) {
        if (o - (D - 1) >= 0) fetch(o - (D - 1), fill_slot);
        asm volatile("cp.async.commit_group;\n" ::: "memory");
        fill_slot = fill_slot + 1 == D ? 0 : fill_slot + 1;
        const Op op = s_ops[o];
        const uint32_t code = op.code;
        asm volatile("cp.async.wait_group %0;\n" ::"n"(D - 1) : "memory");
        const float4 tr = s_tring[use_slot * T + threadIdx.x];
        const float2 sr = s_sring[use_slot * T + threadIdx.x];
        const float2* ring = s_ring + use_slot * (3 * RP * T) + threadIdx.x;
        use_slot = use_slot + 1 == D ? 0 : use_slot + 1;
        float2 p_[RP], m_[RP], z_[RP];
#pragma unroll
        for (int k = 0; k < RP; ++k) {
            p_[k] = ring[(0 * RP + k) * T];
            m_[k] = ring[(1 * RP + k) * T];
            z_[k] = ring[(2 * RP + k) * T];
        }
        // The pre-RF state: the entry state relaxed and shifted. Without a
        // shift in between, the relaxation folds into reverse_op.
        const bool relax = (code & OP_RELAX) != 0;
        float ep = 1.f, ez = 1.f, r0 = 0.f;
        if (relax && op_shift1(code) == 0) {
            ep = tr.w;
            ez = tr.z;
            r0 = 1.f - tr.z;
        } else if (relax) {
            const float2 E1 = dup(tr.z), E2 = dup(tr.w);
#pragma unroll
            for (int k = 0; k < RP; ++k) {
                p_[k] = mul2(p_[k], E2);
                m_[k] = mul2(m_[k], E2);
                z_[k] = mul2(z_[k], E1);
            }
            if (q == 0) z_[0].x += 1.f - tr.z;
            for (int s = 0; s < op_shift1(code); ++s) shift_fwd<RP, L>(p_, m_, q, kill, kill_r);
        } else {
            for (int s = 0; s < op_shift1(code); ++s) shift_fwd<RP, L>(p_, m_, q, kill, kill_r);
        }
        const float2 ev = reverse_op<RP, L>(op, tr, p_, m_, z_, ep, ez, r0, pb, mb, zb,
                                            seed_sign * sr.x, sr.y, lane0, vc, g, q, kill, kill_r);
        my_ev[group] = active ? ev : dup(0.f);
        // Every K ops (and at the end) the warp sums its lanes' partials:
        // entry j of the group is op o + group - j.
        if (++group == K || o == 0) {
            __syncwarp();
            for (int j = lane; j < group; j += 32) {
                float2 acc[4] = {dup(0.f), dup(0.f), dup(0.f), dup(0.f)};
#pragma unroll
                for (int l = 0; l < 32; ++l)
                    acc[l & 3] = __fadd2_rn(acc[l & 3], warp_ev[l * (K + 1) + j]);
                event_out[o + group - 1 - j] =
                    __fadd2_rn(__fadd2_rn(acc[0], acc[1]), __fadd2_rn(acc[2], acc[3]));
            }
            __syncwarp();
            group = 0;
        }
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    write_tissue_partial<L>(a, g, lane, q, active, row);
}

template <int RP, int L, int W>
void launch_adjoint(const AdjointArgs& a, dim3 grid, dim3 block, size_t smem, cudaStream_t s) {
    epg_adjoint_kernel<RP, L, W><<<grid, block, smem, s>>>(a);
}

template <int RP, int L, int W>
void launch_adjoint_trajectory(const AdjointArgs& a, dim3 grid, dim3 block, size_t smem,
                               cudaStream_t s) {
    epg_adjoint_trajectory_kernel<RP, L, W><<<grid, block, smem, s>>>(a);
}

// Entries take orders per lane R (even): the kernel keeps R/2 pairs.

// Entries take orders per lane R (even): the kernel keeps R/2 pairs.
#define TSG_ADJOINT_ENTRY(R, L, W)                              \
    {R, L, W, &launch_adjoint<(R) / 2, L, W>,                   \
     reinterpret_cast<const void*>(&epg_adjoint_kernel<(R) / 2, L, W>)}
#define TSG_ADJOINT_TRAJECTORY_ENTRY(R, L, W)                   \
    {R, L, W, &launch_adjoint_trajectory<(R) / 2, L, W>,        \
     reinterpret_cast<const void*>(&epg_adjoint_trajectory_kernel<(R) / 2, L, W>)}

}  // namespace tsg
