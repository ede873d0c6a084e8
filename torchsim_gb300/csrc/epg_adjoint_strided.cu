// Trajectory-mode reverse sweep for one voxel per lane (up to 20 states),
// over the strided trajectory the one-lane forward sweep stores.
//
// The forward keeps a voxel's R = 2 RP orders as strided pairs (pair k =
// orders k and k + RP) and, in trajectory mode, stores the entry state of
// every even op exactly as it holds it, two pairs per 16-byte granule
// ([train][atom/32][op/2][plane][granule][atom%32] float4): half the bytes of
// every op's state, which is what bounds both sweeps here. This sweep walks
// the ops back in (even, odd) pairs, runs the even op forward once to get the
// odd op's entry state, and keeps its cotangents in the same layout, so:
//   * each stored state arrives by 3 x ceil(RP/2) 16-byte cp.async copies
//     into a ring of shared-memory slots, kTrajRing - 1 pairs ahead of use,
//     from a pointer that moves back one pair per step (the even state is
//     read from the ring twice: before the re-run and for its own step);
//   * a gradient shift moves whole pairs, and in the op shape of an MRF
//     repetition (relax, rotate, record, one shift after) the shift's
//     transpose is folded into the operands of the rotation's transpose: the
//     F+ cotangents are read one pair up and updated in place in increasing
//     order, the F- cotangents read one pair down and written one pair late,
//     so neither side needs a register move;
//   * any other op shape, or a state count below R, takes the general step
//     (reverse_op with the strided shifts).
// Gradient algebra, event partials and their fixed-order reductions are the
// contiguous trajectory sweep's (epg_adjoint.cuh).
#include "epg_adjoint.cuh"

namespace tsg {

namespace {

// The transposed steps of an MRF-shaped op: shift (folded), record,
// rotation, relaxation. The op's relaxation folds into the coefficients
// (pre-RF state = (e2 p, e2 m, e1 z + (1 - e1) at order 0)). Returns this
// lane's (dL/dflip, dL/dduration) of the op.
template <int RP>
__device__ __forceinline__ float2 reverse_mrf_op(const Op& op, const float4& tr,
                                                 const float2 (&p_)[RP], const float2 (&m_)[RP],
                                                 const float2 (&z_)[RP], float2 (&pb)[RP],
                                                 float2 (&mb)[RP], float2 (&zb)[RP], float seed,
                                                 float rec, bool lane0, const VoxelConsts& v,
                                                 TissueGrads& g) {
    const float si = tr.x, co = tr.y, e1 = tr.z, e2 = tr.w;
    const float ep = e2, ez = e1, r0 = 1.f - e1;
    // Cotangents after the shift's transpose: F+ one order down, F- one up,
    // F+[0]'s coupling to F-[1]; the record's seed lands on F+[0].
    const float pb0x = pb[0].x, pb0y = pb[0].y, mb_top = mb[RP - 1].x;
    auto PB = [&](int k) -> float2 { return k + 1 < RP ? pb[k + 1] : make_float2(pb0y, 0.f); };
    float2 mb_prev = make_float2(0.f, mb_top);  // MB(0)
    float pb_seed = 0.f;
    if ((op.code & OP_RECORD) && lane0) {
        pb_seed = seed * v.m0;
        g.m0 = fmaf(seed, rec, g.m0);
    }
    const float2 ch = dup(0.5f * (1.f + co)), sh = dup(0.5f * (1.f - co));
    const float2 hs = dup(0.5f * si), nhs = dup(-0.5f * si);
    const float2 si2 = dup(si), co2 = dup(co);
    const float2 hs_w = dup(0.5f * si * ep), co_z = dup(co * ez);
    const float2 hc_w = dup(0.5f * co * ep), nsi_z = dup(-si * ez);
    const float2 neg1 = dup(-1.f);
    const float2 E1 = dup(e1), E2 = dup(e2);
    float2 ga0 = dup(0.f), ga1 = dup(0.f), A2a = dup(0.f), A2b = dup(0.f), A1 = dup(0.f);
    float fix = 0.f, nzb0 = 0.f;
    float2 pending = dup(0.f);  // the new F- cotangent of the previous pair
#pragma unroll
    for (int k = 0; k < RP; ++k) {
        float2 pbk = PB(k);
        float2 mbk = mb_prev;
        if (k + 1 < RP) mb_prev = mb[k];  // read before this pair's late write
        if (k == 0) pbk.x += pb_seed;
        if (k == 1) mbk.x -= pb0x;
        const float2 zbk = zb[k];
        if (k == 0) fix = r0 * (co * (mbk.x - pbk.x) - si * zbk.x);
        const float2 w = fma2(neg1, m_[k], p_[k]);
        const float2 d = fma2(neg1, pbk, mbk);
        ga0 = fma2(d, fma2(hs_w, w, mul2(co_z, z_[k])), ga0);
        ga1 = fma2(zbk, fma2(hc_w, w, mul2(nsi_z, z_[k])), ga1);
        const float2 npb = fma2(ch, pbk, fma2(sh, mbk, mul2(hs, zbk)));
        const float2 nmb = fma2(sh, pbk, fma2(ch, mbk, mul2(nhs, zbk)));
        const float2 nzb = fma2(si2, d, mul2(co2, zbk));
        if (k == 0) nzb0 = nzb.x;
        A2a = fma2(npb, p_[k], A2a);
        A2b = fma2(nmb, m_[k], A2b);
        A1 = fma2(nzb, z_[k], A1);
        pb[k] = mul2(npb, E2);
        zb[k] = mul2(nzb, E1);
        if (k > 0) mb[k - 1] = pending;
        pending = mul2(nmb, E2);
    }
    mb[RP - 1] = pending;
    const float gsum = (ga0.x + ga1.x) + (ga0.y + ga1.y) + fix;
    g.b1 = fmaf(gsum, op.flip, g.b1);
    const float a2 = ep * ((A2a.x + A2b.x) + (A2a.y + A2b.y));
    const float a1 = ez * (A1.x + A1.y) + (r0 - 1.f) * nzb0;
    g.t2 = fmaf(a2, op.dt * v.w2, g.t2);
    g.t1 = fmaf(a1, op.dt * v.w1, g.t1);
    return make_float2(gsum * v.b1, -v.r2 * a2 - v.r1 * a1);
}

// One op forward on a strided one-lane state (relax, shifts, pulse, spoils;
// the record leaves the state as it is): the odd op's entry state from the
// stored even one. tr = (sin, cos, e1, e2) of the op.
template <int RP>
__device__ __forceinline__ void forward_op_strided(const Op& op, const float4& tr, float2 (&p)[RP],
                                                   float2 (&m)[RP], float2 (&z)[RP], float eff,
                                                   bool kill, int kill_r) {
    const uint32_t code = op.code;
    if (code & OP_RELAX) {
        const float2 E1 = dup(tr.z), E2 = dup(tr.w);
#pragma unroll
        for (int k = 0; k < RP; ++k) {
            p[k] = mul2(p[k], E2);
            m[k] = mul2(m[k], E2);
            z[k] = mul2(z[k], E1);
        }
        z[0].x += 1.f - tr.z;
    }
    for (int s = 0; s < op_shift1(code); ++s) shift_fwd_strided<RP>(p, m, kill, kill_r);
    const int rf = op_rf(code);
    if (rf == RF_ROTATE) {
        const float si = tr.x, co = tr.y;
        const float2 ch = dup(0.5f * (1.f + co)), sh = dup(0.5f * (1.f - co));
        const float2 hs = dup(0.5f * si), si2 = dup(si), nsi2 = dup(-si), co2 = dup(co);
        const float2 neg1 = dup(-1.f);
#pragma unroll
        for (int k = 0; k < RP; ++k) {
            const float2 pk = p[k], mk = m[k], zk = z[k];
            p[k] = fma2(ch, pk, fma2(sh, mk, mul2(nsi2, zk)));
            m[k] = fma2(sh, pk, fma2(ch, mk, mul2(si2, zk)));
            z[k] = fma2(hs, fma2(neg1, mk, pk), mul2(co2, zk));
        }
    } else if (rf == RF_INVERT) {
#pragma unroll
        for (int k = 0; k < RP; ++k) z[k] = mul2(z[k], dup(-eff));
    }
    for (int s = 0; s < op_shift2(code); ++s) shift_fwd_strided<RP>(p, m, kill, kill_r);
    if (code & OP_SPOIL1) {
#pragma unroll
        for (int k = 0; k < RP; ++k) p[k] = m[k] = dup(0.f);
    }
    for (int s = 0; s < op_shift3(code); ++s) shift_fwd_strided<RP>(p, m, kill, kill_r);
    if (code & OP_SPOIL2) {
#pragma unroll
        for (int k = 0; k < RP; ++k) p[k] = m[k] = dup(0.f);
    }
}

// Dynamic shared memory, per ring slot one stored (even) op and the odd op
// after it: the transcendentals [D][2][T] float4, the entry state of the even
// op [D][3][G][T] float4, the (seed, F+[0]) of both [D][2][T] float2; then
// per-lane event partials [T][K + 1] float2 and the ops [n_ops].
template <int RP, int W>
__global__ void __launch_bounds__(32 * W) epg_adjoint_strided_kernel(const AdjointArgs a) {
    extern __shared__ __align__(16) unsigned char s_raw[];
    constexpr int T = 32 * W;
    constexpr int K = kTrajChunk;
    constexpr int D = kTrajRing;
    constexpr int R = 2 * RP;
    constexpr int G = (RP + 1) / 2;
    static_assert(K % 2 == 0, "event groups hold whole pairs of ops");
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int64_t warp_global = int64_t(blockIdx.x) * W + warp;
    const int64_t atom = warp_global * 32 + lane;
    const int64_t train = blockIdx.y;
    const bool active = atom < a.atoms;
    const int64_t ac = active ? atom : 0;
    const int S = a.states;
    const int n_ops = a.n_ops;
    const int n_pairs = (n_ops + 1) >> 1;

    float4* s_tring = reinterpret_cast<float4*>(s_raw);          // [D][2][T]
    float4* s_ring = s_tring + D * 2 * T;                         // [D][3][G][T]
    float2* s_sring = reinterpret_cast<float2*>(s_ring + D * 3 * G * T);  // [D][2][T]
    float2* s_ev = s_sring + D * 2 * T;                           // [T][K + 1]
    Op* s_ops = reinterpret_cast<Op*>(s_ev + T * (K + 1));        // [n_ops]
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

    const bool kill = R > S;
    const int kill_r = S;
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
    const bool lane0 = active;

    // One stored op of this lane's granules is 3 * G * 32 float4 on; the
    // fetch pointer starts at the last pair and moves back one pair per fetch.
    constexpr int op_stride = 3 * G * 32;
    const float4* fetch_ptr = reinterpret_cast<const float4*>(a.traj) +
                              ((train * ((n + 31) >> 5) + (ac >> 5)) * int64_t(n_pairs) +
                               (n_pairs - 1)) * op_stride +
                              (ac & 31);
    const unsigned ring_base = static_cast<unsigned>(__cvta_generic_to_shared(s_ring + threadIdx.x));
    const unsigned sring_base =
        static_cast<unsigned>(__cvta_generic_to_shared(s_sring + threadIdx.x));
    // The next pair to fetch (from the last down) into ring slot `rs`: the
    // even op's entry state, and for it and the odd op after it the seed,
    // the recorded F+[0] and the transcendentals.
    int fetch_pair = n_pairs - 1;
    auto fetch = [&](int rs) {
        const unsigned dst = ring_base + unsigned(rs * 3 * G * T) * 16u;
#pragma unroll
        for (int j = 0; j < 3 * G; ++j)
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(
                             dst + unsigned(j * T) * 16u),
                         "l"(fetch_ptr + j * 32)
                         : "memory");
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int o = 2 * fetch_pair + h;
            const bool here = o < n_ops;
            const Op op = s_ops[here ? o : 2 * fetch_pair];
            const bool rec = here && lane0 && (op.code & OP_RECORD);
            const int64_t r = rec ? op.record : 0;
            const unsigned sdst = sring_base + unsigned((rs * 2 + h) * T) * 8u;
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(sdst),
                         "l"(seed_row + r * seed_stride), "r"(rec ? 4 : 0)
                         : "memory");
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(sdst + 4u),
                         "l"(rec_col + r * n), "r"(rec ? 4 : 0)
                         : "memory");
            // The hardware approximations (|error| ~1e-6 relative for these
            // arguments, an angle of at most a few radians and exponents of a
            // few units): the gradient's tolerance is 1e-4, and the exact
            // routines cost a fifth of this loop's instructions.
            float si, co;
            __sincosf(op.flip * vc.b1, &si, &co);
            s_tring[(rs * 2 + h) * T + threadIdx.x] =
                make_float4(si, co, __expf(-vc.r1 * op.dt), __expf(-vc.r2 * op.dt));
        }
        fetch_ptr -= op_stride;
        --fetch_pair;
    };

    // Pair q sits in ring slot (n_pairs - 1 - q) % D.
#pragma unroll
    for (int j = 1; j < D; ++j) {
        if (fetch_pair >= 0) fetch(j - 1);
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    }
    int use_slot = 0;
    int fill_slot = D - 1;
    int group = 0;  // ops processed since the last event reduction
    const bool fast_ok = !kill;

    float2 p_[RP], m_[RP], z_[RP];
    auto load_entry = [&](const float4* ring) {
#pragma unroll
        for (int j = 0; j < G; ++j) {
            const float4 pp = ring[(0 * G + j) * T];
            const float4 mm = ring[(1 * G + j) * T];
            const float4 zz = ring[(2 * G + j) * T];
            p_[2 * j] = make_float2(pp.x, pp.y);
            m_[2 * j] = make_float2(mm.x, mm.y);
            z_[2 * j] = make_float2(zz.x, zz.y);
            if (2 * j + 1 < RP) {
                p_[2 * j + 1] = make_float2(pp.z, pp.w);
                m_[2 * j + 1] = make_float2(mm.z, mm.w);
                z_[2 * j + 1] = make_float2(zz.z, zz.w);
            }
        }
    };
    // The reverse step of op `op` from its entry state in (p_, m_, z_).
    auto reverse_at = [&](const Op& op, const float4& tr, const float2& sr) -> float2 {
        const uint32_t code = op.code;
        if (fast_ok && (code & kFastMask) == kFastBits)
            return reverse_mrf_op<RP>(op, tr, p_, m_, z_, pb, mb, zb, seed_sign * sr.x, sr.y,
                                      lane0, vc, g);
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
            z_[0].x += 1.f - tr.z;
            for (int s = 0; s < op_shift1(code); ++s) shift_fwd_strided<RP>(p_, m_, kill, kill_r);
        } else {
            for (int s = 0; s < op_shift1(code); ++s) shift_fwd_strided<RP>(p_, m_, kill, kill_r);
        }
        return reverse_op<RP, 1, true>(op, tr, p_, m_, z_, ep, ez, r0, pb, mb, zb,
                                       seed_sign * sr.x, sr.y, lane0, vc, g, 0, kill, kill_r);
    };

    // Not unrolled: a second copy of the body overflows the instruction cache.
#pragma unroll 1
    for (int q = n_pairs - 1; q >= 0; --q) {
        if (fetch_pair >= 0) fetch(fill_slot);
        asm volatile("cp.async.commit_group;\n" ::: "memory");
        fill_slot = fill_slot + 1 == D ? 0 : fill_slot + 1;
        asm volatile("cp.async.wait_group %0;\n" ::"n"(D - 1) : "memory");
        const int o = 2 * q;
        const Op op_even = s_ops[o];
        const float4 tr_even = s_tring[(use_slot * 2) * T + threadIdx.x];
        const float2 sr_even = s_sring[(use_slot * 2) * T + threadIdx.x];
        const float4* ring = s_ring + use_slot * (3 * G * T) + threadIdx.x;
        if (o + 1 < n_ops) {
            // The odd op: its entry state is the even op run forward.
            const Op op_odd = s_ops[o + 1];
            const float4 tr_odd = s_tring[(use_slot * 2 + 1) * T + threadIdx.x];
            const float2 sr_odd = s_sring[(use_slot * 2 + 1) * T + threadIdx.x];
            load_entry(ring);
            forward_op_strided<RP>(op_even, tr_even, p_, m_, z_, vc.eff, kill, kill_r);
            const float2 ev = reverse_at(op_odd, tr_odd, sr_odd);
            my_ev[group++] = active ? ev : dup(0.f);
        }
        load_entry(ring);
        use_slot = use_slot + 1 == D ? 0 : use_slot + 1;
        const float2 ev = reverse_at(op_even, tr_even, sr_even);
        my_ev[group++] = active ? ev : dup(0.f);
        // Every K ops (and at the end) the warp sums its lanes' partials:
        // entry j of the group is op o + group - 1 - j.
        if (group >= K || q == 0) {
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
    write_tissue_partial<1>(a, g, lane, 0, active, row);
}

template <int RP, int W>
void launch_strided(const AdjointArgs& a, dim3 grid, dim3 block, size_t smem, cudaStream_t s) {
    epg_adjoint_strided_kernel<RP, W><<<grid, block, smem, s>>>(a);
}

#define TSG_STRIDED_ENTRY(R, W) \
    {R, 1, W, &launch_strided<(R) / 2, W>, \
     reinterpret_cast<const void*>(&epg_adjoint_strided_kernel<(R) / 2, W>)}

const AdjointEntry kStrided[] = {
    TSG_STRIDED_ENTRY(10, 2), TSG_STRIDED_ENTRY(10, 4),
    TSG_STRIDED_ENTRY(20, 2), TSG_STRIDED_ENTRY(20, 4),
};

}  // namespace

const AdjointEntry* adjoint_strided_entry(int orders, int warps) {
    for (const AdjointEntry& e : kStrided)
        if (e.orders_per_lane == orders && e.warps == warps) return &e;
    return nullptr;
}

}  // namespace tsg
