// One persistent launch over many sequences of uneven length, state count and
// voxel count (the reference runs one launch per sequence, each sized to its
// own problem: sequence/_epg_triton.py:17120-17300).
//
// The work list holds (sequence, voxel tile) units, largest first. Each CTA
// takes the next unit from a global counter (one atomicAdd, no waiting on
// other CTAs), stages that sequence's program in shared memory and runs the
// forward sweep for its voxels. Orders per lane (R, even) are fixed at
// compile time; lanes per voxel (L = ceil(states/R)) are per sequence, so one kernel
// serves every echo-train length: voxels take floor(32/L) slots of a warp and
// the shift's cross-lane moves respect the voxel boundaries through the lane's
// index within its voxel, exactly as in the fixed-shape sweep.
//
// Two loops share the kernel: a CPMG train runs the echo loop (no op
// decoding, the pulse in sum/difference form), any other program the general
// op loop; both keep the relaxation as pending factors that the pulse, the
// inversion and the record apply. 2-warp blocks at 16 orders per lane run an
// instantiation budgeted for 10 blocks per SM.
#include "tsg_internal.h"

namespace tsg {

namespace {

constexpr int kBatchOpChunk = 512;

__device__ __forceinline__ float2 dup(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// Truncation at `states`: the slot of order `states` on the voxel's last lane
// is cleared after every shift. `slot` (that order's index within the lane,
// -1 when the state count fills the lanes exactly) is the same for every lane
// of the block, which runs one sequence, so the switch is a uniform branch
// and only the lane that `kills` clears one value.
template <int RP>
__device__ __forceinline__ void truncate_slot(float2 (&p)[RP], int slot, bool kills) {
    switch (slot) {
#define TSG_TRUNCATE_CASE(k)                                  \
    case k:                                                   \
        if constexpr (k < 2 * RP) {                           \
            if constexpr (k < RP) {                           \
                if (kills) p[k].x = 0.f;                      \
            } else {                                          \
                if (kills) p[(k) - RP].y = 0.f;               \
            }                                                 \
        }                                                     \
        break;
        TSG_TRUNCATE_CASE(0) TSG_TRUNCATE_CASE(1) TSG_TRUNCATE_CASE(2) TSG_TRUNCATE_CASE(3)
        TSG_TRUNCATE_CASE(4) TSG_TRUNCATE_CASE(5) TSG_TRUNCATE_CASE(6) TSG_TRUNCATE_CASE(7)
        TSG_TRUNCATE_CASE(8) TSG_TRUNCATE_CASE(9) TSG_TRUNCATE_CASE(10) TSG_TRUNCATE_CASE(11)
        TSG_TRUNCATE_CASE(12) TSG_TRUNCATE_CASE(13) TSG_TRUNCATE_CASE(14) TSG_TRUNCATE_CASE(15)
#undef TSG_TRUNCATE_CASE
        default:
            break;
    }
}

// One gradient shift of the lane's strided order pairs (local order l in
// pair l % RP, .x below RP and .y above) with a per-sequence lane count L:
// F- moves one order down, F+ one order up, F+[0] = -F-[0] on the voxel's
// first lane, nothing crosses a voxel's edge, and the order `states` is
// cleared (truncate_slot). Whole pairs move except one at each edge.
template <int RP>
__device__ __forceinline__ void shift_pairs(float2 (&p)[RP], float2 (&m)[RP], int q, int L,
                                            int slot, bool kills) {
    const float in_p = __shfl_up_sync(0xffffffffu, p[RP - 1].y, 1);
    const float in_m = __shfl_down_sync(0xffffffffu, m[0].x, 1);
    const float top = (q == L - 1) ? 0.f : in_m;
    const float m_edge = m[0].y;
#pragma unroll
    for (int k = 0; k + 1 < RP; ++k) m[k] = m[k + 1];
    m[RP - 1] = make_float2(m_edge, top);
    const float bottom = (q == 0) ? -m[0].x : in_p;
    const float p_edge = p[RP - 1].x;
#pragma unroll
    for (int k = RP - 1; k > 0; --k) p[k] = p[k - 1];
    p[0] = make_float2(bottom, p_edge);
    truncate_slot<RP>(p, slot, kills);
}

// The pulse on the relaxed state (w2 p, w2 m, w1 z + (1 - w1) at order 0,
// with the factors w1, w2 the relaxation still owes), without the recovery
// term, which only the voxel's first lane adds.
template <int RP>
__device__ __forceinline__ void rotate_pairs(float2 (&P)[RP], float2 (&M)[RP], float2 (&Z)[RP],
                                             float si, float co, float w1, float w2) {
    const float a = 0.5f * (1.f + co) * w2, b = 0.5f * (1.f - co) * w2;
    const float c = si * w1, h = 0.5f * si * w2, d = co * w1;
    const float2 A = dup(a), B = dup(b), C = dup(c), nC = dup(-c), H = dup(h), nH = dup(-h),
                 Dz = dup(d);
#pragma unroll
    for (int k = 0; k < RP; ++k) {
        const float2 p = P[k], m = M[k], z = Z[k];
        P[k] = fma2(A, p, fma2(B, m, mul2(nC, z)));
        M[k] = fma2(B, p, fma2(A, m, mul2(C, z)));
        Z[k] = fma2(H, p, fma2(nH, m, mul2(Dz, z)));
    }
}

// The same pulse in sum/difference form, for the echo loop: with S = p + m
// and D = p - m, P' = k S + T and M' = k S - T where T = e D - c z, and
// Z' = h D + d z (k = w2/2, e = k cos, c = w1 sin, h = k sin, d = w1 cos).
// The coefficient pairs come from the shuffled (sin, sin) and (cos, cos)
// pairs by four paired products; K, W1 and -W1 are fixed per phase.
template <int RP>
__device__ __forceinline__ void rotate_sumdiff(float2 (&P)[RP], float2 (&M)[RP], float2 (&Z)[RP],
                                               float2 si2, float2 co2, float2 K, float2 W1,
                                               float2 nW1) {
    const float2 neg1 = dup(-1.f);
    const float2 E = mul2(co2, K), nC = mul2(si2, nW1), H = mul2(si2, K), Dz = mul2(co2, W1);
#pragma unroll
    for (int k = 0; k < RP; ++k) {
        const float2 p = P[k], m = M[k], z = Z[k];
        const float2 S = __fadd2_rn(p, m);
        const float2 D = fma2(m, neg1, p);
        const float2 T = fma2(E, D, mul2(nC, z));
        const float2 KS = mul2(K, S);
        P[k] = __fadd2_rn(KS, T);
        M[k] = fma2(T, neg1, KS);
        Z[k] = fma2(H, D, mul2(Dz, z));
    }
}

// A refocusing op of a CPMG echo: relax, shift, rotate, shift, nothing else.
// It takes a straight-line path in which the shifts' moves fold into the
// relaxation's and the rotation's own results.
constexpr uint32_t kEchoMask = OP_RELAX | (3u << OP_SHIFT1_SHIFT) | (3u << OP_RF_SHIFT) |
                               (3u << OP_SHIFT2_SHIFT) | OP_SPOIL1 | OP_RECORD |
                               (3u << OP_SHIFT3_SHIFT) | OP_SPOIL2;
constexpr uint32_t kEchoBits = OP_RELAX | (1u << OP_SHIFT1_SHIFT) |
                               (uint32_t(RF_ROTATE) << OP_RF_SHIFT) | (1u << OP_SHIFT2_SHIFT);
// The recording op of a CPMG echo: relax and record, nothing else.
constexpr uint32_t kRecordBits = OP_RELAX | OP_RECORD;

}  // namespace

// Orders are held as pairs (R / 2 float2 per plane) and advanced with the
// paired FP32 instructions; each pulse's sin/cos is evaluated once per voxel:
// lane q of a voxel takes one of every L ops and the voxel's lanes exchange
// the values by shuffle (all lanes of a warp run the same sequence, so the
// shuffles are convergent).
// NARROW instantiations serve 2-warp blocks only, under a register budget
// that lets kNarrowBlocks of them share an SM.
#ifndef TSG_BATCH_NARROW_BLOCKS
#define TSG_BATCH_NARROW_BLOCKS 10
#endif
constexpr int kNarrowBlocks = TSG_BATCH_NARROW_BLOCKS;
template <int R, bool NARROW = false>
__global__ void __launch_bounds__(NARROW ? 64 : 256, NARROW ? kNarrowBlocks : 1) epg_batched_kernel(
    const Op* __restrict__ ops, const tsg_batch_sequence* __restrict__ seqs,
    const tsg_batch_unit* __restrict__ units, int64_t unit_count, int* __restrict__ counter,
    const float* __restrict__ t1v, const float* __restrict__ t2v, const float* __restrict__ m0v,
    const float* __restrict__ b1v, float2* __restrict__ out) {
    constexpr int RP = R / 2;
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
        const int first_lane = lane - q;
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
        // The order `states` falls on the voxel's last lane, at slot S % R
        // (none when the lanes hold exactly S orders).
        const int kill_slot = L * R > S ? S % R : -1;
        const bool kills = q == L - 1;
        float2 P[RP], M[RP], Z[RP];
#pragma unroll
        for (int k = 0; k < RP; ++k) P[k] = M[k] = Z[k] = dup(0.f);
        if (q == 0) Z[0].x = 1.f;
        float last_dt = __int_as_float(0x7fffffff);
        float e1 = 1.f, e2 = 1.f;
        // Relaxation not yet applied to the state: F+ and F- owe a factor pe2,
        // Z owes pe1 and the recovery 1 - pe1 at order 0. A relaxation only
        // multiplies these (a shift moves F+ and F- orders, which share the
        // factor, and leaves Z alone, so it commutes with them); the pulse,
        // the inversion and the record apply them in their own coefficients.
        float pe1 = 1.f, pe2 = 1.f;
        float2* orow = out + sq.output_offset + int64_t(u.voxel_begin + local) * sq.outputs;
        for (int base = 0; base < sq.op_count; base += kBatchOpChunk) {
            const int count = min(kBatchOpChunk, sq.op_count - base);
            __syncthreads();
            for (int i = threadIdx.x; i < count; i += blockDim.x)
                s_ops[i] = ops[sq.op_offset + base + i];
            __syncthreads();
            // A CPMG train held whole in one chunk -- the excitation alone,
            // then per echo the refocusing op and the recording op (echo e
            // recorded as sample e), one interval throughout -- runs the echo
            // loop: no op decoding, the relaxation factors fixed (e at the
            // first echo, e^2 after), the pulse in sum/difference form, the
            // record pointer advanced by one sample per echo.
            if (base == 0 && count == sq.op_count) {
                const bool odd = (count & 1) && count >= 3;
                bool fits = odd;
                for (int i = threadIdx.x; odd && i < count; i += blockDim.x) {
                    const Op o = s_ops[i];
                    if (i == 0)
                        fits &= o.code == (uint32_t(RF_ROTATE) << OP_RF_SHIFT);
                    else
                        fits &= (o.code & kEchoMask) == ((i & 1) ? kEchoBits : kRecordBits) &&
                                o.dt == s_ops[1].dt && ((i & 1) || o.record == (i >> 1) - 1);
                }
                if (__syncthreads_and(fits)) {
                    const int echoes = count >> 1;
                    {
                        float si, co;
                        sincosf(s_ops[0].flip * b1, &si, &co);
                        rotate_pairs<RP>(P, M, Z, si, co, 1.f, 1.f);  // recovery 1 - 1 = 0
                    }
                    const float dt = s_ops[1].dt;
                    const float f1 = expf(-r1 * dt), f2 = expf(-r2 * dt);
                    const float f11 = f1 * f1, f22 = f2 * f2;
                    const float m0f2 = m0 * f2;
                    float w1 = f1;
                    float2 K = dup(0.5f * f2), W1 = dup(f1), nW1 = dup(-f1);
                    float my_si = 0.f, my_co = 1.f;
                    int g = L;  // echoes since the voxel's lanes last evaluated sin/cos
                    float2* rec = orow;
                    for (int e = 0; e < echoes; ++e) {
                        if (g == L) {
                            g = 0;
                            const int j = e + q;
                            float sj = 0.f, cj = 1.f;
                            if (j < echoes) sincosf(s_ops[2 * j + 1].flip * b1, &sj, &cj);
                            my_si = sj;
                            my_co = cj;
                        }
                        const float si = __shfl_sync(0xffffffffu, my_si, first_lane + g);
                        const float co = __shfl_sync(0xffffffffu, my_co, first_lane + g);
                        ++g;
                        shift_pairs<RP>(P, M, q, L, kill_slot, kills);
                        rotate_sumdiff<RP>(P, M, Z, dup(si), dup(co), K, W1, nW1);
                        if (q == 0) {
                            const float r = 1.f - w1;
                            P[0].x = fmaf(-si, r, P[0].x);
                            M[0].x = fmaf(si, r, M[0].x);
                            Z[0].x = fmaf(co, r, Z[0].x);
                        }
                        shift_pairs<RP>(P, M, q, L, kill_slot, kills);
                        if (q == 0 && active) __stcs(rec, make_float2(0.f, m0f2 * P[0].x));
                        ++rec;
                        w1 = f11;
                        K = dup(0.5f * f22);
                        W1 = dup(f11);
                        nW1 = dup(-f11);
                    }
                    continue;
                }
            }
            float my_si = 0.f, my_co = 1.f;
            int g = L;  // ops since the voxel's lanes last evaluated sin/cos
            for (int i = 0; i < count; ++i) {
                if (g == L) {
                    g = 0;
                    const int j = i + q;
                    float sj = 0.f, cj = 1.f;
                    if (j < count) {
                        const Op oj = s_ops[j];
                        if (op_rf(oj.code) == RF_ROTATE) sincosf(oj.flip * b1, &sj, &cj);
                    }
                    my_si = sj;
                    my_co = cj;
                }
                const Op op = s_ops[i];
                const uint32_t code = op.code;
                auto relax = [&]() {
                    if (op.dt != last_dt) {
                        last_dt = op.dt;
                        e1 = expf(-r1 * op.dt);
                        e2 = expf(-r2 * op.dt);
                    }
                    pe1 *= e1;
                    pe2 *= e2;
                };
                // The pulse on the relaxed state (pe2 p, pe2 m, pe1 z + (1 - pe1)
                // at order 0): the factors ride in the coefficients.
                auto rotate = [&]() {
                    const float si = __shfl_sync(0xffffffffu, my_si, first_lane + g);
                    const float co = __shfl_sync(0xffffffffu, my_co, first_lane + g);
                    rotate_pairs<RP>(P, M, Z, si, co, pe1, pe2);
                    if (q == 0) {
                        const float r = 1.f - pe1;
                        P[0].x = fmaf(-si, r, P[0].x);
                        M[0].x = fmaf(si, r, M[0].x);
                        Z[0].x = fmaf(co, r, Z[0].x);
                    }
                    pe1 = pe2 = 1.f;
                };
                if ((code & kEchoMask) == kEchoBits) {
                    relax();
                    shift_pairs<RP>(P, M, q, L, kill_slot, kills);
                    rotate();
                    ++g;
                    shift_pairs<RP>(P, M, q, L, kill_slot, kills);
                    continue;
                }
                if ((code & kEchoMask) == kRecordBits) {
                    relax();
                    if (q == 0 && active)
                        __stcs(orow + op.record, make_float2(0.f, (m0 * pe2) * P[0].x));
                    ++g;
                    continue;
                }
                if (code & OP_RELAX) relax();
                for (int s = 0; s < op_shift1(code); ++s) shift_pairs<RP>(P, M, q, L, kill_slot, kills);
                const int rf = op_rf(code);
                if (rf == RF_ROTATE) {
                    rotate();
                } else if (rf == RF_INVERT) {
                    // Z -> -(pe1 Z + (1 - pe1) at order 0); F+ and F- keep
                    // owing pe2.
                    const float2 f = dup(-pe1);
#pragma unroll
                    for (int k = 0; k < RP; ++k) Z[k] = mul2(Z[k], f);
                    if (q == 0) Z[0].x -= 1.f - pe1;
                    pe1 = 1.f;
                }
                ++g;
                for (int s = 0; s < op_shift2(code); ++s) shift_pairs<RP>(P, M, q, L, kill_slot, kills);
                if (code & OP_SPOIL1) {
#pragma unroll
                    for (int k = 0; k < RP; ++k) P[k] = M[k] = dup(0.f);
                }
                if ((code & OP_RECORD) && q == 0 && active)
                    __stcs(orow + op.record, make_float2(0.f, (m0 * pe2) * P[0].x));
                for (int s = 0; s < op_shift3(code); ++s) shift_pairs<RP>(P, M, q, L, kill_slot, kills);
                if (code & OP_SPOIL2) {
#pragma unroll
                    for (int k = 0; k < RP; ++k) P[k] = M[k] = dup(0.f);
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
        case 16:
            if (warps_per_block == 2)
                epg_batched_kernel<16, true><<<grid, block, 0, s>>>(
                    o, sequences, units, unit_count, counter, tissue->t1_ms, tissue->t2_ms,
                    tissue->m0, tissue->b1, y);
            else
                epg_batched_kernel<16><<<grid, block, 0, s>>>(o, sequences, units, unit_count,
                                                               counter, tissue->t1_ms,
                                                               tissue->t2_ms, tissue->m0,
                                                               tissue->b1, y);
            break;
        default:
            return fail(TSG_ERR_UNSUPPORTED, "orders_per_lane must be 2, 4, 8 or 16");
    }
    TSG_CUDA(cudaGetLastError());
    return TSG_OK;
}
