// The complex EPG forward sweep: one pool, instant RF, with RF and receiver
// phases, a transmit phase (B1phase) and off-resonance (B0) per voxel -- what
// leaves the real subspace (the reference's simulate_range<INSTANT, ONE>,
// src/torchsim/_epg_cpu.cpp:4216-4566, with shift 2164-2174 and rotate
// 2176-2208).
//
// Thread mapping as in the real sweep: one voxel's orders spread over L lanes,
// R orders per lane held as R/2 pairs; each complex plane (F+, F-, Z) is two
// real planes (re, im) of pairs, so a complex product by a per-op coefficient
// is four paired FP32 instructions with no register shuffling. The shift moves
// F- down and F+ up; F+[0] takes the conjugate of the new F-[0] on the
// voxel's first lane.
#include "tsg_internal.h"

namespace tsg {

namespace {

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

template <int RP, int L>
__global__ void __launch_bounds__(256) epg_complex_kernel(const ComplexArgs a) {
    constexpr int R = 2 * RP;
    constexpr int VPW = 32 / L;
    __shared__ Op s_ops[kComplexOpChunk];
    __shared__ float2 s_ph[kComplexOpChunk];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int q = lane % L;
    const int slot = lane / L;
    const int64_t atom = (int64_t(blockIdx.x) * (blockDim.x >> 5) + warp) * VPW + slot;
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
    const bool off_axis = a.b0 != nullptr;
    const bool kill = L * R > a.states;
    const int kill_r = a.states - q * R;

    float2 Pr[RP], Pi[RP], Mr[RP], Mi[RP], Zr[RP], Zi[RP];
#pragma unroll
    for (int k = 0; k < RP; ++k) Pr[k] = Pi[k] = Mr[k] = Mi[k] = Zr[k] = Zi[k] = dup(0.f);
    if (q == 0) Zr[0].x = 1.f;

    const Op* ops = a.ops + train * a.n_ops;
    const float2* phase = a.phase + train * a.n_ops;
    const int64_t out_base = (train * a.atoms + atom) * a.outputs;
    float last_dt = __int_as_float(0x7fffffff);
    float e1 = 1.f, tr = 1.f, ti = 0.f;

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
            if (code & OP_RELAX) {
                if (op.dt != last_dt) {
                    last_dt = op.dt;
                    e1 = expf(-r1 * op.dt);
                    const float e2 = expf(-r2 * op.dt);
                    tr = e2;
                    ti = 0.f;
                    if (off_axis) {
                        // Off-resonance turns F+ by -2 pi B0 dt over the interval.
                        float so, co;
                        sincosf(-2.f * 3.14159265358979323846f * b0 * op.dt, &so, &co);
                        tr = e2 * co;
                        ti = e2 * so;
                    }
                }
                const float2 E1 = dup(e1), T = dup(tr), Ti = dup(ti), nTi = dup(-ti);
#pragma unroll
                for (int k = 0; k < RP; ++k) {
                    // F+ *= (tr + i ti), F- *= (tr - i ti), Z *= e1.
                    const float2 pr = Pr[k], pi = Pi[k], mr = Mr[k], mi = Mi[k];
                    Pr[k] = fma2(nTi, pi, mul2(T, pr));
                    Pi[k] = fma2(Ti, pr, mul2(T, pi));
                    Mr[k] = fma2(Ti, mi, mul2(T, mr));
                    Mi[k] = fma2(nTi, mr, mul2(T, mi));
                    Zr[k] = mul2(Zr[k], E1);
                    Zi[k] = mul2(Zi[k], E1);
                }
                if (q == 0) Zr[0].x += 1.f - e1;
            }
            for (int s = 0; s < op_shift1(code); ++s)
                shift_complex<RP, L>(Pr, Pi, Mr, Mi, q, kill, kill_r);
            const int rf = op_rf(code);
            if (rf == RF_ROTATE) {
                float sa, ca, sp, cp;
                sincosf(op.flip * b1, &sa, &ca);
                sincosf(s_ph[i].x + b1_phase, &sp, &cp);
                const float ch = 0.5f * (1.f + ca), sh = 0.5f * (1.f - ca);
                // e^{2i phi} from e^{i phi}.
                const float c2 = cp * cp - sp * sp, s2 = 2.f * cp * sp;
                const float2 T00 = dup(ch), T22 = dup(ca);
                const float2 A_r = dup(sh * c2), A_i = dup(sh * s2), nA_i = dup(-sh * s2);
                const float2 B_r = dup(sa * sp), B_i = dup(sa * cp), nB_i = dup(-sa * cp);
                const float2 C_r = dup(-0.5f * sa * sp), C_i = dup(0.5f * sa * cp),
                             nC_i = dup(-0.5f * sa * cp);
#pragma unroll
                for (int k = 0; k < RP; ++k) {
                    const float2 pr = Pr[k], pi = Pi[k], mr = Mr[k], mi = Mi[k], zr = Zr[k],
                                 zi = Zi[k];
                    // F+ = ch F+ + A F- + B' Z with A = sh e^{2i phi},
                    //      B' = -i sa e^{i phi} = (sa sp, -sa cp).
                    Pr[k] = fma2(B_r, zr, fma2(B_i, zi, fma2(nA_i, mi, fma2(A_r, mr, mul2(T00, pr)))));
                    Pi[k] = fma2(B_r, zi, fma2(nB_i, zr, fma2(A_i, mr, fma2(A_r, mi, mul2(T00, pi)))));
                    // F- = conj(A) F+ + ch F- + i sa e^{-i phi} Z = (sa sp, sa cp).
                    Mr[k] = fma2(B_r, zr, fma2(nB_i, zi, fma2(A_i, pi, fma2(A_r, pr, mul2(T00, mr)))));
                    Mi[k] = fma2(B_r, zi, fma2(B_i, zr, fma2(nA_i, pr, fma2(A_r, pi, mul2(T00, mi)))));
                    // Z = -i sa/2 e^{-i phi} F+ + i sa/2 e^{i phi} F- + ca Z, with
                    // -i sa/2 e^{-i phi} = (-sa/2 sp, -sa/2 cp) = (C_r, -C_i) and
                    // i sa/2 e^{i phi} = (-sa/2 sp, sa/2 cp) = (C_r, C_i).
                    Zr[k] = fma2(C_r, mr, fma2(nC_i, mi, fma2(C_r, pr, fma2(C_i, pi, mul2(T22, zr)))));
                    Zi[k] = fma2(C_r, mi, fma2(C_i, mr, fma2(C_r, pi, fma2(nC_i, pr, mul2(T22, zi)))));
                }
            } else if (rf == RF_INVERT) {
                const float2 f = dup(-eff);
#pragma unroll
                for (int k = 0; k < RP; ++k) {
                    Zr[k] = mul2(Zr[k], f);
                    Zi[k] = mul2(Zi[k], f);
                }
            }
            for (int s = 0; s < op_shift2(code); ++s)
                shift_complex<RP, L>(Pr, Pi, Mr, Mi, q, kill, kill_r);
            if (code & OP_SPOIL1) {
#pragma unroll
                for (int k = 0; k < RP; ++k) Pr[k] = Pi[k] = Mr[k] = Mi[k] = dup(0.f);
            }
            if ((code & OP_RECORD) && q == 0 && active) {
                // m0 F+[0] demodulated by the receiver phase.
                float sr, cr;
                sincosf(s_ph[i].y, &sr, &cr);
                const float vr = m0 * Pr[0].x, vi = m0 * Pi[0].x;
                put(a.layout, a.out_a, a.out_b, out_base + op.record, vr * cr + vi * sr,
                    vi * cr - vr * sr);
            }
            for (int s = 0; s < op_shift3(code); ++s)
                shift_complex<RP, L>(Pr, Pi, Mr, Mi, q, kill, kill_r);
            if (code & OP_SPOIL2) {
#pragma unroll
                for (int k = 0; k < RP; ++k) Pr[k] = Pi[k] = Mr[k] = Mi[k] = dup(0.f);
            }
        }
    }
}

struct ComplexEntry {
    int orders_per_lane;
    int lanes_per_voxel;
    void (*launch)(const ComplexArgs&, dim3, dim3, cudaStream_t);
};

template <int RP, int L>
void launch_complex(const ComplexArgs& a, dim3 grid, dim3 block, cudaStream_t s) {
    epg_complex_kernel<RP, L><<<grid, block, 0, s>>>(a);
}

#define TSG_COMPLEX_ENTRY(R, L) {R, L, &launch_complex<(R) / 2, L>}

const ComplexEntry kComplex[] = {
    TSG_COMPLEX_ENTRY(10, 1), TSG_COMPLEX_ENTRY(6, 2),  TSG_COMPLEX_ENTRY(4, 4),
    TSG_COMPLEX_ENTRY(4, 5),  TSG_COMPLEX_ENTRY(2, 10), TSG_COMPLEX_ENTRY(4, 8),
    TSG_COMPLEX_ENTRY(4, 16), TSG_COMPLEX_ENTRY(4, 32),
};

}  // namespace

}  // namespace tsg

using namespace tsg;

extern "C" int tsg_epg_forward_complex(const tsg_program* program, const tsg_tissue* tissue,
                                       const tsg_offaxis* offaxis, int64_t atom_count,
                                       int64_t state_count, int layout, float* out_a,
                                       float* out_b, const tsg_launch* launch_shape,
                                       void* stream) {
    if (!program) return fail(TSG_ERR_ARGUMENT, "null program");
    if (!tissue || (atom_count > 0 && (!tissue->t1_ms || !tissue->t2_ms)))
        return fail(TSG_ERR_ARGUMENT, "t1 and t2 are required");
    if (atom_count < 0 || state_count < 1) return fail(TSG_ERR_ARGUMENT, "invalid EPG buffer dimensions");
    if (state_count > 256) return fail(TSG_ERR_CAPACITY, "more than 256 states");
    if (!program->d_phase && program->host.ops > 0)
        return fail(TSG_ERR_ARGUMENT, "the complex path needs a program built with event phases");
    if (layout != TSG_LAYOUT_PLANES && layout != TSG_LAYOUT_COMPLEX_IJ && layout != TSG_LAYOUT_COMPLEX)
        return fail(TSG_ERR_ARGUMENT, "unknown output layout");
    if (layout == TSG_LAYOUT_PLANES ? (!out_a || !out_b) : !out_a)
        return fail(TSG_ERR_ARGUMENT, "null output buffer");
    if (atom_count == 0 || program->host.ops == 0) return TSG_OK;
    if (program->host.trains > 65535) return fail(TSG_ERR_CAPACITY, "more than 65535 trains");
    const int want_l = launch_shape ? launch_shape->lanes_per_voxel : 0;
    const int want_r = launch_shape ? launch_shape->orders_per_lane : 0;
    const int warps = (launch_shape && launch_shape->warps_per_block > 0) ? launch_shape->warps_per_block : 4;
    if (warps < 1 || warps > 8) return fail(TSG_ERR_ARGUMENT, "warps_per_block must be 1..8");
    // Without a request: the entry with the fewest idle order slots per warp,
    // one voxel per lane first.
    const ComplexEntry* best = nullptr;
    double best_waste = 1e30;
    for (const ComplexEntry& e : kComplex) {
        const int padded = e.orders_per_lane * e.lanes_per_voxel;
        if (padded < state_count) continue;
        if (want_l > 0 && e.lanes_per_voxel != want_l) continue;
        if (want_r > 0 && e.orders_per_lane != want_r) continue;
        const int vpw = 32 / e.lanes_per_voxel;
        const double waste = double(32 * e.orders_per_lane) / double(vpw * state_count) *
                             (1.0 + 0.05 * (e.lanes_per_voxel - 1));
        if (waste < best_waste) {
            best_waste = waste;
            best = &e;
        }
    }
    if (!best) return fail(TSG_ERR_UNSUPPORTED, "no complex kernel for this state count / launch shape");
    ComplexArgs a{};
    a.ops = program->d_ops;
    a.phase = program->d_phase;
    a.n_ops = int(program->host.ops);
    a.atoms = atom_count;
    a.states = int(state_count);
    a.outputs = int(program->host.outputs);
    a.t1 = tissue->t1_ms;
    a.t2 = tissue->t2_ms;
    a.m0 = tissue->m0;
    a.b1 = tissue->b1;
    a.inv = tissue->inversion;
    a.b1_phase = offaxis ? offaxis->b1_phase_rad : nullptr;
    a.b0 = offaxis ? offaxis->b0_hz : nullptr;
    a.layout = layout;
    a.out_a = out_a;
    a.out_b = out_b;
    const int vpb = warps * (32 / best->lanes_per_voxel);
    const int64_t blocks = (atom_count + vpb - 1) / vpb;
    if (blocks > 0x7fffffffLL) return fail(TSG_ERR_CAPACITY, "launch too large");
    best->launch(a, dim3(unsigned(blocks), unsigned(program->host.trains)), dim3(32 * warps),
                 static_cast<cudaStream_t>(stream));
    TSG_CUDA(cudaGetLastError());
    return TSG_OK;
}
