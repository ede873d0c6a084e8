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
#include "epg_complex.cuh"

namespace tsg {

namespace {

using namespace complex_detail;

template <int RP, int L, int TM>
__global__ void __launch_bounds__(256) epg_complex_kernel(const ComplexArgs a) {
    using TG = Tangents<TM>;
    constexpr int NT = TG::N;
    constexpr int NA = TG::NA;
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
    const float t1 = a.t1[ac], t2 = a.t2[ac];
    const float r1 = 1000.f / t1;
    const float r2 = 1000.f / t2;
    const float w1 = 1000.f / (t1 * t1), w2 = 1000.f / (t2 * t2);
    const float m0 = a.m0 ? a.m0[ac] : 1.f;
    const float b1 = a.b1 ? a.b1[ac] : 1.f;
    const float eff = a.inv ? a.inv[ac] : 1.f;
    const float b1_phase = a.b1_phase ? a.b1_phase[ac] : 0.f;
    const float b0 = a.b0 ? a.b0[ac] : 0.f;
    const bool off_axis = a.b0 != nullptr;
    const bool kill = L * R > a.states;
    const int kill_r = a.states - q * R;

    float2 Pr[RP], Pi[RP], Mr[RP], Mi[RP], Zr[RP], Zi[RP];
    float2 dPr[NA][RP], dPi[NA][RP], dMr[NA][RP], dMi[NA][RP], dZr[NA][RP], dZi[NA][RP];
#pragma unroll
    for (int k = 0; k < RP; ++k) {
        Pr[k] = Pi[k] = Mr[k] = Mi[k] = Zr[k] = Zi[k] = dup(0.f);
#pragma unroll
        for (int j = 0; j < NA; ++j)
            dPr[j][k] = dPi[j][k] = dMr[j][k] = dMi[j][k] = dZr[j][k] = dZi[j][k] = dup(0.f);
    }
    if (q == 0) Zr[0].x = 1.f;

    const Op* ops = a.ops + train * a.n_ops;
    const float2* phase = a.phase + train * a.n_ops;
    const int64_t row = train * a.atoms + atom;
    const int64_t out_base = row * a.outputs;
    const int64_t jac_base = row * a.jac_cols * a.outputs;
    float last_dt = __int_as_float(0x7fffffff);
    float e1 = 1.f, tr = 1.f, ti = 0.f, k1 = 0.f, k2f = 0.f;
    // Each op's transcendentals are the same for the L lanes of a voxel:
    // lane q evaluates them for one of the next L ops (the pulse's flip and
    // phase, the receiver phase of a record) and the lanes exchange them by
    // shuffle, so each lane evaluates one op's in L.
    float my_sa = 0.f, my_ca = 1.f, my_sp = 0.f, my_cp = 1.f, my_sr = 0.f, my_cr = 1.f;
    const int first_lane = lane - q;

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
            const int g = i % L;
            if constexpr (L > 1) {
                if (g == 0) {
                    const int j = i + q;
                    float sa = 0.f, ca = 1.f, sp = 0.f, cp = 1.f, sr = 0.f, cr = 1.f;
                    if (j < count) {
                        const uint32_t cj = s_ops[j].code;
                        if (op_rf(cj) == RF_ROTATE) {
                            sincosf(s_ops[j].flip * b1, &sa, &ca);
                            sincosf(s_ph[j].x + b1_phase, &sp, &cp);
                        }
                        if (cj & OP_RECORD) sincosf(s_ph[j].y, &sr, &cr);
                    }
                    my_sa = sa;
                    my_ca = ca;
                    my_sp = sp;
                    my_cp = cp;
                    my_sr = sr;
                    my_cr = cr;
                }
            }
            if (code & OP_RELAX) {
                if (op.dt != last_dt) {
                    last_dt = op.dt;
                    e1 = expf(-r1 * op.dt);
                    const float e2 = expf(-r2 * op.dt);
                    // d e1 / dT1 and (d e2 / dT2) / e2.
                    k1 = e1 * (op.dt * w1);
                    k2f = op.dt * w2;
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
                    const float2 pr = Pr[k], pi = Pi[k], mr = Mr[k], mi = Mi[k], zr = Zr[k],
                                 zi = Zi[k];
#pragma unroll
                    for (int j = 0; j < NT; ++j) {
                        float2 xpr = dPr[j][k], xpi = dPi[j][k], xmr = dMr[j][k], xmi = dMi[j][k];
                        if (TG::T2 && j == TG::I_T2) {
                            // d(T F+)/dT2 = T (dF+ + k2f F+), likewise for F-.
                            const float2 K = dup(k2f);
                            xpr = fma2(K, pr, xpr);
                            xpi = fma2(K, pi, xpi);
                            xmr = fma2(K, mr, xmr);
                            xmi = fma2(K, mi, xmi);
                        }
                        dPr[j][k] = fma2(nTi, xpi, mul2(T, xpr));
                        dPi[j][k] = fma2(Ti, xpr, mul2(T, xpi));
                        dMr[j][k] = fma2(Ti, xmi, mul2(T, xmr));
                        dMi[j][k] = fma2(nTi, xmr, mul2(T, xmi));
                        if (TG::T1 && j == TG::I_T1) {
                            dZr[j][k] = fma2(E1, dZr[j][k], mul2(dup(k1), zr));
                            dZi[j][k] = fma2(E1, dZi[j][k], mul2(dup(k1), zi));
                        } else {
                            dZr[j][k] = mul2(dZr[j][k], E1);
                            dZi[j][k] = mul2(dZi[j][k], E1);
                        }
                    }
                    // F+ *= (tr + i ti), F- *= (tr - i ti), Z *= e1.
                    Pr[k] = fma2(nTi, pi, mul2(T, pr));
                    Pi[k] = fma2(Ti, pr, mul2(T, pi));
                    Mr[k] = fma2(Ti, mi, mul2(T, mr));
                    Mi[k] = fma2(nTi, mr, mul2(T, mi));
                    Zr[k] = mul2(zr, E1);
                    Zi[k] = mul2(zi, E1);
                }
                if (q == 0) {
                    Zr[0].x += 1.f - e1;
                    if constexpr (TG::T1) dZr[TG::I_T1][0].x -= k1;
                }
            }
            for (int s = 0; s < op_shift1(code); ++s) {
                shift_complex<RP, L>(Pr, Pi, Mr, Mi, q, kill, kill_r);
#pragma unroll
                for (int j = 0; j < NT; ++j)
                    shift_complex<RP, L>(dPr[j], dPi[j], dMr[j], dMi[j], q, kill, kill_r);
            }
            const int rf = op_rf(code);
            if (rf == RF_ROTATE) {
                float sa, ca, sp, cp;
                if constexpr (L > 1) {
                    const int src = first_lane + g;
                    sa = __shfl_sync(0xffffffffu, my_sa, src);
                    ca = __shfl_sync(0xffffffffu, my_ca, src);
                    sp = __shfl_sync(0xffffffffu, my_sp, src);
                    cp = __shfl_sync(0xffffffffu, my_cp, src);
                } else {
                    sincosf(op.flip * b1, &sa, &ca);
                    sincosf(s_ph[i].x + b1_phase, &sp, &cp);
                }
                // e^{2i phi} from e^{i phi}.
                const float c2 = cp * cp - sp * sp, s2 = 2.f * cp * sp;
                const Pulse u = pulse_of(0.5f * (1.f + ca), ca, 0.5f * (1.f - ca), sa, 0.5f * sa,
                                         c2, s2, cp, sp);
                Pulse du{};
                if constexpr (TG::B1)
                    du = pulse_of(-0.5f * sa, -sa, 0.5f * sa, ca, 0.5f * ca, c2, s2, cp, sp);
                const float2 at = dup(op.flip);  // d alpha / d B1
#pragma unroll
                for (int k = 0; k < RP; ++k) {
                    const float2 pr = Pr[k], pi = Pi[k], mr = Mr[k], mi = Mi[k], zr = Zr[k],
                                 zi = Zi[k];
#pragma unroll
                    for (int j = 0; j < NT; ++j) {
                        float2 opr, opi, omr, omi, ozr, ozi;
                        apply(u, dPr[j][k], dPi[j][k], dMr[j][k], dMi[j][k], dZr[j][k], dZi[j][k],
                              opr, opi, omr, omi, ozr, ozi);
                        if (TG::B1 && j == TG::I_B1) {
                            float2 vpr, vpi, vmr, vmi, vzr, vzi;
                            apply(du, pr, pi, mr, mi, zr, zi, vpr, vpi, vmr, vmi, vzr, vzi);
                            opr = fma2(at, vpr, opr);
                            opi = fma2(at, vpi, opi);
                            omr = fma2(at, vmr, omr);
                            omi = fma2(at, vmi, omi);
                            ozr = fma2(at, vzr, ozr);
                            ozi = fma2(at, vzi, ozi);
                        }
                        dPr[j][k] = opr;
                        dPi[j][k] = opi;
                        dMr[j][k] = omr;
                        dMi[j][k] = omi;
                        dZr[j][k] = ozr;
                        dZi[j][k] = ozi;
                    }
                    apply(u, pr, pi, mr, mi, zr, zi, Pr[k], Pi[k], Mr[k], Mi[k], Zr[k], Zi[k]);
                }
            } else if (rf == RF_INVERT) {
                const float2 f = dup(-eff);
#pragma unroll
                for (int k = 0; k < RP; ++k) {
                    Zr[k] = mul2(Zr[k], f);
                    Zi[k] = mul2(Zi[k], f);
#pragma unroll
                    for (int j = 0; j < NT; ++j) {
                        dZr[j][k] = mul2(dZr[j][k], f);
                        dZi[j][k] = mul2(dZi[j][k], f);
                    }
                }
            }
            for (int s = 0; s < op_shift2(code); ++s) {
                shift_complex<RP, L>(Pr, Pi, Mr, Mi, q, kill, kill_r);
#pragma unroll
                for (int j = 0; j < NT; ++j)
                    shift_complex<RP, L>(dPr[j], dPi[j], dMr[j], dMi[j], q, kill, kill_r);
            }
            if (code & OP_SPOIL1) {
#pragma unroll
                for (int k = 0; k < RP; ++k) {
                    Pr[k] = Pi[k] = Mr[k] = Mi[k] = dup(0.f);
#pragma unroll
                    for (int j = 0; j < NT; ++j) dPr[j][k] = dPi[j][k] = dMr[j][k] = dMi[j][k] = dup(0.f);
                }
            }
            float sr = 0.f, cr = 1.f;
            if (code & OP_RECORD) {
                if constexpr (L > 1) {
                    sr = __shfl_sync(0xffffffffu, my_sr, first_lane + g);
                    cr = __shfl_sync(0xffffffffu, my_cr, first_lane + g);
                } else {
                    sincosf(s_ph[i].y, &sr, &cr);
                }
            }
            if ((code & OP_RECORD) && q == 0 && active) {
                // m0 F+[0] demodulated by the receiver phase, and its columns.
                const int rec = op.record;
                auto demod = [&](float xr, float xi, float& yr, float& yi) {
                    yr = xr * cr + xi * sr;
                    yi = xi * cr - xr * sr;
                };
                float yr, yi;
                demod(Pr[0].x, Pi[0].x, yr, yi);
                if (a.out_a) put(a.layout, a.out_a, a.out_b, out_base + rec, m0 * yr, m0 * yi);
                if constexpr (NT > 0) {
                    if (a.col_m0 >= 0)
                        put(a.layout, a.jac_a, a.jac_b, jac_base + a.col_m0 * a.outputs + rec, yr, yi);
                    const int cols[3] = {a.col_t1, a.col_t2, a.col_b1};
                    const int idx[3] = {TG::I_T1, TG::I_T2, TG::I_B1};
                    const bool has[3] = {bool(TG::T1), bool(TG::T2), bool(TG::B1)};
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        if (!has[c] || cols[c] < 0) continue;
                        float dr, di;
                        demod(dPr[idx[c]][0].x, dPi[idx[c]][0].x, dr, di);
                        put(a.layout, a.jac_a, a.jac_b, jac_base + cols[c] * a.outputs + rec,
                            m0 * dr, m0 * di);
                    }
                }
            }
            for (int s = 0; s < op_shift3(code); ++s) {
                shift_complex<RP, L>(Pr, Pi, Mr, Mi, q, kill, kill_r);
#pragma unroll
                for (int j = 0; j < NT; ++j)
                    shift_complex<RP, L>(dPr[j], dPi[j], dMr[j], dMi[j], q, kill, kill_r);
            }
            if (code & OP_SPOIL2) {
#pragma unroll
                for (int k = 0; k < RP; ++k) {
                    Pr[k] = Pi[k] = Mr[k] = Mi[k] = dup(0.f);
#pragma unroll
                    for (int j = 0; j < NT; ++j) dPr[j][k] = dPi[j][k] = dMr[j][k] = dMi[j][k] = dup(0.f);
                }
            }
        }
    }
}

struct ComplexEntry {
    int orders_per_lane;
    int lanes_per_voxel;
    int tangents;
    void (*launch)(const ComplexArgs&, dim3, dim3, cudaStream_t);
};

template <int RP, int L, int TM>
void launch_complex(const ComplexArgs& a, dim3 grid, dim3 block, cudaStream_t s) {
    epg_complex_kernel<RP, L, TM><<<grid, block, 0, s>>>(a);
}

#define TSG_COMPLEX_ENTRY(R, L, TM) {R, L, TM, &launch_complex<(R) / 2, L, TM>}

const ComplexEntry kComplex[] = {
    TSG_COMPLEX_ENTRY(10, 1, 0), TSG_COMPLEX_ENTRY(6, 2, 0),  TSG_COMPLEX_ENTRY(4, 4, 0),
    TSG_COMPLEX_ENTRY(4, 5, 0),  TSG_COMPLEX_ENTRY(2, 10, 0), TSG_COMPLEX_ENTRY(4, 8, 0),
    TSG_COMPLEX_ENTRY(4, 16, 0), TSG_COMPLEX_ENTRY(4, 32, 0),
    // Tangent kernels: T1|T2 and T1|T2|B1.
    TSG_COMPLEX_ENTRY(2, 5, 3),  TSG_COMPLEX_ENTRY(4, 4, 3),  TSG_COMPLEX_ENTRY(4, 5, 3),
    TSG_COMPLEX_ENTRY(2, 10, 3), TSG_COMPLEX_ENTRY(4, 8, 3),  TSG_COMPLEX_ENTRY(4, 16, 3),
    TSG_COMPLEX_ENTRY(4, 32, 3), TSG_COMPLEX_ENTRY(2, 5, 7),  TSG_COMPLEX_ENTRY(4, 4, 7),
    TSG_COMPLEX_ENTRY(4, 5, 7),  TSG_COMPLEX_ENTRY(2, 10, 7), TSG_COMPLEX_ENTRY(4, 8, 7),
    TSG_COMPLEX_ENTRY(4, 16, 7), TSG_COMPLEX_ENTRY(4, 32, 7),
};

// The entry of a tangent family for a state count and launch request.
const ComplexEntry* choose_complex(int tangents, int64_t states, const tsg_launch* want) {
    const int want_l = want ? want->lanes_per_voxel : 0;
    const int want_r = want ? want->orders_per_lane : 0;
    const ComplexEntry* best = nullptr;
    double best_waste = 1e30;
    for (const ComplexEntry& e : kComplex) {
        if (e.tangents != tangents) continue;
        const int padded = e.orders_per_lane * e.lanes_per_voxel;
        if (padded < states) continue;
        if (want_l > 0 && e.lanes_per_voxel != want_l) continue;
        if (want_r > 0 && e.orders_per_lane != want_r) continue;
        const int vpw = 32 / e.lanes_per_voxel;
        // Fewest idle order slots per warp, fewer lanes per voxel first.
        const double waste = double(32 * e.orders_per_lane) / double(vpw * states) *
                             (1.0 + 0.05 * (e.lanes_per_voxel - 1));
        if (waste < best_waste) {
            best_waste = waste;
            best = &e;
        }
    }
    return best;
}

int launch_complex_sweep(const tsg_program* program, const ComplexArgs& base, int tangents,
                         int64_t atom_count, int64_t state_count, const tsg_launch* launch_shape,
                         cudaStream_t stream) {
    const int warps = (launch_shape && launch_shape->warps_per_block > 0) ? launch_shape->warps_per_block : 4;
    if (warps < 1 || warps > 8) return fail(TSG_ERR_ARGUMENT, "warps_per_block must be 1..8");
    const ComplexEntry* best = choose_complex(tangents, state_count, launch_shape);
    if (!best) return fail(TSG_ERR_UNSUPPORTED, "no complex kernel for this state count / launch shape");
    const int vpb = warps * (32 / best->lanes_per_voxel);
    const int64_t blocks = (atom_count + vpb - 1) / vpb;
    if (blocks > 0x7fffffffLL) return fail(TSG_ERR_CAPACITY, "launch too large");
    best->launch(base, dim3(unsigned(blocks), unsigned(program->host.trains)), dim3(32 * warps),
                 stream);
    TSG_CUDA(cudaGetLastError());
    return TSG_OK;
}

int complex_common(const tsg_program* program, const tsg_tissue* tissue, int64_t atom_count,
                   int64_t state_count, int layout) {
    if (!program) return fail(TSG_ERR_ARGUMENT, "null program");
    if (!tissue || (atom_count > 0 && (!tissue->t1_ms || !tissue->t2_ms)))
        return fail(TSG_ERR_ARGUMENT, "t1 and t2 are required");
    if (atom_count < 0 || state_count < 1) return fail(TSG_ERR_ARGUMENT, "invalid EPG buffer dimensions");
    if (state_count > 256) return fail(TSG_ERR_CAPACITY, "more than 256 states");
    if (!program->d_phase && program->host.ops > 0)
        return fail(TSG_ERR_ARGUMENT, "the complex path needs a program built with event phases");
    if (layout != TSG_LAYOUT_PLANES && layout != TSG_LAYOUT_COMPLEX_IJ && layout != TSG_LAYOUT_COMPLEX)
        return fail(TSG_ERR_ARGUMENT, "unknown output layout");
    if (program->host.trains > 65535) return fail(TSG_ERR_CAPACITY, "more than 65535 trains");
    return TSG_OK;
}

ComplexArgs complex_args(const tsg_program* program, const tsg_tissue* tissue,
                         const tsg_offaxis* offaxis, int64_t atom_count, int64_t state_count,
                         int layout) {
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
    a.col_t1 = a.col_t2 = a.col_b1 = a.col_m0 = -1;
    return a;
}

}  // namespace

}  // namespace tsg

using namespace tsg;

extern "C" int tsg_epg_forward_complex(const tsg_program* program, const tsg_tissue* tissue,
                                       const tsg_offaxis* offaxis, int64_t atom_count,
                                       int64_t state_count, int layout, float* out_a,
                                       float* out_b, const tsg_launch* launch_shape,
                                       void* stream) {
    int rc = complex_common(program, tissue, atom_count, state_count, layout);
    if (rc) return rc;
    if (layout == TSG_LAYOUT_PLANES ? (!out_a || !out_b) : !out_a)
        return fail(TSG_ERR_ARGUMENT, "null output buffer");
    if (atom_count == 0 || program->host.ops == 0) return TSG_OK;
    ComplexArgs a = complex_args(program, tissue, offaxis, atom_count, state_count, layout);
    a.out_a = out_a;
    a.out_b = out_b;
    return launch_complex_sweep(program, a, 0, atom_count, state_count, launch_shape,
                                static_cast<cudaStream_t>(stream));
}

extern "C" int tsg_epg_forward_tangents_complex(const tsg_program* program, const tsg_tissue* tissue,
                                                const tsg_offaxis* offaxis, int64_t atom_count,
                                                int64_t state_count, unsigned tangent_mask,
                                                const int32_t* columns, int32_t column_count,
                                                int layout, float* sig_a, float* sig_b,
                                                float* jac_a, float* jac_b,
                                                const tsg_launch* launch_shape, void* stream) {
    int rc = complex_common(program, tissue, atom_count, state_count, layout);
    if (rc) return rc;
    if (!columns || column_count < 0) return fail(TSG_ERR_ARGUMENT, "null column map");
    if (tangent_mask & ~unsigned(TSG_TANGENT_T1 | TSG_TANGENT_T2 | TSG_TANGENT_B1))
        return fail(TSG_ERR_UNSUPPORTED, "the complex path carries T1, T2 and B1 tangents");
    if (columns[3] >= 0) return fail(TSG_ERR_UNSUPPORTED, "no inversion-efficiency column on the complex path");
    const unsigned bits[3] = {TSG_TANGENT_T1, TSG_TANGENT_T2, TSG_TANGENT_B1};
    for (int i = 0; i < 5; ++i)
        if (columns[i] >= column_count) return fail(TSG_ERR_ARGUMENT, "column out of range");
    for (int i = 0; i < 3; ++i)
        if (columns[i] >= 0 && !(tangent_mask & bits[i]))
            return fail(TSG_ERR_ARGUMENT, "column given for a tangent not in the mask");
    if (layout == TSG_LAYOUT_PLANES ? (!jac_a || !jac_b) : !jac_a)
        return fail(TSG_ERR_ARGUMENT, "null Jacobian buffer");
    if (atom_count == 0 || program->host.ops == 0) return TSG_OK;
    ComplexArgs a = complex_args(program, tissue, offaxis, atom_count, state_count, layout);
    a.out_a = sig_a;
    a.out_b = sig_b;
    if (layout == TSG_LAYOUT_PLANES && (!sig_a || !sig_b)) a.out_a = a.out_b = nullptr;
    a.jac_a = jac_a;
    a.jac_b = jac_b;
    a.jac_cols = column_count;
    a.col_t1 = columns[0];
    a.col_t2 = columns[1];
    a.col_b1 = columns[2];
    a.col_m0 = columns[4];
    const int family = (tangent_mask & TSG_TANGENT_B1) ? 7 : 3;
    return launch_complex_sweep(program, a, family, atom_count, state_count, launch_shape,
                                static_cast<cudaStream_t>(stream));
}
