// One general forward-mode direction on the complex path: the reference's
// complex simulate_jvp_range (src/torchsim/_epg_cpu.cpp:2470-3005) for one
// pool and instant RF, along any combination of per-voxel directions (T1, T2,
// M0, B1, inversion efficiency, B1phase, B0) and per-event directions
// (duration, flip, phase -- a pulse's phase, or an ADC's receiver phase). It
// writes the tangent of the recorded sample only, as the reference's does.
//
// The tangent system (dF+, dF-, dZ) is carried beside the state through
// every micro-step, with the same thread mapping as the complex forward
// (orders over L lanes, pairs of orders per register):
//   relax   F+ *= T, F- *= conj(T), Z *= e1 (+ 1 - e1 on Z0), with
//           T = e2 e^{-2 pi i B0 dt}; dT = T (de2/e2 - 2 pi i d(B0 dt)),
//           de1 and de2 from dT1, dT2 and d dt;
//   pulse   X' = U X, dX' = U dX + (dalpha U_alpha + dphi U_phi) X, with
//           alpha = flip B1, phi = RF phase + B1phase;
//   invert  Z' = -eff Z, dZ' = -eff dZ - deff Z;
//   record  y = m0 F+[0] e^{-i psi}: dy = (dm0 F + m0 dF - i dpsi m0 F) e^{-i psi}.
#include "epg_complex.cuh"

namespace tsg {

namespace {

using namespace complex_detail;

// Per op of the program: (d dt, d flip, d pulse phase, d receiver phase).
__global__ void gather_complex_directions(const OpSource* src, int64_t n_ops, int64_t trains,
                                          int64_t events, const float* ddur, const float* dflip,
                                          const float* dphase, float4* out) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n_ops * trains) return;
    const int64_t t = i / n_ops;
    const OpSource s = src[i];
    float4 d = make_float4(0.f, 0.f, 0.f, 0.f);
    if (ddur && s.dt_event >= 0) d.x = ddur[t * events + s.dt_event];
    if (dflip && s.rf_event >= 0) d.y = dflip[t * events + s.rf_event];
    if (dphase && s.rf_event >= 0) d.z = dphase[t * events + s.rf_event];
    if (dphase && s.rec_event >= 0) d.w = dphase[t * events + s.rec_event];
    out[i] = d;
}

__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }

struct ComplexDirection {
    const float* t1;
    const float* t2;
    const float* m0;
    const float* b1;
    const float* inv;
    const float* b1_phase;
    const float* b0;
    const float4* op_dir;  // [train][ops]
};

__device__ __forceinline__ void cmul(float2 ar, float2 ai, float br, float bi, float2& outr,
                                     float2& outi) {
    // (ar + i ai) * (br + i bi), pairs of orders at once.
    outr = fma2(dup(-bi), ai, mul2(dup(br), ar));
    outi = fma2(dup(bi), ar, mul2(dup(br), ai));
}

template <int RP, int L>
__global__ void __launch_bounds__(256)
    epg_complex_tangent_kernel(const ComplexArgs a, const ComplexDirection d) {
    constexpr int R = 2 * RP;
    constexpr int VPW = 32 / L;
    __shared__ Op s_ops[kComplexOpChunk];
    __shared__ float2 s_ph[kComplexOpChunk];
    __shared__ float4 s_dir[kComplexOpChunk];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int q = lane % L;
    const int slot = lane / L;
    const int64_t atom = (int64_t(blockIdx.x) * (blockDim.x >> 5) + warp) * VPW + slot;
    const int64_t train = blockIdx.y;
    const bool active = slot < VPW && atom < a.atoms;
    const int64_t ac = active ? atom : 0;
    const float t1 = a.t1[ac], t2 = a.t2[ac];
    const float r1 = 1000.f / t1, r2 = 1000.f / t2;
    const float m0 = a.m0 ? a.m0[ac] : 1.f;
    const float b1 = a.b1 ? a.b1[ac] : 1.f;
    const float eff = a.inv ? a.inv[ac] : 1.f;
    const float b1_phase = a.b1_phase ? a.b1_phase[ac] : 0.f;
    const float b0 = a.b0 ? a.b0[ac] : 0.f;
    const bool off_axis = a.b0 != nullptr;
    // Directions; a property the run does not declare carries none.
    const float g_t1 = d.t1 ? d.t1[ac] : 0.f;
    const float g_t2 = d.t2 ? d.t2[ac] : 0.f;
    const float g_m0 = (a.m0 && d.m0) ? d.m0[ac] : 0.f;
    const float g_b1 = (a.b1 && d.b1) ? d.b1[ac] : 0.f;
    const float g_inv = (a.inv && d.inv) ? d.inv[ac] : 0.f;
    const float g_b1p = (a.b1_phase && d.b1_phase) ? d.b1_phase[ac] : 0.f;
    const float g_b0 = (off_axis && d.b0) ? d.b0[ac] : 0.f;
    const float s1 = 1000.f * g_t1 / (t1 * t1), s2 = 1000.f * g_t2 / (t2 * t2);
    const bool kill = L * R > a.states;
    const int kill_r = a.states - q * R;
    constexpr float kTwoPi = 2.f * 3.14159265358979323846f;

    float2 Pr[RP], Pi[RP], Mr[RP], Mi[RP], Zr[RP], Zi[RP];
    float2 dPr[RP], dPi[RP], dMr[RP], dMi[RP], dZr[RP], dZi[RP];
#pragma unroll
    for (int k = 0; k < RP; ++k)
        Pr[k] = Pi[k] = Mr[k] = Mi[k] = Zr[k] = Zi[k] = dPr[k] = dPi[k] = dMr[k] = dMi[k] =
            dZr[k] = dZi[k] = dup(0.f);
    if (q == 0) Zr[0].x = 1.f;

    const Op* ops = a.ops + train * a.n_ops;
    const float2* phase = a.phase + train * a.n_ops;
    const float4* dirs = d.op_dir + train * a.n_ops;
    const int64_t out_base = (train * a.atoms + atom) * a.outputs;

    for (int base = 0; base < a.n_ops; base += kComplexOpChunk) {
        const int count = min(kComplexOpChunk, a.n_ops - base);
        __syncthreads();
        for (int i = threadIdx.x; i < count; i += blockDim.x) {
            s_ops[i] = ops[base + i];
            s_ph[i] = phase[base + i];
            s_dir[i] = dirs[base + i];
        }
        __syncthreads();
        for (int i = 0; i < count; ++i) {
            const Op op = s_ops[i];
            const float4 od = s_dir[i];
            const uint32_t code = op.code;
            if (code & OP_RELAX) {
                const float dt = op.dt, ddt = od.x;
                const float e1 = expf(-r1 * dt), e2 = expf(-r2 * dt);
                const float e1t = e1 * (dt * s1 - r1 * ddt);
                const float e2t = e2 * (dt * s2 - r2 * ddt);
                float so = 0.f, co = 1.f, at = 0.f;
                if (off_axis) {
                    sincosf(-kTwoPi * b0 * dt, &so, &co);
                    at = -kTwoPi * (g_b0 * dt + b0 * ddt);
                }
                // T = e2 e^{i angle}; dT = e2t e^{i angle} + e2 i at e^{i angle}.
                const float tr = e2 * co, ti = e2 * so;
                const float dtr = e2t * co - e2 * at * so, dti = e2t * so + e2 * at * co;
#pragma unroll
                for (int k = 0; k < RP; ++k) {
                    float2 ar, ai, br, bi;
                    // F+: T dP + dT P.
                    cmul(dPr[k], dPi[k], tr, ti, ar, ai);
                    cmul(Pr[k], Pi[k], dtr, dti, br, bi);
                    dPr[k] = add2(ar, br);
                    dPi[k] = add2(ai, bi);
                    cmul(Pr[k], Pi[k], tr, ti, Pr[k], Pi[k]);
                    // F-: conj(T) dM + conj(dT) M.
                    cmul(dMr[k], dMi[k], tr, -ti, ar, ai);
                    cmul(Mr[k], Mi[k], dtr, -dti, br, bi);
                    dMr[k] = add2(ar, br);
                    dMi[k] = add2(ai, bi);
                    cmul(Mr[k], Mi[k], tr, -ti, Mr[k], Mi[k]);
                    // Z: e1 dZ + de1 Z.
                    dZr[k] = fma2(dup(e1t), Zr[k], mul2(dup(e1), dZr[k]));
                    dZi[k] = fma2(dup(e1t), Zi[k], mul2(dup(e1), dZi[k]));
                    Zr[k] = mul2(Zr[k], dup(e1));
                    Zi[k] = mul2(Zi[k], dup(e1));
                }
                if (q == 0) {
                    Zr[0].x += 1.f - e1;
                    dZr[0].x -= e1t;
                }
            }
            for (int s = 0; s < op_shift1(code); ++s) {
                shift_complex<RP, L>(Pr, Pi, Mr, Mi, q, kill, kill_r);
                shift_complex<RP, L>(dPr, dPi, dMr, dMi, q, kill, kill_r);
            }
            const int rf = op_rf(code);
            if (rf == RF_ROTATE) {
                float sa, ca, sp, cp;
                sincosf(op.flip * b1, &sa, &ca);
                sincosf(s_ph[i].x + b1_phase, &sp, &cp);
                const float c2 = cp * cp - sp * sp, s2p = 2.f * cp * sp;
                const Pulse u = pulse_of(0.5f * (1.f + ca), ca, 0.5f * (1.f - ca), sa, 0.5f * sa,
                                         c2, s2p, cp, sp);
                const float da = od.y * b1 + op.flip * g_b1;  // d alpha
                const float dp = od.z + g_b1p;                 // d phi
                // dU = da U_alpha + dp U_phi, entry by entry.
                const Pulse du = pulse_raw(
                    da * (-0.5f * sa), da * (-sa),
                    da * (0.5f * sa * c2) + dp * (-(1.f - ca) * s2p),
                    da * (0.5f * sa * s2p) + dp * ((1.f - ca) * c2),
                    da * (ca * sp) + dp * (sa * cp), da * (ca * cp) + dp * (-sa * sp),
                    da * (-0.5f * ca * sp) + dp * (-0.5f * sa * cp),
                    da * (0.5f * ca * cp) + dp * (-0.5f * sa * sp));
#pragma unroll
                for (int k = 0; k < RP; ++k) {
                    float2 opr, opi, omr, omi, ozr, ozi, vpr, vpi, vmr, vmi, vzr, vzi;
                    apply(u, dPr[k], dPi[k], dMr[k], dMi[k], dZr[k], dZi[k], opr, opi, omr, omi,
                          ozr, ozi);
                    apply(du, Pr[k], Pi[k], Mr[k], Mi[k], Zr[k], Zi[k], vpr, vpi, vmr, vmi, vzr,
                          vzi);
                    dPr[k] = add2(opr, vpr);
                    dPi[k] = add2(opi, vpi);
                    dMr[k] = add2(omr, vmr);
                    dMi[k] = add2(omi, vmi);
                    dZr[k] = add2(ozr, vzr);
                    dZi[k] = add2(ozi, vzi);
                    apply(u, Pr[k], Pi[k], Mr[k], Mi[k], Zr[k], Zi[k], Pr[k], Pi[k], Mr[k], Mi[k],
                          Zr[k], Zi[k]);
                }
            } else if (rf == RF_INVERT) {
                const float2 f = dup(-eff), g = dup(-g_inv);
#pragma unroll
                for (int k = 0; k < RP; ++k) {
                    dZr[k] = fma2(g, Zr[k], mul2(f, dZr[k]));
                    dZi[k] = fma2(g, Zi[k], mul2(f, dZi[k]));
                    Zr[k] = mul2(Zr[k], f);
                    Zi[k] = mul2(Zi[k], f);
                }
            }
            for (int s = 0; s < op_shift2(code); ++s) {
                shift_complex<RP, L>(Pr, Pi, Mr, Mi, q, kill, kill_r);
                shift_complex<RP, L>(dPr, dPi, dMr, dMi, q, kill, kill_r);
            }
            if (code & OP_SPOIL1) {
#pragma unroll
                for (int k = 0; k < RP; ++k)
                    Pr[k] = Pi[k] = Mr[k] = Mi[k] = dPr[k] = dPi[k] = dMr[k] = dMi[k] = dup(0.f);
            }
            if ((code & OP_RECORD) && q == 0 && active) {
                float sr, cr;
                sincosf(s_ph[i].y, &sr, &cr);
                // x e^{-i psi} for x = dm0 F + m0 dF, then - i dpsi m0 F e^{-i psi}.
                const float fr = Pr[0].x, fi = Pi[0].x;
                const float xr = g_m0 * fr + m0 * dPr[0].x, xi = g_m0 * fi + m0 * dPi[0].x;
                const float yr = fr * cr + fi * sr, yi = fi * cr - fr * sr;
                const float dpsi = od.w;
                const float tr_ = (xr * cr + xi * sr) + dpsi * m0 * yi;
                const float ti_ = (xi * cr - xr * sr) - dpsi * m0 * yr;
                put(a.layout, a.jac_a, a.jac_b, out_base + op.record, tr_, ti_);
            }
            for (int s = 0; s < op_shift3(code); ++s) {
                shift_complex<RP, L>(Pr, Pi, Mr, Mi, q, kill, kill_r);
                shift_complex<RP, L>(dPr, dPi, dMr, dMi, q, kill, kill_r);
            }
            if (code & OP_SPOIL2) {
#pragma unroll
                for (int k = 0; k < RP; ++k)
                    Pr[k] = Pi[k] = Mr[k] = Mi[k] = dPr[k] = dPi[k] = dMr[k] = dMi[k] = dup(0.f);
            }
        }
    }
}

struct TangentEntry {
    int orders_per_lane;
    int lanes_per_voxel;
    void (*launch)(const ComplexArgs&, const ComplexDirection&, dim3, dim3, cudaStream_t);
};

template <int RP, int L>
void launch_tangent(const ComplexArgs& a, const ComplexDirection& d, dim3 grid, dim3 block,
                    cudaStream_t s) {
    epg_complex_tangent_kernel<RP, L><<<grid, block, 0, s>>>(a, d);
}

#define TSG_TANGENT_ENTRY(R, L) {R, L, &launch_tangent<(R) / 2, L>}

const TangentEntry kTangent[] = {
    TSG_TANGENT_ENTRY(2, 5),  TSG_TANGENT_ENTRY(4, 4),  TSG_TANGENT_ENTRY(4, 5),
    TSG_TANGENT_ENTRY(2, 10), TSG_TANGENT_ENTRY(4, 8),  TSG_TANGENT_ENTRY(4, 16),
    TSG_TANGENT_ENTRY(4, 32),
};

}  // namespace

}  // namespace tsg

using namespace tsg;

extern "C" int tsg_epg_tangent_complex(const tsg_program* program, const tsg_tissue* tissue,
                                       const tsg_offaxis* offaxis, int64_t atom_count,
                                       int64_t state_count, const tsg_direction* direction,
                                       const tsg_offaxis_direction* offaxis_direction, int layout,
                                       float* out_a, float* out_b, const tsg_launch* launch_shape,
                                       void* stream) {
    if (!program) return fail(TSG_ERR_ARGUMENT, "null program");
    if (!tissue || (atom_count > 0 && (!tissue->t1_ms || !tissue->t2_ms)))
        return fail(TSG_ERR_ARGUMENT, "t1 and t2 are required");
    if (atom_count < 0 || state_count < 1) return fail(TSG_ERR_ARGUMENT, "invalid EPG buffer dimensions");
    if (state_count > 128) return fail(TSG_ERR_CAPACITY, "more than 128 states");
    if (!program->d_phase && program->host.ops > 0)
        return fail(TSG_ERR_ARGUMENT, "the complex path needs a program built with event phases");
    if (layout != TSG_LAYOUT_PLANES && layout != TSG_LAYOUT_COMPLEX_IJ && layout != TSG_LAYOUT_COMPLEX)
        return fail(TSG_ERR_ARGUMENT, "unknown output layout");
    if (layout == TSG_LAYOUT_PLANES ? (!out_a || !out_b) : !out_a)
        return fail(TSG_ERR_ARGUMENT, "null output buffer");
    if (program->host.trains > 65535) return fail(TSG_ERR_CAPACITY, "more than 65535 trains");
    if (atom_count == 0 || program->host.ops == 0) return TSG_OK;
    const int warps = (launch_shape && launch_shape->warps_per_block > 0)
                          ? launch_shape->warps_per_block : 4;
    if (warps < 1 || warps > 8) return fail(TSG_ERR_ARGUMENT, "warps_per_block must be 1..8");
    const int want_l = launch_shape ? launch_shape->lanes_per_voxel : 0;
    const int want_r = launch_shape ? launch_shape->orders_per_lane : 0;
    const TangentEntry* best = nullptr;
    double best_waste = 1e30;
    for (const TangentEntry& e : kTangent) {
        if (e.orders_per_lane * e.lanes_per_voxel < state_count) continue;
        if (want_l > 0 && e.lanes_per_voxel != want_l) continue;
        if (want_r > 0 && e.orders_per_lane != want_r) continue;
        const double waste = double(32 * e.orders_per_lane) /
                             double((32 / e.lanes_per_voxel) * state_count) *
                             (1.0 + 0.05 * (e.lanes_per_voxel - 1));
        if (waste < best_waste) {
            best_waste = waste;
            best = &e;
        }
    }
    if (!best) return fail(TSG_ERR_UNSUPPORTED, "no complex tangent kernel for this launch shape");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int64_t n = program->host.ops * program->host.trains;
    float4* dirs = nullptr;
    TSG_CUDA(cudaMallocAsync(&dirs, size_t(n) * sizeof(float4), s));
    const float* ddur = direction ? direction->duration_s : nullptr;
    const float* dflip = direction ? direction->flip_rad : nullptr;
    const float* dphase = offaxis_direction ? offaxis_direction->phase_rad : nullptr;
    gather_complex_directions<<<unsigned((n + 255) / 256), 256, 0, s>>>(
        program->d_src, program->host.ops, program->host.trains, program->host.events, ddur,
        dflip, dphase, dirs);
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
    a.jac_a = out_a;
    a.jac_b = out_b;
    ComplexDirection d{};
    if (direction) {
        d.t1 = direction->t1_ms;
        d.t2 = direction->t2_ms;
        d.m0 = direction->m0;
        d.b1 = direction->b1;
        d.inv = direction->inversion;
    }
    if (offaxis_direction) {
        d.b1_phase = offaxis_direction->b1_phase_rad;
        d.b0 = offaxis_direction->b0_hz;
    }
    d.op_dir = dirs;
    const int vpb = warps * (32 / best->lanes_per_voxel);
    const int64_t blocks = (atom_count + vpb - 1) / vpb;
    int rc = TSG_OK;
    if (blocks > 0x7fffffffLL) {
        rc = fail(TSG_ERR_CAPACITY, "launch too large");
    } else {
        best->launch(a, d, dim3(unsigned(blocks), unsigned(program->host.trains)),
                     dim3(32 * warps), s);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rc = cuda_fail(e, "complex tangent launch");
    }
    cudaFreeAsync(dirs, s);
    return rc;
}
