// C ABI of the second-order sweeps (epg_second.cuh): planning, the device
// entry points and the host-buffer drop-in for the reference's
// _epg_cpu.simulate_vjp_jvp (src/torchsim/_epg_cpu.cpp:11572-11760).
#include <algorithm>
#include <mutex>
#include <vector>

#include "epg_second.cuh"

extern "C" int tsg_program_create(const float*, const int32_t*, const float*, const uint8_t*,
                                  const int32_t*, int64_t, int64_t, int, const float*,
                                  tsg_program**);
extern "C" int tsg_program_destroy(tsg_program*);

namespace tsg {

extern const SecondEntry kSecondK1[];
extern const int kSecondK1Count;
extern const SecondEntry kSecondK2[];
extern const int kSecondK2Count;
extern const SecondEntry kSecondK3[];
extern const int kSecondK3Count;
extern const SecondEntry kSecondHotT1[];
extern const int kSecondHotT1Count;
extern const SecondEntry kSecondHotT2[];
extern const int kSecondHotT2Count;
extern const SecondEntry kSecondHotB1[];
extern const int kSecondHotB1Count;
extern const SecondEntry kSecondHotT1T2[];
extern const int kSecondHotT1T2Count;
extern const SecondEntry kSecondHotT1B1[];
extern const int kSecondHotT1B1Count;
extern const SecondEntry kSecondHotT2B1[];
extern const int kSecondHotT2B1Count;
extern const SecondEntry kSecondHotT1T2B1[];
extern const int kSecondHotT1T2B1Count;

const SecondEntry* second_table(int k, int hot, int* count) {
    if (hot == 0) {
        switch (k) {
            case 1: *count = kSecondK1Count; return kSecondK1;
            case 2: *count = kSecondK2Count; return kSecondK2;
            case 3: *count = kSecondK3Count; return kSecondK3;
            default: break;
        }
    } else {
        switch (hot) {
            case 1: *count = kSecondHotT1Count; return kSecondHotT1;
            case 2: *count = kSecondHotT2Count; return kSecondHotT2;
            case 3: *count = kSecondHotB1Count; return kSecondHotB1;
            case 1 | 2 << 2: *count = kSecondHotT1T2Count; return kSecondHotT1T2;
            case 1 | 3 << 2: *count = kSecondHotT1B1Count; return kSecondHotT1B1;
            case 2 | 3 << 2: *count = kSecondHotT2B1Count; return kSecondHotT2B1;
            case 1 | 2 << 2 | 3 << 4: *count = kSecondHotT1T2B1Count; return kSecondHotT1T2B1;
            default: break;
        }
    }
    *count = 0;
    return nullptr;
}

namespace {

// Per-op directions of each of the K directions, from their per-event
// duration and flip tangents: [K][train][ops] (d dt, d flip).
__global__ void gather_second_directions(const OpSource* src, int64_t ops, int64_t trains,
                                         int64_t events, const float* ddur, const float* dflip,
                                         float2* out) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= ops * trains) return;
    const int64_t t = i / ops;
    const OpSource s = src[i];
    float a = 0.f, b = 0.f;
    if (ddur && s.dt_event >= 0) a = ddur[t * events + s.dt_event];
    if (dflip && s.rf_event >= 0) b = dflip[t * events + s.rf_event];
    out[i] = make_float2(a, b);
}

// Sums the per-warp event partials and scatters them to the events the ops
// came from (adding): curvature into curve_*, with two pairs also the values
// into value_*. One block per (op, train): each thread sums a fixed stride of
// warps, then a fixed tree over the threads (deterministic).
__global__ void __launch_bounds__(kEventReduceThreads)
    reduce_second_events(const float2* partial, int64_t warps, int64_t n_ops, int64_t trains,
                         int64_t events, int pairs, const OpSource* src, float* curve_flip,
                         float* curve_dt, float* value_flip, float* value_dt) {
    __shared__ float4 s_sum[kEventReduceThreads];
    const int64_t op = blockIdx.x;
    const int64_t t = blockIdx.y;
    const float2* p = partial + (t * warps * n_ops + op) * pairs;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int64_t w = threadIdx.x; w < warps; w += kEventReduceThreads) {
        const float2 x = p[w * n_ops * pairs];
        acc.x += x.x;
        acc.y += x.y;
        if (pairs == 2) {
            const float2 y = p[w * n_ops * pairs + 1];
            acc.z += y.x;
            acc.w += y.y;
        }
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
            if (curve_flip) curve_flip[t * events + s.rf_event] += c.x;
            if (value_flip) value_flip[t * events + s.rf_event] += c.z;
        }
        if (s.dt_event >= 0) {
            if (curve_dt) curve_dt[t * events + s.dt_event] += c.y;
            if (value_dt) value_dt[t * events + s.dt_event] += c.w;
        }
    }
}

// Per atom, sums the trains' tissue partials in train order and adds them
// to the gradients: curvature (5 slots), then the values of each direction.
struct TissueSlots {
    float* slot[1 + kSecondMaxK][5];
};

__global__ void reduce_second_tissue(const float* partial, int64_t atoms, int64_t trains, int nv,
                                     TissueSlots out) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= atoms) return;
    for (int j = 0; j < nv; ++j) {
        float sum = 0.f;
        for (int64_t t = 0; t < trains; ++t) sum += partial[(t * atoms + i) * nv + j];
        float* dst = out.slot[j / 5][j % 5];
        if (dst) dst[i] += sum;
    }
}

int event_pairs(int k, int hot) { return (k == 1 && hot == 0) ? 2 : 1; }
int tissue_values(int k, int hot) { return hot ? 5 : 5 * (1 + k); }

struct SecondPlan {
    const SecondEntry* entry = nullptr;
    int64_t blocks = 0;
    int64_t warps_per_train = 0;
    int64_t trajectory_bytes = 0;  // states, then (256-aligned) the records
    int64_t state_bytes = 0;
    int64_t workspace_bytes = 0;   // directions, event partials, tissue partials
    int64_t dir_bytes = 0;
    int64_t event_bytes = 0;
    size_t smem = 0;
};

// The kernel pair and buffer sizes. Without a requested shape: two orders
// per lane (the fewest registers, so the most resident warps), on the fewest
// lanes that hold the states; four orders where two would need more than 32
// lanes.
int second_plan(const tsg_program* prog, int64_t atoms, int64_t states, int k, int hot,
                const tsg_launch* want, bool event_directions, SecondPlan* plan) {
    if (!prog) return fail(TSG_ERR_ARGUMENT, "null program");
    if (atoms < 0 || states < 1) return fail(TSG_ERR_ARGUMENT, "invalid EPG buffer dimensions");
    if (k < 1 || k > kSecondMaxK) return fail(TSG_ERR_ARGUMENT, "1 to 3 directions");
    if (states > 64) return fail(TSG_ERR_CAPACITY, "second order takes at most 64 states");
    int count = 0;
    const SecondEntry* table = second_table(k, hot, &count);
    if (!table) return fail(TSG_ERR_ARGUMENT, "unknown direction set");
    const SecondEntry* best = nullptr;
    auto better = [](const SecondEntry& e, const SecondEntry* b) {
        if (!b) return true;
        if (e.orders_per_lane != b->orders_per_lane) return e.orders_per_lane < b->orders_per_lane;
        return e.lanes_per_voxel < b->lanes_per_voxel;
    };
    for (int i = 0; i < count; ++i) {
        const SecondEntry& e = table[i];
        if (want && want->lanes_per_voxel > 0 && e.lanes_per_voxel != want->lanes_per_voxel) continue;
        if (want && want->orders_per_lane > 0 && e.orders_per_lane != want->orders_per_lane) continue;
        if (e.lanes_per_voxel * e.orders_per_lane < states) continue;
        if (better(e, best)) best = &e;
    }
    if (!best) return fail(TSG_ERR_UNSUPPORTED, "no second-order kernel for this state count / launch shape");
    plan->entry = best;
    const int64_t ops = prog->host.ops;
    const int64_t trains = prog->host.trains;
    const int vpb = kSecondWarps * (32 / best->lanes_per_voxel);
    plan->blocks = (atoms + vpb - 1) / vpb;
    plan->warps_per_train = plan->blocks * kSecondWarps;
    plan->state_bytes = second_trajectory_floats(trains, atoms, ops, best->lanes_per_voxel,
                                                 best->orders_per_lane, k) * 4;
    plan->trajectory_bytes =
        align256(plan->state_bytes) + second_record_floats(trains, atoms, prog->host.outputs, k) * 4;
    plan->dir_bytes = event_directions ? align256(int64_t(k) * trains * ops * 8) : 0;
    plan->event_bytes = align256(trains * plan->warps_per_train * ops * event_pairs(k, hot) * 8);
    plan->workspace_bytes = plan->dir_bytes + plan->event_bytes +
                            trains * atoms * tissue_values(k, hot) * int64_t(sizeof(float));
    // The reverse sweep's rings (states per lane; transcendentals, seeds and
    // records per voxel slot), its ops and op directions.
    const int T = 32 * kSecondWarps;
    const int RP = best->orders_per_lane / 2;
    const size_t slots = size_t(vpb), slots4 = (slots + 3) & ~size_t(3);
    plan->smem = size_t(kSecondRing) *
                     (sizeof(float2) * size_t((k + 1) * 3 * RP) * T +
                      sizeof(float2) * size_t(k + 1) * slots + sizeof(float) * slots4) +
                 sizeof(float4) * slots * size_t(best->lanes_per_voxel) +
                 sizeof(Op) * size_t(ops) + (event_directions ? sizeof(float2) * size_t(k * ops) : 0);
    if (plan->smem > 220 * 1024)
        return fail(TSG_ERR_CAPACITY, "the program does not fit in shared memory for the reverse sweep");
    if (plan->blocks > 0x7fffffffLL || trains > 65535) return fail(TSG_ERR_CAPACITY, "launch too large");
    return TSG_OK;
}

bool has_event_directions(const tsg_direction* d, int k) {
    for (int i = 0; i < k; ++i)
        if (d[i].duration_s || d[i].flip_rad) return true;
    return false;
}

int check_common(const tsg_program* prog, const tsg_tissue* tissue, int64_t atoms) {
    if (!prog) return fail(TSG_ERR_ARGUMENT, "null program");
    if (!tissue || (atoms > 0 && (!tissue->t1_ms || !tissue->t2_ms)))
        return fail(TSG_ERR_ARGUMENT, "t1 and t2 are required");
    return TSG_OK;
}

SecondArgs base_second_args(const tsg_program* prog, const tsg_tissue* tissue, int64_t atoms,
                            int64_t states) {
    SecondArgs a{};
    a.ops = prog->d_ops;
    a.n_ops = int(prog->host.ops);
    a.atoms = atoms;
    a.states = int(states);
    a.outputs = int(prog->host.outputs);
    a.t1 = tissue->t1_ms;
    a.t2 = tissue->t2_ms;
    a.m0 = tissue->m0;
    a.b1 = tissue->b1;
    a.inv = tissue->inversion;
    return a;
}

void set_directions(SecondArgs& a, const tsg_direction* d, int k) {
    for (int i = 0; i < k; ++i) {
        a.dir[i][0] = d[i].t1_ms;
        a.dir[i][1] = d[i].t2_ms;
        a.dir[i][2] = d[i].m0;
        a.dir[i][3] = d[i].b1;
        a.dir[i][4] = d[i].inversion;
    }
}

// Fills the per-op directions of the K directions into `dirs`.
int gather_all(const tsg_program* prog, const tsg_direction* d, int k, float2* dirs,
               cudaStream_t s) {
    const int64_t n = prog->host.ops * prog->host.trains;
    if (n == 0) return TSG_OK;
    for (int i = 0; i < k; ++i) {
        gather_second_directions<<<unsigned((n + 255) / 256), 256, 0, s>>>(
            prog->d_src, prog->host.ops, prog->host.trains, prog->host.events, d[i].duration_s,
            d[i].flip_rad, dirs + i * n);
        TSG_CUDA(cudaGetLastError());
    }
    return TSG_OK;
}

// The one-hot direction code of a TSG_TANGENT_T1 | T2 | B1 mask (those
// properties' unit tangents, in that order), and its direction count.
int hot_code(unsigned mask, int* k) {
    int code = 0, n = 0;
    const unsigned bits[3] = {TSG_TANGENT_T1, TSG_TANGENT_T2, TSG_TANGENT_B1};
    for (int p = 0; p < 3; ++p)
        if (mask & bits[p]) code |= (p + 1) << (2 * n++);
    *k = n;
    return code;
}

int run_forward(const tsg_program* program, const SecondPlan& plan, SecondArgs a, int with_m0,
                int layout, float* sig_a, float* sig_b, float* jac_a, float* jac_b,
                void* trajectory, cudaStream_t s) {
    if (!trajectory) return fail(TSG_ERR_ARGUMENT, "null trajectory");
    if (layout != TSG_LAYOUT_PLANES && layout != TSG_LAYOUT_COMPLEX_IJ && layout != TSG_LAYOUT_COMPLEX)
        return fail(TSG_ERR_ARGUMENT, "unknown layout");
    if (layout == TSG_LAYOUT_PLANES && ((sig_a && !sig_b) || (jac_a && !jac_b)))
        return fail(TSG_ERR_ARGUMENT, "the planes layout writes the imaginary plane");
    a.layout = layout;
    a.with_m0 = with_m0 ? 1 : 0;
    a.sig_a = sig_a;
    a.sig_b = layout == TSG_LAYOUT_PLANES ? sig_b : nullptr;
    a.jac_a = jac_a;
    a.jac_b = layout == TSG_LAYOUT_PLANES ? jac_b : nullptr;
    a.traj = static_cast<float2*>(trajectory);
    a.traj_rec = reinterpret_cast<float*>(static_cast<char*>(trajectory) + align256(plan.state_bytes));
    const int vpb = 4 * (32 / plan.entry->lanes_per_voxel);
    const int64_t blocks = (a.atoms + vpb - 1) / vpb;
    if (blocks > 0x7fffffffLL) return fail(TSG_ERR_CAPACITY, "too many voxels for one launch");
    plan.entry->forward(a, dim3(unsigned(blocks), unsigned(program->host.trains)), dim3(128), 0, s);
    TSG_CUDA(cudaGetLastError());
    return TSG_OK;
}

int run_reverse(const tsg_program* program, const SecondPlan& plan, SecondArgs a, int k, int hot,
                int with_m0, const float* seed_signal, const float* seed_derivatives,
                int seed_layout, const void* trajectory, const tsg_gradients* curvature,
                const tsg_gradients* values, char* ws, int64_t workspace_bytes, cudaStream_t s) {
    if (!trajectory || !ws || !seed_derivatives)
        return fail(TSG_ERR_ARGUMENT, "null trajectory, workspace or seed");
    if (workspace_bytes < plan.workspace_bytes) return fail(TSG_ERR_ARGUMENT, "workspace too small");
    if (seed_layout != TSG_LAYOUT_PLANES && seed_layout != TSG_LAYOUT_COMPLEX_IJ)
        return fail(TSG_ERR_ARGUMENT, "unknown seed layout");
    a.traj = const_cast<float2*>(static_cast<const float2*>(trajectory));
    a.traj_rec = reinterpret_cast<float*>(const_cast<char*>(static_cast<const char*>(trajectory)) +
                                          align256(plan.state_bytes));
    a.with_m0 = with_m0 ? 1 : 0;
    a.seed0 = seed_signal;
    a.seed = seed_derivatives;
    a.seed_layout = seed_layout;
    a.event_partial = reinterpret_cast<float2*>(ws + plan.dir_bytes);
    a.tissue_partial = reinterpret_cast<float*>(ws + plan.dir_bytes + plan.event_bytes);
    a.warps_per_train = plan.warps_per_train;
    if (plan.smem > 48 * 1024)
        TSG_CUDA(cudaFuncSetAttribute(plan.entry->reverse_fn,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, int(plan.smem)));
    plan.entry->reverse(a, dim3(unsigned(plan.blocks), unsigned(program->host.trains)),
                        dim3(32 * kSecondWarps), plan.smem, s);
    TSG_CUDA(cudaGetLastError());
    const int64_t ops = program->host.ops;
    const int pairs = event_pairs(k, hot);
    reduce_second_events<<<dim3(unsigned(ops), unsigned(program->host.trains)),
                           kEventReduceThreads, 0, s>>>(
        a.event_partial, plan.warps_per_train, ops, program->host.trains, program->host.events,
        pairs, program->d_src, curvature ? curvature->flip_rad : nullptr,
        curvature ? curvature->duration_s : nullptr,
        pairs == 2 && values ? values->flip_rad : nullptr,
        pairs == 2 && values ? values->duration_s : nullptr);
    TSG_CUDA(cudaGetLastError());
    TissueSlots slots{};
    if (curvature) {
        slots.slot[0][0] = curvature->t1_ms;
        slots.slot[0][1] = curvature->t2_ms;
        slots.slot[0][2] = curvature->m0;
        slots.slot[0][3] = curvature->b1;
        slots.slot[0][4] = curvature->inversion;
    }
    if (values && hot == 0)
        for (int i = 0; i < k; ++i) {
            slots.slot[1 + i][0] = values[i].t1_ms;
            slots.slot[1 + i][1] = values[i].t2_ms;
            slots.slot[1 + i][2] = values[i].m0;
            slots.slot[1 + i][3] = values[i].b1;
            slots.slot[1 + i][4] = values[i].inversion;
        }
    reduce_second_tissue<<<unsigned((a.atoms + 127) / 128), 128, 0, s>>>(
        a.tissue_partial, a.atoms, program->host.trains, tissue_values(k, hot), slots);
    TSG_CUDA(cudaGetLastError());
    return TSG_OK;
}

}  // namespace

}  // namespace tsg

using namespace tsg;

extern "C" int tsg_epg_second_plan(const tsg_program* program, int64_t atom_count,
                                   int64_t state_count, int direction_count,
                                   int event_directions, const tsg_launch* launch,
                                   int64_t* trajectory_bytes, int64_t* workspace_bytes) {
    SecondPlan plan;
    int rc = second_plan(program, atom_count, state_count, direction_count, 0, launch,
                         event_directions != 0, &plan);
    if (rc) return rc;
    if (trajectory_bytes) *trajectory_bytes = plan.trajectory_bytes;
    if (workspace_bytes) *workspace_bytes = plan.workspace_bytes;
    return TSG_OK;
}

extern "C" int tsg_epg_second_forward(const tsg_program* program, const tsg_tissue* tissue,
                                      int64_t atom_count, int64_t state_count,
                                      const tsg_direction* directions, int direction_count,
                                      int with_m0, int layout, float* sig_a, float* sig_b,
                                      float* jac_a, float* jac_b, void* trajectory,
                                      void* workspace, const tsg_launch* launch, void* stream) {
    int rc = check_common(program, tissue, atom_count);
    if (rc) return rc;
    const int k = direction_count;
    if (!directions) return fail(TSG_ERR_ARGUMENT, "null directions");
    if (k < 1 || k > kSecondMaxK) return fail(TSG_ERR_ARGUMENT, "1 to 3 directions");
    const bool evdir = has_event_directions(directions, k);
    SecondPlan plan;
    rc = second_plan(program, atom_count, state_count, k, 0, launch, evdir, &plan);
    if (rc) return rc;
    if (atom_count == 0 || program->host.ops == 0) return TSG_OK;
    if (evdir && !workspace) return fail(TSG_ERR_ARGUMENT, "null workspace");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    SecondArgs a = base_second_args(program, tissue, atom_count, state_count);
    set_directions(a, directions, k);
    if (evdir) {
        a.op_dir = static_cast<const float2*>(workspace);
        rc = gather_all(program, directions, k, static_cast<float2*>(workspace), s);
        if (rc) return rc;
    }
    return run_forward(program, plan, a, with_m0, layout, sig_a, sig_b, jac_a, jac_b, trajectory, s);
}

extern "C" int tsg_epg_second_reverse(const tsg_program* program, const tsg_tissue* tissue,
                                      int64_t atom_count, int64_t state_count,
                                      const tsg_direction* directions, int direction_count,
                                      int with_m0, const float* seed_signal,
                                      const float* seed_derivatives, int seed_layout,
                                      const void* trajectory,
                                      const tsg_gradients* curvature, const tsg_gradients* values,
                                      void* workspace, int64_t workspace_bytes,
                                      const tsg_launch* launch, void* stream) {
    int rc = check_common(program, tissue, atom_count);
    if (rc) return rc;
    const int k = direction_count;
    if (!directions) return fail(TSG_ERR_ARGUMENT, "null directions");
    if (k < 1 || k > kSecondMaxK) return fail(TSG_ERR_ARGUMENT, "1 to 3 directions");
    const bool evdir = has_event_directions(directions, k);
    SecondPlan plan;
    rc = second_plan(program, atom_count, state_count, k, 0, launch, evdir, &plan);
    if (rc) return rc;
    if (atom_count == 0 || program->host.ops == 0) return TSG_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    SecondArgs a = base_second_args(program, tissue, atom_count, state_count);
    set_directions(a, directions, k);
    char* ws = static_cast<char*>(workspace);
    if (evdir && ws) {
        a.op_dir = reinterpret_cast<const float2*>(ws);
        rc = gather_all(program, directions, k, reinterpret_cast<float2*>(ws), s);
        if (rc) return rc;
    }
    return run_reverse(program, plan, a, k, 0, with_m0, seed_signal, seed_derivatives, seed_layout,
                       trajectory, curvature, values, ws, workspace_bytes, s);
}

extern "C" int tsg_epg_design_plan(const tsg_program* program, int64_t atom_count,
                                   int64_t state_count, unsigned tangent_mask,
                                   const tsg_launch* launch, int64_t* trajectory_bytes,
                                   int64_t* workspace_bytes) {
    int k = 0;
    const int hot = hot_code(tangent_mask, &k);
    if (k == 0 || (tangent_mask & ~7u)) return fail(TSG_ERR_ARGUMENT, "tangent_mask takes T1, T2, B1");
    SecondPlan plan;
    int rc = second_plan(program, atom_count, state_count, k, hot, launch, false, &plan);
    if (rc) return rc;
    if (trajectory_bytes) *trajectory_bytes = plan.trajectory_bytes;
    if (workspace_bytes) *workspace_bytes = plan.workspace_bytes;
    return TSG_OK;
}

extern "C" int tsg_epg_design_forward(const tsg_program* program, const tsg_tissue* tissue,
                                      int64_t atom_count, int64_t state_count,
                                      unsigned tangent_mask, int with_m0, int layout,
                                      float* sig_a, float* sig_b, float* jac_a, float* jac_b,
                                      void* trajectory, const tsg_launch* launch, void* stream) {
    int rc = check_common(program, tissue, atom_count);
    if (rc) return rc;
    int k = 0;
    const int hot = hot_code(tangent_mask, &k);
    if (k == 0 || (tangent_mask & ~7u)) return fail(TSG_ERR_ARGUMENT, "tangent_mask takes T1, T2, B1");
    SecondPlan plan;
    rc = second_plan(program, atom_count, state_count, k, hot, launch, false, &plan);
    if (rc) return rc;
    if (atom_count == 0 || program->host.ops == 0) return TSG_OK;
    SecondArgs a = base_second_args(program, tissue, atom_count, state_count);
    return run_forward(program, plan, a, with_m0, layout, sig_a, sig_b, jac_a, jac_b, trajectory,
                       static_cast<cudaStream_t>(stream));
}

extern "C" int tsg_epg_design_reverse(const tsg_program* program, const tsg_tissue* tissue,
                                      int64_t atom_count, int64_t state_count,
                                      unsigned tangent_mask, int with_m0,
                                      const float* seed_signal, const float* seed_derivatives,
                                      int seed_layout, const void* trajectory,
                                      const tsg_gradients* curvature, void* workspace,
                                      int64_t workspace_bytes, const tsg_launch* launch,
                                      void* stream) {
    int rc = check_common(program, tissue, atom_count);
    if (rc) return rc;
    int k = 0;
    const int hot = hot_code(tangent_mask, &k);
    if (k == 0 || (tangent_mask & ~7u)) return fail(TSG_ERR_ARGUMENT, "tangent_mask takes T1, T2, B1");
    SecondPlan plan;
    rc = second_plan(program, atom_count, state_count, k, hot, launch, false, &plan);
    if (rc) return rc;
    if (atom_count == 0 || program->host.ops == 0) return TSG_OK;
    SecondArgs a = base_second_args(program, tissue, atom_count, state_count);
    return run_reverse(program, plan, a, k, hot, with_m0, seed_signal, seed_derivatives,
                       seed_layout, trajectory, curvature, nullptr, static_cast<char*>(workspace),
                       workspace_bytes, static_cast<cudaStream_t>(stream));
}

// ---- the host-buffer drop-in -------------------------------------------------

namespace tsg {
namespace {
std::mutex g_second_mutex;
constexpr int TISSUE = 17, PACKED = 26, FLOATS = 20, TAIL = 13;
}  // namespace
}  // namespace tsg

extern "C" int tsg_epg_simulate_vjp_jvp(void* const* pointers, int64_t pointer_count,
                                        int64_t atom_count, int64_t train_count,
                                        int64_t event_count, int64_t state_count,
                                        int64_t output_count, int real_axis, int features) {
    constexpr int64_t expected = PACKED + 3 * FLOATS + 2 + TAIL;
    if (!pointers || pointer_count != expected)
        return fail(TSG_ERR_ARGUMENT, "wrong number of buffer pointers");
    if (atom_count < 0 || train_count < 1 || event_count < 0 || state_count < 1 || output_count < 0)
        return fail(TSG_ERR_ARGUMENT, "invalid EPG buffer dimensions");
    if (real_axis != 1)
        return fail(TSG_ERR_UNSUPPORTED, "only the real-subspace path (real_axis == 1) is built");
    const int tangents = PACKED, seeds = PACKED + FLOATS, value_slots = seeds + 2,
              curve_slots = value_slots + FLOATS, tail = curve_slots + FLOATS;
    for (int i = 0; i < TAIL; ++i)
        if (pointers[tail + i] != nullptr)
            return fail(TSG_ERR_UNSUPPORTED, "transition tables, pools and per-voxel pulses are not built");
    if (features & 2) return fail(TSG_ERR_UNSUPPORTED, "flow is not built");
    for (int idx : {7, 9, 12}) {
        const float* v = static_cast<const float*>(pointers[idx]);
        if (v && (idx != 7 || (features & 4)))
            for (int64_t i = 0; i < atom_count; ++i)
                if (v[i] != 0.f) return fail(TSG_ERR_UNSUPPORTED, "diffusion and second pools are not built");
    }
    std::lock_guard<std::mutex> guard(g_second_mutex);
    cudaStream_t s = nullptr;
    const float* duration = static_cast<const float*>(pointers[TISSUE + 0]);
    const int32_t* kind = static_cast<const int32_t*>(pointers[TISSUE + 1]);
    const float* flip = static_cast<const float*>(pointers[TISSUE + 2]);
    const uint8_t* action = static_cast<const uint8_t*>(pointers[TISSUE + 4]);
    const int32_t* oindex = static_cast<const int32_t*>(pointers[TISSUE + 5]);
    // Unmerged: every event keeps its own op, so every event's duration
    // derivative is formed.
    tsg_program* prog = nullptr;
    int rc = tsg_program_create(duration, kind, flip, action, oindex, train_count, event_count, 1,
                                nullptr, &prog);
    if (rc) return rc;
    if (prog->host.outputs > output_count) {
        tsg_program_destroy(prog);
        return fail(TSG_ERR_ARGUMENT, "output index beyond output_count");
    }
    prog->host.outputs = output_count;
    std::vector<void*> owned;
    auto dev = [&](size_t bytes, void** out) -> int {
        *out = nullptr;
        cudaError_t e = cudaMallocAsync(out, bytes ? bytes : 4, s);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMallocAsync");
        owned.push_back(*out);
        return TSG_OK;
    };
    auto up = [&](const void* host, size_t bytes, void** out) -> int {
        *out = nullptr;
        if (!host || bytes == 0) return TSG_OK;
        int r = dev(bytes, out);
        if (r) return r;
        cudaError_t e = cudaMemcpyAsync(*out, host, bytes, cudaMemcpyHostToDevice, s);
        return e == cudaSuccess ? TSG_OK : cuda_fail(e, "cudaMemcpyAsync(H2D)");
    };
    const size_t ab = size_t(atom_count) * 4;
    const size_t eb = size_t(train_count) * size_t(event_count) * 4;
    const size_t ob = size_t(train_count) * size_t(atom_count) * size_t(output_count) * 4;
    const bool live_m0 = features & 16, live_b1 = features & 8, live_inv = features & 32;
    void *t1 = nullptr, *t2 = nullptr, *m0 = nullptr, *b1 = nullptr, *inv = nullptr;
    void *d_t1 = nullptr, *d_t2 = nullptr, *d_m0 = nullptr, *d_b1 = nullptr, *d_inv = nullptr;
    void *d_dur = nullptr, *d_flip = nullptr, *seed = nullptr, *traj = nullptr, *work = nullptr,
         *g = nullptr;
    if (!rc) rc = up(pointers[0], ab, &t1);
    if (!rc) rc = up(pointers[1], ab, &t2);
    if (!rc && live_m0) rc = up(pointers[2], ab, &m0);
    if (!rc && live_b1) rc = up(pointers[3], ab, &b1);
    if (!rc && live_inv) rc = up(pointers[6], ab, &inv);
    if (!rc) rc = up(pointers[tangents + 0], ab, &d_t1);
    if (!rc) rc = up(pointers[tangents + 1], ab, &d_t2);
    if (!rc && live_m0) rc = up(pointers[tangents + 2], ab, &d_m0);
    if (!rc && live_b1) rc = up(pointers[tangents + 3], ab, &d_b1);
    if (!rc && live_inv) rc = up(pointers[tangents + 6], ab, &d_inv);
    if (!rc) rc = up(pointers[tangents + TISSUE + 0], eb, &d_dur);
    if (!rc) rc = up(pointers[tangents + TISSUE + 1], eb, &d_flip);
    if (!rc) rc = up(pointers[seeds + 1], ob, &seed);  // the imaginary seed plane acts
    tsg_tissue tissue{static_cast<float*>(t1), static_cast<float*>(t2), static_cast<float*>(m0),
                      static_cast<float*>(b1), static_cast<float*>(inv)};
    tsg_direction dir{static_cast<float*>(d_t1), static_cast<float*>(d_t2),
                      static_cast<float*>(d_m0), static_cast<float*>(d_b1),
                      static_cast<float*>(d_inv), static_cast<float*>(d_dur),
                      static_cast<float*>(d_flip)};
    int64_t traj_bytes = 0, work_bytes = 0;
    if (!rc)
        rc = tsg_epg_second_plan(prog, atom_count, state_count, 1, d_dur || d_flip, nullptr,
                                 &traj_bytes, &work_bytes);
    if (!rc && atom_count > 0) rc = dev(size_t(traj_bytes), &traj);
    if (!rc && atom_count > 0) rc = dev(size_t(work_bytes), &work);
    // Device gradients: value then curvature, each 5 tissue rows of atoms,
    // then flip and duration rows.
    const size_t side = 5 * ab + 2 * eb;
    if (!rc) rc = dev(2 * side, &g);
    float* gf = static_cast<float*>(g);
    auto grads_at = [&](float* base) {
        return tsg_gradients{base, base + atom_count, base + 2 * atom_count,
                             base + 3 * atom_count, base + 4 * atom_count, base + 5 * atom_count,
                             base + 5 * atom_count + train_count * event_count};
    };
    if (!rc) {
        cudaMemsetAsync(g, 0, 2 * side, s);
        const tsg_gradients value = grads_at(gf), curve = grads_at(gf + side / 4);
        if (atom_count > 0 && seed) {
            rc = tsg_epg_second_forward(prog, &tissue, atom_count, state_count, &dir, 1, 0,
                                        TSG_LAYOUT_PLANES, nullptr, nullptr, nullptr, nullptr,
                                        traj, work, nullptr, s);
            if (!rc)
                rc = tsg_epg_second_reverse(prog, &tissue, atom_count, state_count, &dir, 1, 0,
                                            nullptr, static_cast<float*>(seed), TSG_LAYOUT_PLANES,
                                            traj, &curve, &value, work, work_bytes, nullptr, s);
        }
        // Slots: 17 tissue, then duration, flip, phase (_epg_cpu.cpp:11680-11706).
        const int tissue_slot[5] = {0, 1, 2, 3, 6};
        for (int half = 0; half < 2 && !rc; ++half) {
            void* const* slots = pointers + (half == 0 ? value_slots : curve_slots);
            const float* base = gf + half * (side / 4);
            auto down = [&](void* dst, const float* src, size_t bytes) {
                if (!dst || rc) return;
                cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s);
                if (e != cudaSuccess) rc = cuda_fail(e, "cudaMemcpyAsync(D2H)");
            };
            for (int j = 0; j < 5; ++j) down(slots[tissue_slot[j]], base + j * atom_count, ab);
            down(slots[TISSUE + 0], base + 5 * atom_count + train_count * event_count, eb);
            down(slots[TISSUE + 1], base + 5 * atom_count, eb);
        }
    }
    for (void* p : owned) cudaFreeAsync(p, s);
    cudaError_t es = cudaStreamSynchronize(s);
    if (!rc && es != cudaSuccess) rc = cuda_fail(es, "cudaStreamSynchronize");
    if (!rc) {
        // Directions the real subspace divides out, and those not built,
        // carry no gradient here; neither does the event phase.
        for (int half = 0; half < 2; ++half) {
            void* const* slots = pointers + (half == 0 ? value_slots : curve_slots);
            for (int j : {4, 5, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16})
                if (slots[j]) std::fill_n(static_cast<float*>(slots[j]), atom_count, 0.f);
            if (slots[TISSUE + 2])
                std::fill_n(static_cast<float*>(slots[TISSUE + 2]), train_count * event_count, 0.f);
        }
    }
    tsg_program_destroy(prog);
    return rc;
}
