// The C ABI: program management, launch selection, the device-resident
// sweep entry points and the host-buffer drop-ins for the reference's
// _epg_cpu.simulate / simulate_jvp (src/torchsim/_epg_cpu.cpp:10740, 11017).
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "tsg_internal.h"

namespace tsg {

namespace {

struct Table {
    const SweepEntry* entries;
    int count;
};

Table table_for(int mode) {
    switch (mode) {
        case MODE_FORWARD: return {kSweepForward, kSweepForwardCount};
        case MODE_T12: return {kSweepT12, kSweepT12Count};
        case MODE_T12B: return {kSweepT12B, kSweepT12BCount};
        case MODE_T12BI: return {kSweepT12BI, kSweepT12BICount};
        case MODE_GENERAL: return {kSweepGeneral, kSweepGeneralCount};
        case MODE_GN: return {kSweepGN, kSweepGNCount};
    }
    return {nullptr, 0};
}

int sm_count() {
    static int count = [] {
        int dev = 0, n = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        return n > 0 ? n : 1;
    }();
    return count;
}

// Built-in launch heuristic: the fewest padded orders (L*R >= states), then
// enough lanes in flight to fill the GPU, then the fewest lanes per voxel
// (each lane of a voxel repeats the per-pulse exp/sincos).
const SweepEntry* choose(int mode, int states, int64_t work_items, const tsg_launch* want,
                         int* warps) {
    Table t = table_for(mode);
    *warps = (want && want->warps_per_block > 0) ? want->warps_per_block : 4;
    if (want && want->lanes_per_voxel > 0 && want->orders_per_lane > 0) {
        for (int i = 0; i < t.count; ++i)
            if (t.entries[i].lanes_per_voxel == want->lanes_per_voxel &&
                t.entries[i].orders_per_lane == want->orders_per_lane &&
                t.entries[i].min_blocks == want->min_blocks_per_sm &&
                want->lanes_per_voxel * want->orders_per_lane >= states) {
                if (t.entries[i].min_blocks > 0 && *warps > 4) return nullptr;
                return &t.entries[i];
            }
        return nullptr;
    }
    // Measured preferences on GB300 (launch-shape sweeps of each family):
    // one voxel per lane wherever its orders fit the registers, five lanes of
    // four orders for the four-system dictionary sweep at 20 states (with the
    // register-budget variant once the grid is large).
    struct Preferred {
        int mode, max_states, lanes, orders, min_blocks;
        int64_t min_items;
    };
    static const Preferred kPreferred[] = {
        {MODE_FORWARD, 10, 1, 10, 0, 0}, {MODE_FORWARD, 20, 1, 20, 0, 0},
        {MODE_T12, 10, 1, 10, 0, 0},     {MODE_GENERAL, 10, 1, 10, 0, 0},
        {MODE_GN, 10, 1, 10, 3, 0},      {MODE_T12B, 20, 5, 4, 5, 65536},
        {MODE_T12B, 20, 5, 4, 0, 0},     {MODE_T12BI, 10, 5, 2, 0, 0},
        {MODE_T12BI, 20, 5, 4, 0, 0},
    };
    if (!(want && (want->lanes_per_voxel > 0 || want->orders_per_lane > 0))) {
        for (const Preferred& p : kPreferred) {
            if (p.mode != mode || states > p.max_states || work_items < p.min_items) continue;
            if (p.min_blocks > 0 && *warps > 4) continue;
            for (int i = 0; i < t.count; ++i)
                if (t.entries[i].lanes_per_voxel == p.lanes && t.entries[i].orders_per_lane == p.orders &&
                    t.entries[i].min_blocks == p.min_blocks)
                    return &t.entries[i];
        }
    }
    const int64_t target_lanes = int64_t(sm_count()) * 1024;
    const SweepEntry* best = nullptr;
    double best_score = 1e300;
    for (int i = 0; i < t.count; ++i) {
        const SweepEntry& e = t.entries[i];
        const int padded = e.lanes_per_voxel * e.orders_per_lane;
        if (padded < states) continue;
        if (e.min_blocks > 0) continue;  // register-budget variants: by request only
        if (want && want->lanes_per_voxel > 0 && e.lanes_per_voxel != want->lanes_per_voxel) continue;
        const int vpw = 32 / e.lanes_per_voxel;
        const double waste = double(padded) / states * 32.0 / double(vpw * e.lanes_per_voxel);
        const double lanes = double(work_items) * e.lanes_per_voxel;
        const double fill = std::min(1.0, lanes / double(target_lanes));
        // Time ~ padded orders x lane redundancy / GPU fill.
        const double redundancy = 1.0 + 0.15 * (e.lanes_per_voxel - 1) / e.orders_per_lane;
        const double score = waste * redundancy / std::max(fill, 1e-3);
        if (score < best_score) {
            best_score = score;
            best = &e;
        }
    }
    return best;
}

int mode_for_mask(unsigned mask) {
    if (mask == 0) return MODE_FORWARD;
    if ((mask & ~3u) == 0) return MODE_T12;
    if ((mask & ~7u) == 0) return MODE_T12B;
    if ((mask & ~15u) == 0) return MODE_T12BI;
    return -1;
}

int launch(int mode, const tsg_program* prog, const SweepArgs& args, int64_t atoms, int states,
           const tsg_launch* want, cudaStream_t stream) {
    int warps = 4;
    const SweepEntry* e = choose(mode, states, atoms * prog->host.trains, want, &warps);
    if (!e) return fail(TSG_ERR_UNSUPPORTED, "no sweep kernel for this state count / launch shape");
    if (warps < 1 || warps > 8) return fail(TSG_ERR_ARGUMENT, "warps_per_block must be 1..8");
    if (atoms == 0 || prog->host.ops == 0) return TSG_OK;
    const int64_t vpb = int64_t(warps) * (32 / e->lanes_per_voxel);
    const int64_t blocks = (atoms + vpb - 1) / vpb;
    if (blocks > 0x7fffffffLL) return fail(TSG_ERR_CAPACITY, "too many voxels for one launch");
    if (prog->host.trains > 65535) return fail(TSG_ERR_CAPACITY, "more than 65535 trains");
    dim3 grid(unsigned(blocks), unsigned(prog->host.trains));
    e->launch(args, grid, dim3(32 * warps), 0, stream);
    TSG_CUDA(cudaGetLastError());
    return TSG_OK;
}

SweepArgs base_args(const tsg_program* prog, const tsg_tissue* tissue, int64_t atoms,
                    int64_t states) {
    SweepArgs a{};
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
    a.col_t1 = a.col_t2 = a.col_b1 = a.col_inv = a.col_m0 = a.col_gen = -1;
    a.ckpt_every = 1;
    return a;
}

int check_common(const tsg_program* prog, const tsg_tissue* tissue, int64_t atoms, int64_t states) {
    if (!prog) return fail(TSG_ERR_ARGUMENT, "null program");
    if (!tissue || (atoms > 0 && (!tissue->t1_ms || !tissue->t2_ms)))
        return fail(TSG_ERR_ARGUMENT, "t1 and t2 are required");
    if (atoms < 0 || states < 1) return fail(TSG_ERR_ARGUMENT, "invalid EPG buffer dimensions");
    if (states > 256) return fail(TSG_ERR_CAPACITY, "more than 256 states");
    return TSG_OK;
}

}  // namespace

}  // namespace tsg

using namespace tsg;

extern "C" int tsg_version(void) { return 1; }

namespace tsg {

int create_program(const float* duration_s, const int32_t* kind, const float* flip_rad,
                   const float* phase_rad, const uint8_t* action, const int32_t* output_index,
                   int64_t train_count, int64_t event_count, int unmerged,
                   const float* duration_tangent, tsg_program** out) {
    if (!out) return fail(TSG_ERR_ARGUMENT, "null output handle");
    *out = nullptr;
    auto* prog = new tsg_program();
    int rc = compile_program(duration_s, kind, flip_rad, action, output_index, train_count,
                             event_count, unmerged != 0, duration_tangent, &prog->host, phase_rad);
    if (rc != TSG_OK) {
        delete prog;
        return rc;
    }
    if (!prog->host.phase.empty()) {
        const size_t bytes = prog->host.phase.size() * sizeof(float2);
        cudaError_t e = cudaMalloc(&prog->d_phase, bytes);
        if (e == cudaSuccess)
            e = cudaMemcpy(prog->d_phase, prog->host.phase.data(), bytes, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaFree(prog->d_phase);
            delete prog;
            return cuda_fail(e, "cudaMemcpy(program phases)");
        }
    }
    cudaGetDevice(&prog->device);
    const size_t n = prog->host.op.size();
    if (n > 0) {
        cudaError_t e1 = cudaMalloc(&prog->d_ops, n * sizeof(Op));
        cudaError_t e2 = cudaMalloc(&prog->d_src, n * sizeof(OpSource));
        if (e1 != cudaSuccess || e2 != cudaSuccess) {
            cudaFree(prog->d_ops);
            cudaFree(prog->d_src);
            delete prog;
            return cuda_fail(e1 != cudaSuccess ? e1 : e2, "cudaMalloc(program)");
        }
        cudaError_t e3 = cudaMemcpy(prog->d_ops, prog->host.op.data(), n * sizeof(Op),
                                    cudaMemcpyHostToDevice);
        cudaError_t e4 = cudaMemcpy(prog->d_src, prog->host.src.data(), n * sizeof(OpSource),
                                    cudaMemcpyHostToDevice);
        if (e3 != cudaSuccess || e4 != cudaSuccess) {
            cudaFree(prog->d_ops);
            cudaFree(prog->d_src);
            cudaFree(prog->d_phase);
            delete prog;
            return cuda_fail(e3 != cudaSuccess ? e3 : e4, "cudaMemcpy(program)");
        }
    }
    *out = prog;
    return TSG_OK;
}

}  // namespace tsg

extern "C" int tsg_program_create(const float* duration_s, const int32_t* kind,
                                  const float* flip_rad, const uint8_t* action,
                                  const int32_t* output_index, int64_t train_count,
                                  int64_t event_count, int unmerged,
                                  const float* duration_tangent, tsg_program** out) {
    return create_program(duration_s, kind, flip_rad, nullptr, action, output_index, train_count,
                          event_count, unmerged, duration_tangent, out);
}

extern "C" int tsg_program_create_phased(const float* duration_s, const int32_t* kind,
                                         const float* flip_rad, const float* phase_rad,
                                         const uint8_t* action, const int32_t* output_index,
                                         int64_t train_count, int64_t event_count,
                                         tsg_program** out) {
    if (!phase_rad && event_count > 0) return fail(TSG_ERR_ARGUMENT, "null phase buffer");
    return create_program(duration_s, kind, flip_rad, phase_rad, action, output_index,
                          train_count, event_count, 0, nullptr, out);
}

extern "C" int tsg_program_plan(const float* duration_s, const int32_t* kind,
                                const float* flip_rad, const uint8_t* action,
                                const int32_t* output_index, int64_t train_count,
                                int64_t event_count, int unmerged, const float* duration_tangent,
                                int64_t* op_count, int64_t* output_count, float* dt_out,
                                float* flip_out, int32_t* record_out, uint32_t* code_out,
                                int64_t capacity) {
    HostProgram host;
    int rc = compile_program(duration_s, kind, flip_rad, action, output_index, train_count,
                             event_count, unmerged != 0, duration_tangent, &host);
    if (rc) return rc;
    if (op_count) *op_count = host.ops;
    if (output_count) *output_count = host.outputs;
    const int64_t n = std::min<int64_t>(capacity, int64_t(host.op.size()));
    for (int64_t i = 0; i < n; ++i) {
        if (dt_out) dt_out[i] = host.op[i].dt;
        if (flip_out) flip_out[i] = host.op[i].flip;
        if (record_out) record_out[i] = host.op[i].record;
        if (code_out) code_out[i] = host.op[i].code;
    }
    return TSG_OK;
}

extern "C" int tsg_program_destroy(tsg_program* program) {
    if (!program) return TSG_OK;
    if (!program->view) {
        cudaFree(program->d_ops);
        cudaFree(program->d_src);
        cudaFree(program->d_phase);
    }
    delete program;
    return TSG_OK;
}

// ---- programs rebound on the device -----------------------------------------

namespace tsg {
namespace {

// Every op of the template takes its dt from its relaxation's source event
// and its flip from its rotation's source event in the new per-event buffers;
// codes, records and sources are the template's.
__global__ void rebind_kernel(const Op* __restrict__ tmpl, const OpSource* __restrict__ src,
                              int64_t ops, int64_t events, int64_t total,
                              const float* __restrict__ duration, const float* __restrict__ flip,
                              Op* __restrict__ out) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const int64_t base = (i / ops) * events;
    Op op = tmpl[i];
    const OpSource s = src[i];
    if ((op.code & OP_RELAX) && s.dt_event >= 0) op.dt = duration[base + s.dt_event];
    if (op_rf(op.code) == RF_ROTATE && s.rf_event >= 0) op.flip = flip[base + s.rf_event];
    out[i] = op;
}

// x[0], x[0]+x[1], ... summed left to right in float32, one rounding per
// addition, as a sequential loop on the host does.
__global__ void sequential_sum_kernel(const float* __restrict__ x, int64_t n,
                                      float* __restrict__ out) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    float acc = 0.f;
    for (int64_t i = 0; i < n; ++i) {
        acc = i == 0 ? x[0] : __fadd_rn(acc, x[i]);
        out[i] = acc;
    }
}

}  // namespace
}  // namespace tsg

extern "C" int tsg_program_view(const tsg_program* tmpl, void* device_ops, tsg_program** out) {
    if (!out) return fail(TSG_ERR_ARGUMENT, "null output handle");
    *out = nullptr;
    if (!tmpl) return fail(TSG_ERR_ARGUMENT, "null program");
    if (tmpl->host.op.size() && !device_ops) return fail(TSG_ERR_ARGUMENT, "null op array");
    auto* prog = new tsg_program();
    prog->host = tmpl->host;
    prog->d_ops = static_cast<Op*>(device_ops);
    prog->d_src = tmpl->d_src;
    prog->d_phase = tmpl->d_phase;
    prog->device = tmpl->device;
    prog->view = true;
    *out = prog;
    return TSG_OK;
}

extern "C" int tsg_program_rebind(const tsg_program* tmpl, const float* duration_s,
                                  const float* flip_rad, void* device_ops, void* stream) {
    if (!tmpl) return fail(TSG_ERR_ARGUMENT, "null program");
    const int64_t total = int64_t(tmpl->host.op.size());
    if (total == 0) return TSG_OK;
    if (!duration_s || !flip_rad || !device_ops)
        return fail(TSG_ERR_ARGUMENT, "null rebind buffer");
    const int threads = 256;
    rebind_kernel<<<unsigned((total + threads - 1) / threads), threads, 0,
                    static_cast<cudaStream_t>(stream)>>>(
        tmpl->d_ops, tmpl->d_src, tmpl->host.ops, tmpl->host.events, total, duration_s, flip_rad,
        static_cast<Op*>(device_ops));
    TSG_CUDA(cudaGetLastError());
    return TSG_OK;
}

extern "C" int tsg_sequential_sum(const float* x, int64_t n, float* out, void* stream) {
    if (n < 0) return fail(TSG_ERR_ARGUMENT, "negative length");
    if (n == 0) return TSG_OK;
    if (!x || !out) return fail(TSG_ERR_ARGUMENT, "null buffer");
    sequential_sum_kernel<<<1, 32, 0, static_cast<cudaStream_t>(stream)>>>(x, n, out);
    TSG_CUDA(cudaGetLastError());
    return TSG_OK;
}

extern "C" int tsg_program_info(const tsg_program* p, int64_t* trains, int64_t* ops,
                                int64_t* outputs, int64_t* events) {
    if (!p) return fail(TSG_ERR_ARGUMENT, "null program");
    if (trains) *trains = p->host.trains;
    if (ops) *ops = p->host.ops;
    if (outputs) *outputs = p->host.outputs;
    if (events) *events = p->host.events;
    return TSG_OK;
}

extern "C" int tsg_epg_forward(const tsg_program* program, const tsg_tissue* tissue,
                               int64_t atom_count, int64_t state_count, int layout,
                               float* out_a, float* out_b, const tsg_launch* launch_shape,
                               void* stream) {
    int rc = check_common(program, tissue, atom_count, state_count);
    if (rc) return rc;
    if (atom_count == 0) return TSG_OK;
    if (layout < TSG_LAYOUT_PLANES || layout > TSG_LAYOUT_COMPLEX)
        return fail(TSG_ERR_ARGUMENT, "unknown layout");
    if (layout == TSG_LAYOUT_PLANES ? !out_b : !out_a)
        return fail(TSG_ERR_ARGUMENT, "null output buffer");
    SweepArgs a = base_args(program, tissue, atom_count, state_count);
    a.layout = layout;
    a.sig_a = out_a;
    a.sig_b = out_b;
    return launch(MODE_FORWARD, program, a, atom_count, int(state_count), launch_shape,
                  static_cast<cudaStream_t>(stream));
}

extern "C" int tsg_epg_forward_checkpointed(const tsg_program* program, const tsg_tissue* tissue,
                                            int64_t atom_count, int64_t state_count, int layout,
                                            float* out_a, float* out_b, float* checkpoints,
                                            int ops_per_checkpoint, const tsg_launch* launch_shape,
                                            void* stream) {
    int rc = check_common(program, tissue, atom_count, state_count);
    if (rc) return rc;
    if (ops_per_checkpoint < 1) return fail(TSG_ERR_ARGUMENT, "ops_per_checkpoint must be >= 1");
    if (atom_count == 0) return TSG_OK;
    if (!checkpoints) return fail(TSG_ERR_ARGUMENT, "null checkpoint buffer");
    SweepArgs a = base_args(program, tissue, atom_count, state_count);
    a.layout = layout;
    a.sig_a = out_a;
    a.sig_b = out_b;
    if (layout == TSG_LAYOUT_PLANES ? !out_b : !out_a) a.sig_a = a.sig_b = nullptr;
    tsg_launch pinned{};
    if (ops_per_checkpoint == 1) {
        // Trajectory mode: every op's entry state, then the recorded F+[0]
        // values. Up to 20 states the sweep runs one voxel per lane with the
        // reverse sweep's orders and stores its registers as they are.
        const int64_t state_bytes = trajectory_state_bytes(program->host.trains, program->host.ops,
                                                           atom_count, state_count);
        a.traj = reinterpret_cast<float2*>(checkpoints);
        a.traj_rec = reinterpret_cast<float*>(reinterpret_cast<char*>(checkpoints) +
                                              align256(state_bytes));
        const int orders = trajectory_strided_orders(state_count);
        if (orders > 0) {
            a.traj_strided = 1;
            pinned.lanes_per_voxel = 1;
            pinned.orders_per_lane = orders;
            pinned.warps_per_block = launch_shape ? launch_shape->warps_per_block : 0;
            launch_shape = &pinned;
        }
    } else {
        a.ckpt = checkpoints;
        a.ckpt_every = ops_per_checkpoint;
        a.ckpt_count = int((program->host.ops + ops_per_checkpoint - 1) / ops_per_checkpoint);
    }
    return launch(MODE_FORWARD, program, a, atom_count, int(state_count), launch_shape,
                  static_cast<cudaStream_t>(stream));
}

extern "C" int tsg_epg_forward_tangents(const tsg_program* program, const tsg_tissue* tissue,
                                        int64_t atom_count, int64_t state_count,
                                        unsigned tangent_mask, const int32_t* columns,
                                        int32_t column_count, int layout, float* sig_a,
                                        float* sig_b, float* jac_a, float* jac_b,
                                        const tsg_launch* launch_shape, void* stream) {
    int rc = check_common(program, tissue, atom_count, state_count);
    if (rc) return rc;
    if (!columns || column_count < 0) return fail(TSG_ERR_ARGUMENT, "null column map");
    if (atom_count == 0) return TSG_OK;
    const int mode = mode_for_mask(tangent_mask);
    if (mode < 0) return fail(TSG_ERR_UNSUPPORTED, "unknown tangent bits");
    for (int i = 0; i < 5; ++i)
        if (columns[i] >= column_count) return fail(TSG_ERR_ARGUMENT, "column out of range");
    const unsigned bits[4] = {TSG_TANGENT_T1, TSG_TANGENT_T2, TSG_TANGENT_B1, TSG_TANGENT_INVERSION};
    for (int i = 0; i < 4; ++i)
        if (columns[i] >= 0 && !(tangent_mask & bits[i]))
            return fail(TSG_ERR_ARGUMENT, "column given for a tangent not in the mask");
    const bool any_col = columns[0] >= 0 || columns[1] >= 0 || columns[2] >= 0 ||
                         columns[3] >= 0 || columns[4] >= 0;
    if (any_col && (layout == TSG_LAYOUT_PLANES ? !jac_b : !jac_a))
        return fail(TSG_ERR_ARGUMENT, "null Jacobian buffer");
    SweepArgs a = base_args(program, tissue, atom_count, state_count);
    a.layout = layout;
    a.sig_a = sig_a;
    a.sig_b = sig_b;
    if (layout == TSG_LAYOUT_PLANES && !sig_b) a.sig_a = nullptr;
    a.jac_a = jac_a;
    a.jac_b = jac_b;
    a.jac_cols = column_count;
    a.col_t1 = columns[0];
    a.col_t2 = columns[1];
    a.col_b1 = columns[2];
    a.col_inv = columns[3];
    a.col_m0 = columns[4];
    return launch(mode, program, a, atom_count, int(state_count), launch_shape,
                  static_cast<cudaStream_t>(stream));
}

extern "C" int tsg_gn_evaluate(const tsg_program* program, const tsg_tissue* tissue,
                               int64_t atom_count, int64_t state_count, const void* measured,
                               const int64_t* measured_rows, double* normal_equations,
                               const tsg_launch* launch_shape, void* stream) {
    int rc = check_common(program, tissue, atom_count, state_count);
    if (rc) return rc;
    if (atom_count == 0) return TSG_OK;
    if (!measured || !normal_equations) return fail(TSG_ERR_ARGUMENT, "null measured or output buffer");
    if (program->host.trains != 1) return fail(TSG_ERR_UNSUPPORTED, "Gauss-Newton runs one train");
    SweepArgs a = base_args(program, tissue, atom_count, state_count);
    a.layout = TSG_LAYOUT_COMPLEX_IJ;
    a.measured = static_cast<const float2*>(measured);
    a.measured_rows = measured_rows;
    a.gn_out = normal_equations;
    return launch(MODE_GN, program, a, atom_count, int(state_count), launch_shape,
                  static_cast<cudaStream_t>(stream));
}

namespace tsg {
namespace {

// (d dt, d flip) per op from per-event directions, through the op sources.
__global__ void gather_directions(const OpSource* src, int64_t n_ops, int64_t trains,
                                  int64_t events, const float* ddur, const float* dflip,
                                  float2* out) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n_ops * trains) return;
    const int64_t t = i / n_ops;
    const OpSource s = src[i];
    float a = 0.f, b = 0.f;
    if (ddur && s.dt_event >= 0) a = ddur[t * events + s.dt_event];
    if (dflip && s.rf_event >= 0) b = dflip[t * events + s.rf_event];
    out[i] = make_float2(a, b);
}

}  // namespace
}  // namespace tsg

extern "C" int tsg_epg_tangent(const tsg_program* program, const tsg_tissue* tissue,
                               int64_t atom_count, int64_t state_count,
                               const tsg_direction* direction, float* out_real, float* out_imag,
                               const tsg_launch* launch_shape, void* stream) {
    int rc = check_common(program, tissue, atom_count, state_count);
    if (rc) return rc;
    if (!direction) return fail(TSG_ERR_ARGUMENT, "null direction");
    if (atom_count == 0) return TSG_OK;
    if (!out_imag) return fail(TSG_ERR_ARGUMENT, "null output");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int64_t n = program->host.ops * program->host.trains;
    float2* dirs = nullptr;
    if (n > 0) {
        TSG_CUDA(cudaMallocAsync(&dirs, size_t(n) * sizeof(float2), s));
        gather_directions<<<unsigned((n + 255) / 256), 256, 0, s>>>(
            program->d_src, program->host.ops, program->host.trains, program->host.events,
            direction->duration_s, direction->flip_rad, dirs);
    }
    SweepArgs a = base_args(program, tissue, atom_count, state_count);
    a.op_dir = dirs;
    a.g_t1 = direction->t1_ms;
    a.g_t2 = direction->t2_ms;
    a.g_m0 = direction->m0;
    a.g_b1 = direction->b1;
    a.g_inv = direction->inversion;
    a.layout = TSG_LAYOUT_PLANES;
    a.jac_a = out_real;
    a.jac_b = out_imag;
    a.jac_cols = 1;
    a.col_gen = 0;
    rc = launch(MODE_GENERAL, program, a, atom_count, int(state_count), launch_shape, s);
    if (dirs) cudaFreeAsync(dirs, s);
    return rc;
}

// ---- host-buffer drop-ins --------------------------------------------------

namespace tsg {
namespace {

constexpr int TISSUE_COUNT = 17, EVENT_COUNT = 9, PACKED_COUNT = TISSUE_COUNT + EVENT_COUNT,
              FLOAT_COUNT = 20, TAIL_COUNT = 13;
// Feature bits of the reference's mask (src/torchsim/_epg_cpu.cpp:91-98).
constexpr int F_OFF_AXIS = 1, F_MOVING = 2, F_DIFFUSING = 4, F_TRANSMIT = 8, F_DENSITY = 16,
              F_INVERTING = 32;

// Copies n host floats to a fresh device allocation.
int upload(const void* host, size_t bytes, std::vector<void*>& owned, void** out,
           cudaStream_t s) {
    *out = nullptr;
    if (!host || bytes == 0) return TSG_OK;
    void* d = nullptr;
    TSG_CUDA(cudaMallocAsync(&d, bytes, s));
    owned.push_back(d);
    TSG_CUDA(cudaMemcpyAsync(d, host, bytes, cudaMemcpyHostToDevice, s));
    *out = d;
    return TSG_OK;
}

int dense_device(size_t bytes, std::vector<void*>& owned, void** out, cudaStream_t s) {
    void* d = nullptr;
    TSG_CUDA(cudaMallocAsync(&d, bytes ? bytes : 4, s));
    owned.push_back(d);
    *out = d;
    return TSG_OK;
}

void free_all(std::vector<void*>& owned, cudaStream_t s) {
    for (void* p : owned) cudaFreeAsync(p, s);
    owned.clear();
}

// The checks the real-subspace, single-pool subset needs of a pointer
// sequence in the reference's order.
int check_subset(void* const* ptrs, int64_t count, int64_t expected, int tail_begin,
                 int64_t atoms, int real_axis, int features, int64_t trains,
                 bool complex_ok = false) {
    if (!ptrs || count != expected) return fail(TSG_ERR_ARGUMENT, "wrong number of buffer pointers");
    if (real_axis != 1 && !complex_ok)
        return fail(TSG_ERR_UNSUPPORTED, "only the real-subspace path (real_axis == 1) is built");
    for (int i = 0; i < TAIL_COUNT; ++i)
        if (ptrs[tail_begin + i] != nullptr)
            return fail(TSG_ERR_UNSUPPORTED, "transition tables, pools and per-voxel pulses are not built");
    if (features & F_MOVING) return fail(TSG_ERR_UNSUPPORTED, "flow is not built");
    if ((features & F_OFF_AXIS) && real_axis == 1) {
        // The caller established the real subspace; off-axis terms must be
        // zero for that verdict, so they are only checked here.
        for (int idx : {4, 5}) {
            const float* v = static_cast<const float*>(ptrs[idx]);
            if (v)
                for (int64_t i = 0; i < atoms; ++i)
                    if (v[i] != 0.f)
                        return fail(TSG_ERR_UNSUPPORTED, "off-resonance / transmit phase leave the real subspace");
        }
    }
    if (features & F_DIFFUSING) {
        const float* d = static_cast<const float*>(ptrs[7]);
        if (d)
            for (int64_t i = 0; i < atoms; ++i)
                if (d[i] != 0.f) return fail(TSG_ERR_UNSUPPORTED, "diffusion is not built");
    }
    for (int idx : {9, 12}) {  // bound_fraction, pool_b_fraction gate the second pools
        const float* v = static_cast<const float*>(ptrs[idx]);
        if (v)
            for (int64_t i = 0; i < atoms; ++i)
                if (v[i] != 0.f) return fail(TSG_ERR_UNSUPPORTED, "second pools are not built");
    }
    // The shim index buffer (event slot 6) is not read: a single-pool run is
    // single-shim, every index is row 0.
    (void)trains;
    return TSG_OK;
}

std::mutex g_dropin_mutex;

// Output bytes (both planes) per chunk of a chunked drop-in call.
constexpr size_t kDropinChunkBytes = size_t(64) << 20;

// The forward of a single-train drop-in call in chunks of atoms: chunk c is
// swept on one stream into device slot c % 2 (both planes zeroed first: the
// caller's rows may be wider than the program's outputs), and copied to the
// caller's planes on a second stream while chunk c + 1 is swept. Both
// streams are blocking, so they order after the uploads on the caller's
// stream `s` and before what it does next.
int simulate_chunked(tsg_program* prog, const tsg_tissue& tissue, const tsg_offaxis& off,
                     bool complex_path, int64_t atoms, int64_t states, size_t row_bytes,
                     float* out_real, float* out_imag, std::vector<void*>& owned,
                     cudaStream_t s) {
    const int64_t per_chunk =
        std::max<int64_t>(1, int64_t(kDropinChunkBytes / (2 * row_bytes)));
    const int64_t chunks = (atoms + per_chunk - 1) / per_chunk;
    const size_t slot_bytes = size_t(per_chunk) * row_bytes;
    void* planes[2][2] = {};
    for (int slot = 0; slot < 2; ++slot)
        for (int pl = 0; pl < 2; ++pl) {
            int rc = dense_device(slot_bytes, owned, &planes[slot][pl], s);
            if (rc) return rc;
        }
    cudaStream_t sc = nullptr, sk = nullptr;
    cudaEvent_t done[2] = {}, freed[2] = {};
    int rc = TSG_OK;
    auto check = [&](cudaError_t e, const char* what) {
        if (!rc && e != cudaSuccess) rc = cuda_fail(e, what);
    };
    check(cudaStreamCreate(&sc), "cudaStreamCreate");
    check(cudaStreamCreate(&sk), "cudaStreamCreate");
    for (int i = 0; i < 2; ++i) {
        check(cudaEventCreateWithFlags(&done[i], cudaEventDisableTiming), "cudaEventCreate");
        check(cudaEventCreateWithFlags(&freed[i], cudaEventDisableTiming), "cudaEventCreate");
    }
    auto sweep = [&](int64_t c) {
        const int slot = int(c & 1);
        const int64_t a = c * per_chunk;
        const int64_t n = std::min(per_chunk, atoms - a);
        if (c >= 2) check(cudaStreamWaitEvent(sc, freed[slot], 0), "cudaStreamWaitEvent");
        check(cudaMemsetAsync(planes[slot][0], 0, size_t(n) * row_bytes, sc), "cudaMemsetAsync");
        check(cudaMemsetAsync(planes[slot][1], 0, size_t(n) * row_bytes, sc), "cudaMemsetAsync");
        auto at = [&](const float* p) -> const float* { return p ? p + a : nullptr; };
        tsg_tissue part{at(tissue.t1_ms), at(tissue.t2_ms), at(tissue.m0), at(tissue.b1),
                        at(tissue.inversion)};
        float* pr = static_cast<float*>(planes[slot][0]);
        float* pi = static_cast<float*>(planes[slot][1]);
        if (!rc) {
            if (complex_path) {
                tsg_offaxis poff{at(off.b1_phase_rad), at(off.b0_hz)};
                rc = tsg_epg_forward_complex(prog, &part, &poff, n, states, TSG_LAYOUT_PLANES, pr,
                                             pi, nullptr, sc);
            } else {
                rc = tsg_epg_forward(prog, &part, n, states, TSG_LAYOUT_PLANES, pr, pi, nullptr,
                                     sc);
            }
        }
        check(cudaEventRecord(done[slot], sc), "cudaEventRecord");
    };
    auto copy_back = [&](int64_t c) {
        const int slot = int(c & 1);
        const int64_t a = c * per_chunk;
        const int64_t n = std::min(per_chunk, atoms - a);
        const size_t off_bytes = size_t(a) * row_bytes, bytes = size_t(n) * row_bytes;
        check(cudaStreamWaitEvent(sk, done[slot], 0), "cudaStreamWaitEvent");
        check(cudaMemcpyAsync(reinterpret_cast<char*>(out_real) + off_bytes, planes[slot][0],
                              bytes, cudaMemcpyDeviceToHost, sk),
              "cudaMemcpyAsync(outputs)");
        check(cudaMemcpyAsync(reinterpret_cast<char*>(out_imag) + off_bytes, planes[slot][1],
                              bytes, cudaMemcpyDeviceToHost, sk),
              "cudaMemcpyAsync(outputs)");
        check(cudaEventRecord(freed[slot], sk), "cudaEventRecord");
    };
    if (!rc) sweep(0);
    for (int64_t c = 0; c < chunks && !rc; ++c) {
        // The next chunk's sweep goes out before this chunk's copies, which
        // may hold the host until they finish (pageable destinations).
        if (c + 1 < chunks) sweep(c + 1);
        copy_back(c);
    }
    if (sk) check(cudaStreamSynchronize(sk), "cudaStreamSynchronize");
    if (sc) check(cudaStreamSynchronize(sc), "cudaStreamSynchronize");
    for (int i = 0; i < 2; ++i) {
        if (done[i]) cudaEventDestroy(done[i]);
        if (freed[i]) cudaEventDestroy(freed[i]);
    }
    if (sc) cudaStreamDestroy(sc);
    if (sk) cudaStreamDestroy(sk);
    return rc;
}

}  // namespace
}  // namespace tsg

extern "C" int tsg_epg_simulate(void* const* pointers, int64_t pointer_count, int64_t atom_count,
                                int64_t train_count, int64_t event_count, int64_t state_count,
                                int64_t output_count, int real_axis, int features) {
    constexpr int64_t expected = PACKED_COUNT + 2 + TAIL_COUNT;
    if (atom_count < 0 || train_count < 1 || event_count < 0 || state_count < 1 || output_count < 0)
        return fail(TSG_ERR_ARGUMENT, "invalid EPG buffer dimensions");
    // Off the real subspace (real_axis != 1) the complex kernel runs, as the
    // reference's simulate switches to simulate_range (_epg_cpu.cpp:10860-10900).
    int rc = check_subset(pointers, pointer_count, expected, PACKED_COUNT + 2, atom_count,
                          real_axis, features, train_count, true);
    if (rc) return rc;
    const bool complex_path = real_axis != 1;
    std::lock_guard<std::mutex> guard(g_dropin_mutex);
    const float* duration = static_cast<const float*>(pointers[TISSUE_COUNT + 0]);
    const int32_t* kind = static_cast<const int32_t*>(pointers[TISSUE_COUNT + 1]);
    const float* flip = static_cast<const float*>(pointers[TISSUE_COUNT + 2]);
    const float* phase = static_cast<const float*>(pointers[TISSUE_COUNT + 3]);
    const uint8_t* action = static_cast<const uint8_t*>(pointers[TISSUE_COUNT + 4]);
    const int32_t* oindex = static_cast<const int32_t*>(pointers[TISSUE_COUNT + 5]);
    float* out_real = static_cast<float*>(pointers[PACKED_COUNT]);
    float* out_imag = static_cast<float*>(pointers[PACKED_COUNT + 1]);
    if (!out_real || !out_imag) return fail(TSG_ERR_ARGUMENT, "null output plane");
    tsg_program* prog = nullptr;
    if (complex_path)
        rc = tsg_program_create_phased(duration, kind, flip, phase, action, oindex, train_count,
                                       event_count, &prog);
    else
        rc = tsg_program_create(duration, kind, flip, action, oindex, train_count, event_count, 0,
                                nullptr, &prog);
    if (rc) return rc;
    if (prog->host.outputs > output_count) {
        tsg_program_destroy(prog);
        return fail(TSG_ERR_ARGUMENT, "output index beyond output_count");
    }
    cudaStream_t s = nullptr;
    std::vector<void*> owned;
    const size_t abytes = size_t(atom_count) * sizeof(float);
    void *t1, *t2, *m0 = nullptr, *b1 = nullptr, *inv = nullptr, *dr, *di;
    void *b1p = nullptr, *b0 = nullptr;
    rc = upload(pointers[0], abytes, owned, &t1, s);
    if (!rc) rc = upload(pointers[1], abytes, owned, &t2, s);
    if (!rc && (features & F_DENSITY)) rc = upload(pointers[2], abytes, owned, &m0, s);
    if (!rc && (features & F_TRANSMIT)) rc = upload(pointers[3], abytes, owned, &b1, s);
    if (!rc && (features & F_INVERTING)) rc = upload(pointers[6], abytes, owned, &inv, s);
    if (!rc && complex_path && (features & F_OFF_AXIS)) {
        rc = upload(pointers[4], abytes, owned, &b1p, s);
        if (!rc) rc = upload(pointers[5], abytes, owned, &b0, s);
    }
    const size_t obytes = size_t(train_count) * size_t(atom_count) * size_t(output_count) * 4;
    const size_t row_bytes = size_t(output_count) * 4;
    if (!rc && train_count == 1 && row_bytes > 0 && obytes > 2 * kDropinChunkBytes) {
        // Large single-train calls: the atoms go in chunks swept into two
        // device slots, each chunk's planes copied back while the next one
        // is swept (the device-to-host copies bound such a call).
        tsg_tissue tissue{static_cast<float*>(t1), static_cast<float*>(t2),
                          static_cast<float*>(m0), static_cast<float*>(b1),
                          static_cast<float*>(inv)};
        tsg_offaxis off{static_cast<float*>(b1p), static_cast<float*>(b0)};
        prog->host.outputs = output_count;
        rc = simulate_chunked(prog, tissue, off, complex_path, atom_count, state_count,
                              row_bytes, out_real, out_imag, owned, s);
        free_all(owned, s);
        cudaError_t es = cudaStreamSynchronize(s);
        if (!rc && es != cudaSuccess) rc = cuda_fail(es, "cudaStreamSynchronize");
        tsg_program_destroy(prog);
        return rc;
    }
    if (!rc) rc = dense_device(obytes, owned, &dr, s);
    if (!rc) rc = dense_device(obytes, owned, &di, s);
    if (!rc && obytes) {
        cudaMemsetAsync(dr, 0, obytes, s);
        cudaMemsetAsync(di, 0, obytes, s);
    }
    if (!rc) {
        // The kernels index outputs by the program's output count; the caller
        // may give a wider row.
        tsg_tissue tissue{static_cast<float*>(t1), static_cast<float*>(t2),
                          static_cast<float*>(m0), static_cast<float*>(b1),
                          static_cast<float*>(inv)};
        prog->host.outputs = output_count;
        if (complex_path) {
            tsg_offaxis off{static_cast<float*>(b1p), static_cast<float*>(b0)};
            rc = tsg_epg_forward_complex(prog, &tissue, &off, atom_count, state_count,
                                         TSG_LAYOUT_PLANES, static_cast<float*>(dr),
                                         static_cast<float*>(di), nullptr, s);
        } else {
            rc = tsg_epg_forward(prog, &tissue, atom_count, state_count, TSG_LAYOUT_PLANES,
                                 static_cast<float*>(dr), static_cast<float*>(di), nullptr, s);
        }
    }
    if (!rc && obytes) {
        cudaError_t e1 = cudaMemcpyAsync(out_real, dr, obytes, cudaMemcpyDeviceToHost, s);
        cudaError_t e2 = cudaMemcpyAsync(out_imag, di, obytes, cudaMemcpyDeviceToHost, s);
        if (e1 != cudaSuccess || e2 != cudaSuccess)
            rc = cuda_fail(e1 != cudaSuccess ? e1 : e2, "cudaMemcpyAsync(outputs)");
    }
    free_all(owned, s);
    cudaError_t es = cudaStreamSynchronize(s);
    if (!rc && es != cudaSuccess) rc = cuda_fail(es, "cudaStreamSynchronize");
    tsg_program_destroy(prog);
    return rc;
}

extern "C" int tsg_epg_simulate_jvp(void* const* pointers, int64_t pointer_count,
                                    int64_t atom_count, int64_t train_count, int64_t event_count,
                                    int64_t state_count, int64_t output_count, int real_axis,
                                    int features) {
    constexpr int64_t expected = PACKED_COUNT + FLOAT_COUNT + 2 + TAIL_COUNT;
    if (atom_count < 0 || train_count < 1 || event_count < 0 || state_count < 1 || output_count < 0)
        return fail(TSG_ERR_ARGUMENT, "invalid EPG buffer dimensions");
    // Off the real subspace (real_axis != 1) the complex tangent kernel runs,
    // as the reference's dispatch_jvp picks simulate_jvp_range there
    // (_epg_cpu.cpp:10957-10980).
    int rc = check_subset(pointers, pointer_count, expected, PACKED_COUNT + FLOAT_COUNT + 2,
                          atom_count, real_axis, features, train_count, true);
    if (rc) return rc;
    const bool complex_path = real_axis != 1;
    std::lock_guard<std::mutex> guard(g_dropin_mutex);
    void* const* tan = pointers + PACKED_COUNT;  // FLOAT_INPUTS order
    const float* duration = static_cast<const float*>(pointers[TISSUE_COUNT + 0]);
    const int32_t* kind = static_cast<const int32_t*>(pointers[TISSUE_COUNT + 1]);
    const float* flip = static_cast<const float*>(pointers[TISSUE_COUNT + 2]);
    const float* phase = static_cast<const float*>(pointers[TISSUE_COUNT + 3]);
    const uint8_t* action = static_cast<const uint8_t*>(pointers[TISSUE_COUNT + 4]);
    const int32_t* oindex = static_cast<const int32_t*>(pointers[TISSUE_COUNT + 5]);
    const float* dur_tangent = static_cast<const float*>(tan[TISSUE_COUNT + 0]);
    float* out_real = static_cast<float*>(pointers[PACKED_COUNT + FLOAT_COUNT]);
    float* out_imag = static_cast<float*>(pointers[PACKED_COUNT + FLOAT_COUNT + 1]);
    if (!out_real || !out_imag) return fail(TSG_ERR_ARGUMENT, "null output plane");
    if (complex_path && event_count > 0 && !phase) return fail(TSG_ERR_ARGUMENT, "null phase buffer");
    tsg_program* prog = nullptr;
    rc = create_program(duration, kind, flip, complex_path ? phase : nullptr, action, oindex,
                        train_count, event_count, 0, dur_tangent, &prog);
    if (rc) return rc;
    if (prog->host.outputs > output_count) {
        tsg_program_destroy(prog);
        return fail(TSG_ERR_ARGUMENT, "output index beyond output_count");
    }
    cudaStream_t s = nullptr;
    std::vector<void*> owned;
    const size_t abytes = size_t(atom_count) * sizeof(float);
    const size_t ebytes = size_t(train_count) * size_t(event_count) * sizeof(float);
    void *t1, *t2, *m0 = nullptr, *b1 = nullptr, *inv = nullptr, *b1p = nullptr, *b0 = nullptr;
    // Tangents: t1, t2, m0, b1, inversion; duration, flip; b1 phase, b0, phase.
    void* g[10] = {};
    void *dr, *di;
    rc = upload(pointers[0], abytes, owned, &t1, s);
    if (!rc) rc = upload(pointers[1], abytes, owned, &t2, s);
    if (!rc && (features & F_DENSITY)) rc = upload(pointers[2], abytes, owned, &m0, s);
    if (!rc && (features & F_TRANSMIT)) rc = upload(pointers[3], abytes, owned, &b1, s);
    if (!rc && (features & F_INVERTING)) rc = upload(pointers[6], abytes, owned, &inv, s);
    if (!rc && complex_path && (features & F_OFF_AXIS)) {
        rc = upload(pointers[4], abytes, owned, &b1p, s);
        if (!rc) rc = upload(pointers[5], abytes, owned, &b0, s);
    }
    const int tissue_idx[5] = {0, 1, 2, 3, 6};
    for (int k = 0; k < 5 && !rc; ++k) rc = upload(tan[tissue_idx[k]], abytes, owned, &g[k], s);
    if (!rc) rc = upload(tan[TISSUE_COUNT + 0], ebytes, owned, &g[5], s);
    if (!rc) rc = upload(tan[TISSUE_COUNT + 1], ebytes, owned, &g[6], s);
    if (!rc && complex_path) {
        rc = upload(tan[4], abytes, owned, &g[7], s);
        if (!rc) rc = upload(tan[5], abytes, owned, &g[8], s);
        if (!rc) rc = upload(tan[TISSUE_COUNT + 2], ebytes, owned, &g[9], s);
    }
    const size_t obytes = size_t(train_count) * size_t(atom_count) * size_t(output_count) * 4;
    if (!rc) rc = dense_device(obytes, owned, &dr, s);
    if (!rc) rc = dense_device(obytes, owned, &di, s);
    if (!rc && obytes) {
        cudaMemsetAsync(dr, 0, obytes, s);
        cudaMemsetAsync(di, 0, obytes, s);
    }
    if (!rc) {
        tsg_tissue tissue{static_cast<float*>(t1), static_cast<float*>(t2),
                          static_cast<float*>(m0), static_cast<float*>(b1),
                          static_cast<float*>(inv)};
        tsg_direction dir{static_cast<float*>(g[0]), static_cast<float*>(g[1]),
                          static_cast<float*>(g[2]), static_cast<float*>(g[3]),
                          static_cast<float*>(g[4]), static_cast<float*>(g[5]),
                          static_cast<float*>(g[6])};
        prog->host.outputs = output_count;
        if (complex_path) {
            tsg_offaxis off{static_cast<float*>(b1p), static_cast<float*>(b0)};
            tsg_offaxis_direction odir{static_cast<float*>(g[7]), static_cast<float*>(g[8]),
                                       static_cast<float*>(g[9])};
            rc = tsg_epg_tangent_complex(prog, &tissue, &off, atom_count, state_count, &dir,
                                         &odir, TSG_LAYOUT_PLANES, static_cast<float*>(dr),
                                         static_cast<float*>(di), nullptr, s);
        } else {
            rc = tsg_epg_tangent(prog, &tissue, atom_count, state_count, &dir,
                                 static_cast<float*>(dr), static_cast<float*>(di), nullptr, s);
        }
    }
    if (!rc && obytes) {
        cudaError_t e1 = cudaMemcpyAsync(out_real, dr, obytes, cudaMemcpyDeviceToHost, s);
        cudaError_t e2 = cudaMemcpyAsync(out_imag, di, obytes, cudaMemcpyDeviceToHost, s);
        if (e1 != cudaSuccess || e2 != cudaSuccess)
            rc = cuda_fail(e1 != cudaSuccess ? e1 : e2, "cudaMemcpyAsync(outputs)");
    }
    free_all(owned, s);
    cudaError_t es = cudaStreamSynchronize(s);
    if (!rc && es != cudaSuccess) rc = cuda_fail(es, "cudaStreamSynchronize");
    tsg_program_destroy(prog);
    return rc;
}

// ---- measurement ------------------------------------------------------------

namespace tsg {
namespace {

// Eight independent FMA chains per thread: the FP32 CUDA-core issue rate with
// nothing else in the way, the denominator of the sweep kernels' roofline.
__global__ void fp32_probe_kernel(float* out, int iters, float seed) {
    float a0 = seed + threadIdx.x, a1 = a0 + 1.f, a2 = a0 + 2.f, a3 = a0 + 3.f;
    float a4 = a0 + 4.f, a5 = a0 + 5.f, a6 = a0 + 6.f, a7 = a0 + 7.f;
    const float b = 0.999999f, c = 1e-6f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            a0 = fmaf(a0, b, c); a1 = fmaf(a1, b, c); a2 = fmaf(a2, b, c); a3 = fmaf(a3, b, c);
            a4 = fmaf(a4, b, c); a5 = fmaf(a5, b, c); a6 = fmaf(a6, b, c); a7 = fmaf(a7, b, c);
        }
    }
    const float s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
    if (s == 123456.f) out[blockIdx.x] = s;  // keeps the chains live
}

// The same with paired FP32 FMAs (two lanes' worth of work per instruction).
__global__ void fp32x2_probe_kernel(float* out, int iters, float seed) {
    float2 a0 = make_float2(seed + threadIdx.x, seed - threadIdx.x);
    float2 a1 = make_float2(a0.x + 1.f, a0.y + 1.f), a2 = make_float2(a0.x + 2.f, a0.y + 2.f);
    float2 a3 = make_float2(a0.x + 3.f, a0.y + 3.f);
    const float2 b = make_float2(0.999999f, 0.999999f), c = make_float2(1e-6f, 1e-6f);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            a0 = __ffma2_rn(a0, b, c); a1 = __ffma2_rn(a1, b, c);
            a2 = __ffma2_rn(a2, b, c); a3 = __ffma2_rn(a3, b, c);
        }
    }
    const float s = (a0.x + a0.y + a1.x + a1.y) + (a2.x + a2.y + a3.x + a3.y);
    if (s == 123456.f) out[blockIdx.x] = s;
}

}  // namespace
}  // namespace tsg

extern "C" int tsg_probe_fp32x2(int64_t blocks, int threads, int iters, float* out, void* stream,
                                double* flops) {
    if (blocks < 1 || threads < 32 || threads > 1024 || iters < 1 || !out)
        return fail(TSG_ERR_ARGUMENT, "invalid probe shape");
    fp32x2_probe_kernel<<<unsigned(blocks), threads, 0, static_cast<cudaStream_t>(stream)>>>(
        out, iters, 1.0f);
    TSG_CUDA(cudaGetLastError());
    if (flops) *flops = double(blocks) * threads * double(iters) * 4.0 * 8.0 * 2.0;
    return TSG_OK;
}

extern "C" int tsg_probe_fp32(int64_t blocks, int threads, int iters, float* out, void* stream,
                              double* flops) {
    if (blocks < 1 || threads < 32 || threads > 1024 || iters < 1 || !out)
        return fail(TSG_ERR_ARGUMENT, "invalid probe shape");
    fp32_probe_kernel<<<unsigned(blocks), threads, 0, static_cast<cudaStream_t>(stream)>>>(
        out, iters, 1.0f);
    TSG_CUDA(cudaGetLastError());
    if (flops) *flops = double(blocks) * threads * double(iters) * 4.0 * 8.0 * 2.0;
    return TSG_OK;
}
