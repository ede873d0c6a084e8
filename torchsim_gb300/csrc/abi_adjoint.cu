// C ABI of the checkpointed adjoint: planning, the device entry point and
// the host-buffer drop-in for the reference's _epg_cpu.simulate_vjp
// (src/torchsim/_epg_cpu.cpp:11150-11400).
#include <algorithm>
#include <mutex>
#include <vector>

#include "tsg_internal.h"

extern "C" int tsg_epg_forward_checkpointed(const tsg_program*, const tsg_tissue*, int64_t, int64_t,
                                            int, float*, float*, float*, int, const tsg_launch*,
                                            void*);
extern "C" int tsg_program_create(const float*, const int32_t*, const float*, const uint8_t*,
                                  const int32_t*, int64_t, int64_t, int, const float*,
                                  tsg_program**);
extern "C" int tsg_program_destroy(tsg_program*);

namespace tsg {

__global__ void reduce_event_gradients(const float2* partial, int64_t warps, int64_t n_ops,
                                       int64_t trains, int64_t events, const OpSource* src,
                                       float* grad_flip, float* grad_duration);
__global__ void reduce_tissue_gradients(const float* partial, int64_t atoms, int64_t trains,
                                        float* g_t1, float* g_t2, float* g_m0, float* g_b1,
                                        float* g_inv);

namespace {

// Shared memory a block may give the segment's pre-RF states.
constexpr size_t kStageBudget = 100 * 1024;

struct AdjointPlan {
    const AdjointEntry* entry = nullptr;
    bool trajectory = false;
    int warps = 4;
    int ops_per_checkpoint = 1;
    int checkpoint_count = 0;
    int64_t blocks = 0;
    int64_t warps_per_train = 0;
    int64_t checkpoint_bytes = 0;
    int64_t workspace_bytes = 0;
    size_t smem = 0;
};

int sm_count_adj() {
    static int count = [] {
        int dev = 0, n = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        return n > 0 ? n : 152;
    }();
    return count;
}

int make_plan_with(const tsg_program* prog, int64_t atoms, int64_t states, const tsg_launch* want,
                   int ops_per_checkpoint, bool one_lane, AdjointPlan* plan) {
    plan->warps = (want && want->warps_per_block > 0) ? want->warps_per_block : (one_lane ? 2 : 4);
    // ops_per_checkpoint == 1 is trajectory mode: the forward stores every
    // op's entry state and the reverse sweep re-runs nothing.
    const bool trajectory = ops_per_checkpoint == 1;
    plan->trajectory = trajectory;
    int table_count = 0;
    const AdjointEntry* table = adjoint_table(plan->warps, trajectory, &table_count);
    if (!table) return fail(TSG_ERR_ARGUMENT, "the adjoint takes 2 or 4 warps per block");
    const AdjointEntry* best = nullptr;
    double best_score = 1e300;
    const double target = double(sm_count_adj()) * 512.0;
    for (int i = 0; i < table_count; ++i) {
        const AdjointEntry& e = table[i];
        const int padded = e.lanes_per_voxel * e.orders_per_lane;
        if (padded < states) continue;
        if (want && want->lanes_per_voxel > 0 && e.lanes_per_voxel != want->lanes_per_voxel) continue;
        if (want && want->orders_per_lane > 0 && e.orders_per_lane != want->orders_per_lane) continue;
        if (one_lane && e.lanes_per_voxel != 1) continue;
        const int vpw = 32 / e.lanes_per_voxel;
        const double waste = double(padded) / double(states) * 32.0 /
                             double(vpw * e.lanes_per_voxel);
        const double lanes = double(atoms * prog->host.trains) * e.lanes_per_voxel;
        const double fill = std::min(1.0, lanes / target);
        const double score = waste / std::max(fill, 1e-3) *
                             (1.0 + 0.1 * (e.lanes_per_voxel - 1) / e.orders_per_lane);
        if (score < best_score) {
            best_score = score;
            best = &e;
        }
    }
    if (!best) return fail(TSG_ERR_UNSUPPORTED, "no adjoint kernel for this state count / launch shape");
    plan->entry = best;
    const int threads = 32 * plan->warps;
    const int vpb = plan->warps * (32 / best->lanes_per_voxel);
    const int64_t ops = prog->host.ops;
    const int64_t event_bytes = prog->host.trains * ((atoms + vpb - 1) / vpb) * plan->warps * ops *
                                int64_t(sizeof(float2));
    const int64_t tissue_bytes = prog->host.trains * atoms * 5 * int64_t(sizeof(float));
    plan->blocks = (atoms + vpb - 1) / vpb;
    plan->warps_per_train = plan->blocks * plan->warps;
    plan->workspace_bytes = align256(event_bytes) + tissue_bytes;
    if (trajectory) {
        // Shared memory: a chunk of ops, their transcendentals, the lanes'
        // event partials (rows of chunk + 1) and the entry-state ring.
        plan->ops_per_checkpoint = 1;
        plan->checkpoint_count = int(ops);
        plan->checkpoint_bytes =
            align256(trajectory_state_bytes(prog->host.trains, ops, atoms, states)) +
            trajectory_record_bytes(prog->host.trains, prog->host.outputs, atoms);
        if (ops > kTrajMaxOps)
            return fail(TSG_ERR_CAPACITY, "trajectory mode takes at most 2048 ops; use checkpoints");
        plan->smem = size_t(kTrajRing) * threads *
                         (sizeof(float4) + sizeof(float2) +
                          sizeof(float2) * 3 * size_t(best->orders_per_lane / 2)) +
                     sizeof(float2) * size_t(threads) * (kTrajChunk + 1) + sizeof(Op) * size_t(ops);
        if (plan->smem > 200 * 1024)
            return fail(TSG_ERR_CAPACITY, "trajectory ring does not fit in shared memory");
        return TSG_OK;
    }
    // Per op of a segment: the op, its transcendentals per voxel, the
    // pre-RF state (3 planes x orders x threads) and each lane's event
    // partials (float2; one more column pads the rows to an odd length).
    const size_t per_op = sizeof(Op) + sizeof(float4) * size_t(vpb) +
                          size_t(3) * best->orders_per_lane * threads * sizeof(float) +
                          sizeof(float2) * size_t(threads) + sizeof(float) * size_t(threads);
    // Fixed: the event rows' pad column and the prefetched checkpoint.
    const size_t pad = sizeof(float2) * size_t(threads) +
                       size_t(3) * best->orders_per_lane * threads * sizeof(float);
    int c = ops_per_checkpoint;
    if (c <= 0) c = int(std::max<size_t>(1, std::min<size_t>(64, (kStageBudget - pad) / per_op)));
    if (size_t(c) * per_op + pad > 200 * 1024)
        return fail(TSG_ERR_CAPACITY, "segment does not fit in shared memory");
    plan->ops_per_checkpoint = c;
    plan->checkpoint_count = int((ops + c - 1) / c);
    plan->checkpoint_bytes = prog->host.trains * atoms * int64_t(plan->checkpoint_count) * 3 * states *
                             int64_t(sizeof(float));
    plan->smem = size_t(c) * per_op + pad;
    return TSG_OK;
}

// Trajectory mode up to 20 states: one voxel per lane on the strided
// trajectory (the forward's own register order); a requested lane or order
// count is not used, its warps per block (2 or 4) are.
int make_strided_plan(const tsg_program* prog, int64_t atoms, int64_t states,
                      const tsg_launch* want, AdjointPlan* plan) {
    const int orders = trajectory_strided_orders(states);
    const int warps = (want && want->warps_per_block == 4) ? 4 : 2;
    if (want && want->warps_per_block > 0 && want->warps_per_block != 2 &&
        want->warps_per_block != 4)
        return fail(TSG_ERR_ARGUMENT, "the adjoint takes 2 or 4 warps per block");
    const AdjointEntry* entry = adjoint_strided_entry(orders, warps);
    if (!entry) return fail(TSG_ERR_UNSUPPORTED, "no strided trajectory kernel");
    const int64_t ops = prog->host.ops;
    if (ops > kTrajMaxOps)
        return fail(TSG_ERR_CAPACITY, "trajectory mode takes at most 2048 ops; use checkpoints");
    plan->entry = entry;
    plan->trajectory = true;
    plan->warps = warps;
    plan->ops_per_checkpoint = 1;
    plan->checkpoint_count = int(ops);
    const int threads = 32 * warps;
    plan->blocks = (atoms + threads - 1) / threads;
    plan->warps_per_train = plan->blocks * warps;
    const int64_t event_bytes = prog->host.trains * plan->warps_per_train * ops *
                                int64_t(sizeof(float2));
    const int64_t tissue_bytes = prog->host.trains * atoms * 5 * int64_t(sizeof(float));
    plan->workspace_bytes = align256(event_bytes) + tissue_bytes;
    plan->checkpoint_bytes =
        align256(trajectory_state_bytes(prog->host.trains, ops, atoms, states)) +
        trajectory_record_bytes(prog->host.trains, prog->host.outputs, atoms);
    const size_t granules = size_t(trajectory_granules(orders));
    // Per ring slot: an even op's entry state, and transcendentals, seed and
    // record of it and of the odd op after it.
    plan->smem = size_t(kTrajRing) * threads *
                     (2 * sizeof(float4) + 2 * sizeof(float2) + sizeof(float4) * 3 * granules) +
                 sizeof(float2) * size_t(threads) * (kTrajChunk + 1) + sizeof(Op) * size_t(ops);
    if (plan->smem > 200 * 1024)
        return fail(TSG_ERR_CAPACITY, "trajectory ring does not fit in shared memory");
    return TSG_OK;
}

int make_plan(const tsg_program* prog, int64_t atoms, int64_t states, const tsg_launch* want,
              int ops_per_checkpoint, AdjointPlan* plan) {
    if (!prog) return fail(TSG_ERR_ARGUMENT, "null program");
    if (atoms < 0 || states < 1) return fail(TSG_ERR_ARGUMENT, "invalid EPG buffer dimensions");
    if (states > 256) return fail(TSG_ERR_CAPACITY, "more than 256 states");
    if (ops_per_checkpoint == 1 && trajectory_strided_orders(states) > 0)
        return make_strided_plan(prog, atoms, states, want, plan);
    const bool shaped = want && (want->lanes_per_voxel > 0 || want->orders_per_lane > 0);
    // One voxel per lane up to 20 states (measured best), two warps a block;
    // a requested segment too long for its shared memory takes the
    // multi-lane shapes instead.
    if (!shaped && states <= 20) {
        AdjointPlan trial;
        if (make_plan_with(prog, atoms, states, want, ops_per_checkpoint, true, &trial) == TSG_OK) {
            *plan = trial;
            return TSG_OK;
        }
    }
    return make_plan_with(prog, atoms, states, want, ops_per_checkpoint, false, plan);
}

}  // namespace

// Runs the reverse sweep and the two reductions with a given plan and
// caller-provided checkpoints and workspace.
int run_adjoint(const tsg_program* prog, const tsg_tissue* tissue, int64_t atoms, int64_t states,
                const float* seed, int seed_layout, const float* ckpt, const AdjointPlan& plan,
                const tsg_gradients* grads, void* workspace, cudaStream_t stream) {
    if (atoms == 0 || prog->host.ops == 0) return TSG_OK;
    const int64_t ops = prog->host.ops;
    const int64_t event_bytes = prog->host.trains * plan.warps_per_train * ops * int64_t(sizeof(float2));
    AdjointArgs a{};
    a.ops = prog->d_ops;
    a.n_ops = int(ops);
    a.atoms = atoms;
    a.states = int(states);
    a.outputs = int(prog->host.outputs);
    a.t1 = tissue->t1_ms;
    a.t2 = tissue->t2_ms;
    a.m0 = tissue->m0;
    a.b1 = tissue->b1;
    a.inv = tissue->inversion;
    a.seed = seed;
    a.seed_layout = seed_layout;
    if (plan.trajectory) {
        const int64_t state_bytes =
            trajectory_state_bytes(prog->host.trains, ops, atoms, states);
        a.traj = reinterpret_cast<const float2*>(ckpt);
        a.traj_rec = reinterpret_cast<const float*>(reinterpret_cast<const char*>(ckpt) +
                                                    align256(state_bytes));
    } else {
        a.ckpt = ckpt;
    }
    a.ckpt_every = plan.ops_per_checkpoint;
    a.ckpt_count = plan.checkpoint_count;
    a.event_partial = static_cast<float2*>(workspace);
    a.warps_per_train = plan.warps_per_train;
    a.tissue_partial = reinterpret_cast<float*>(static_cast<char*>(workspace) +
                                                ((event_bytes + 255) / 256) * 256);
    if (plan.blocks > 0x7fffffffLL || prog->host.trains > 65535)
        return fail(TSG_ERR_CAPACITY, "launch too large");
    if (plan.smem > 48 * 1024)
        TSG_CUDA(cudaFuncSetAttribute(plan.entry->kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      int(plan.smem)));
    plan.entry->launch(a, dim3(unsigned(plan.blocks), unsigned(prog->host.trains)),
                       dim3(32 * plan.warps), plan.smem, stream);
    TSG_CUDA(cudaGetLastError());
    if (grads && (grads->flip_rad || grads->duration_s)) {
        reduce_event_gradients<<<dim3(unsigned(ops), unsigned(prog->host.trains)),
                                 kEventReduceThreads, 0, stream>>>(
            a.event_partial, plan.warps_per_train, ops, prog->host.trains, prog->host.events,
            prog->d_src, grads->flip_rad, grads->duration_s);
    }
    TSG_CUDA(cudaGetLastError());
    reduce_tissue_gradients<<<unsigned((atoms + 127) / 128), 128, 0, stream>>>(
        a.tissue_partial, atoms, prog->host.trains, grads ? grads->t1_ms : nullptr,
        grads ? grads->t2_ms : nullptr, grads ? grads->m0 : nullptr, grads ? grads->b1 : nullptr,
        grads ? grads->inversion : nullptr);
    TSG_CUDA(cudaGetLastError());
    return TSG_OK;
}

}  // namespace tsg

using namespace tsg;

extern "C" int tsg_epg_adjoint_plan(const tsg_program* program, int64_t atom_count,
                                    int64_t state_count, const tsg_launch* launch,
                                    int ops_per_checkpoint, int* resolved_ops_per_checkpoint,
                                    int64_t* checkpoint_bytes, int64_t* workspace_bytes) {
    AdjointPlan plan;
    int rc = make_plan(program, atom_count, state_count, launch, ops_per_checkpoint, &plan);
    if (rc) return rc;
    if (resolved_ops_per_checkpoint) *resolved_ops_per_checkpoint = plan.ops_per_checkpoint;
    if (checkpoint_bytes) *checkpoint_bytes = plan.checkpoint_bytes;
    if (workspace_bytes) *workspace_bytes = plan.workspace_bytes;
    return TSG_OK;
}

extern "C" int tsg_epg_adjoint(const tsg_program* program, const tsg_tissue* tissue,
                               int64_t atom_count, int64_t state_count, const float* seed,
                               int seed_layout, const float* checkpoints, int ops_per_checkpoint,
                               const tsg_gradients* gradients, void* workspace,
                               int64_t workspace_bytes, const tsg_launch* launch, void* stream) {
    if (!tissue || (atom_count > 0 && (!tissue->t1_ms || !tissue->t2_ms)))
        return fail(TSG_ERR_ARGUMENT, "t1 and t2 are required");
    AdjointPlan plan;
    int rc = make_plan(program, atom_count, state_count, launch, ops_per_checkpoint, &plan);
    if (rc) return rc;
    if (atom_count == 0) return TSG_OK;
    if (!seed || !checkpoints || !workspace) return fail(TSG_ERR_ARGUMENT, "null seed, checkpoints or workspace");
    if (workspace_bytes < plan.workspace_bytes) return fail(TSG_ERR_ARGUMENT, "workspace too small");
    if (seed_layout != TSG_LAYOUT_PLANES && seed_layout != TSG_LAYOUT_COMPLEX_IJ)
        return fail(TSG_ERR_ARGUMENT, "unknown seed layout");
    return run_adjoint(program, tissue, atom_count, state_count, seed, seed_layout, checkpoints, plan,
                       gradients, workspace, static_cast<cudaStream_t>(stream));
}

// ---- the host-buffer drop-in -------------------------------------------------

namespace tsg {
namespace {
std::mutex g_vjp_mutex;
constexpr int TISSUE = 17, PACKED = 26, FLOATS = 20, TAIL = 13;
}  // namespace
}  // namespace tsg

namespace tsg {
namespace {

// The complex path of the drop-in (the reference's complex simulate_vjp_range
// single-pool instant case): a phased program compiled unmerged, so every
// event's duration and phase gradient is formed; both seed planes act.
int simulate_vjp_complex(void* const* pointers, int64_t atom_count, int64_t train_count,
                         int64_t event_count, int64_t state_count, int64_t output_count,
                         int features) {
    if (features & 2) return fail(TSG_ERR_UNSUPPORTED, "flow is not built");
    for (int idx : {7, 9, 12}) {
        const float* v = static_cast<const float*>(pointers[idx]);
        if (v && (idx != 7 || (features & 4)))
            for (int64_t i = 0; i < atom_count; ++i)
                if (v[i] != 0.f) return fail(TSG_ERR_UNSUPPORTED, "diffusion and second pools are not built");
    }
    std::lock_guard<std::mutex> guard(g_vjp_mutex);
    cudaStream_t s = nullptr;
    const float* duration = static_cast<const float*>(pointers[TISSUE + 0]);
    const int32_t* kind = static_cast<const int32_t*>(pointers[TISSUE + 1]);
    const float* flip = static_cast<const float*>(pointers[TISSUE + 2]);
    const float* phase = static_cast<const float*>(pointers[TISSUE + 3]);
    const uint8_t* action = static_cast<const uint8_t*>(pointers[TISSUE + 4]);
    const int32_t* oindex = static_cast<const int32_t*>(pointers[TISSUE + 5]);
    if (!phase && event_count > 0) return fail(TSG_ERR_ARGUMENT, "null phase buffer");
    tsg_program* prog = nullptr;
    int rc = create_program(duration, kind, flip, phase, action, oindex, train_count, event_count, 1,
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
    void *t1 = nullptr, *t2 = nullptr, *m0 = nullptr, *b1 = nullptr, *inv = nullptr;
    void *b1p = nullptr, *b0 = nullptr, *sr = nullptr, *si = nullptr, *traj = nullptr,
         *work = nullptr, *g = nullptr;
    int64_t traj_bytes = 0, work_bytes = 0;
    if (!rc) rc = up(pointers[0], ab, &t1);
    if (!rc) rc = up(pointers[1], ab, &t2);
    if (!rc && (features & 16)) rc = up(pointers[2], ab, &m0);
    if (!rc && (features & 8)) rc = up(pointers[3], ab, &b1);
    if (!rc && (features & 32)) rc = up(pointers[6], ab, &inv);
    if (!rc && (features & 1)) rc = up(pointers[4], ab, &b1p);
    if (!rc && (features & 1)) rc = up(pointers[5], ab, &b0);
    if (!rc) rc = up(pointers[PACKED + 0], ob, &sr);
    if (!rc) rc = up(pointers[PACKED + 1], ob, &si);
    if (!rc) rc = tsg_epg_complex_adjoint_plan(prog, atom_count, state_count, nullptr, &traj_bytes,
                                               &work_bytes);
    if (!rc && atom_count > 0) rc = dev(size_t(traj_bytes), &traj);
    if (!rc && atom_count > 0) rc = dev(size_t(work_bytes), &work);
    // Device gradients: 7 per-atom rows (t1, t2, m0, b1, inversion, b1 phase,
    // b0), then flip, duration and phase rows.
    const size_t gb = 7 * ab + 3 * eb;
    if (!rc) rc = dev(gb, &g);
    if (!rc) {
        cudaMemsetAsync(g, 0, gb, s);
        float* gf = static_cast<float*>(g);
        float* ev = gf + 7 * atom_count;
        const int64_t te = train_count * event_count;
        tsg_gradients grads{gf, gf + atom_count, gf + 2 * atom_count, gf + 3 * atom_count,
                            gf + 4 * atom_count, ev, ev + te};
        tsg_offaxis_gradients ogr{gf + 5 * atom_count, gf + 6 * atom_count, ev + 2 * te};
        tsg_tissue tissue{static_cast<float*>(t1), static_cast<float*>(t2), static_cast<float*>(m0),
                          static_cast<float*>(b1), static_cast<float*>(inv)};
        tsg_offaxis off{static_cast<float*>(b1p), static_cast<float*>(b0)};
        if (atom_count > 0 && sr && si) {
            rc = tsg_epg_forward_complex_trajectory(prog, &tissue, &off, atom_count, state_count,
                                                    TSG_LAYOUT_PLANES, nullptr, nullptr, traj,
                                                    nullptr, s);
            if (!rc)
                rc = tsg_epg_adjoint_complex(prog, &tissue, &off, atom_count, state_count,
                                             static_cast<float*>(sr), static_cast<float*>(si),
                                             TSG_LAYOUT_PLANES, traj, &grads, &ogr, work,
                                             work_bytes, nullptr, s);
        }
        if (!rc) {
            // Slots: 17 tissue, then flip, phase, duration (_epg_cpu.cpp:11243-11253).
            void* const* slots = pointers + PACKED + 2;
            const int tissue_slot[7] = {0, 1, 2, 3, 6, 4, 5};
            auto down = [&](void* dst, const float* src, size_t bytes) {
                if (!dst || rc) return;
                cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s);
                if (e != cudaSuccess) rc = cuda_fail(e, "cudaMemcpyAsync(D2H)");
            };
            for (int k = 0; k < 7; ++k) down(slots[tissue_slot[k]], gf + k * atom_count, ab);
            down(slots[TISSUE + 0], ev, eb);
            down(slots[TISSUE + 1], ev + 2 * te, eb);
            down(slots[TISSUE + 2], ev + te, eb);
        }
    }
    for (void* p : owned) cudaFreeAsync(p, s);
    cudaError_t es = cudaStreamSynchronize(s);
    if (!rc && es != cudaSuccess) rc = cuda_fail(es, "cudaStreamSynchronize");
    if (!rc) {
        // Directions not built carry no gradient here.
        void* const* slots = pointers + PACKED + 2;
        for (int k : {7, 8, 9, 10, 11, 12, 13, 14, 15, 16})
            if (slots[k]) std::fill_n(static_cast<float*>(slots[k]), atom_count, 0.f);
    }
    tsg_program_destroy(prog);
    return rc;
}

}  // namespace
}  // namespace tsg

extern "C" int tsg_epg_simulate_vjp(void* const* pointers, int64_t pointer_count,
                                    int64_t atom_count, int64_t train_count, int64_t event_count,
                                    int64_t state_count, int64_t output_count, int real_axis,
                                    int features) {
    constexpr int64_t expected = PACKED + 2 + FLOATS + TAIL;
    if (!pointers || pointer_count != expected)
        return fail(TSG_ERR_ARGUMENT, "wrong number of buffer pointers");
    if (atom_count < 0 || train_count < 1 || event_count < 0 || state_count < 1 || output_count < 0)
        return fail(TSG_ERR_ARGUMENT, "invalid EPG buffer dimensions");
    for (int i = 0; i < TAIL; ++i)
        if (pointers[PACKED + 2 + FLOATS + i] != nullptr && i != TAIL - 3)  // GRADIENT slot may be given
            return fail(TSG_ERR_UNSUPPORTED, "transition tables, pools and per-voxel pulses are not built");
    if (real_axis != 1)
        return simulate_vjp_complex(pointers, atom_count, train_count, event_count, state_count,
                                    output_count, features);
    if (features & 2) return fail(TSG_ERR_UNSUPPORTED, "flow is not built");
    for (int idx : {7, 9, 12}) {
        const float* v = static_cast<const float*>(pointers[idx]);
        if (v && (idx != 7 || (features & 4)))
            for (int64_t i = 0; i < atom_count; ++i)
                if (v[i] != 0.f) return fail(TSG_ERR_UNSUPPORTED, "diffusion and second pools are not built");
    }
    std::lock_guard<std::mutex> guard(g_vjp_mutex);
    cudaStream_t s = nullptr;
    const float* duration = static_cast<const float*>(pointers[TISSUE + 0]);
    const int32_t* kind = static_cast<const int32_t*>(pointers[TISSUE + 1]);
    const float* flip = static_cast<const float*>(pointers[TISSUE + 2]);
    const uint8_t* action = static_cast<const uint8_t*>(pointers[TISSUE + 4]);
    const int32_t* oindex = static_cast<const int32_t*>(pointers[TISSUE + 5]);
    tsg_program* prog = nullptr;
    int rc = tsg_program_create(duration, kind, flip, action, oindex, train_count, event_count, 1,
                                nullptr, &prog);
    if (rc) return rc;
    if (prog->host.outputs > output_count) {
        tsg_program_destroy(prog);
        return fail(TSG_ERR_ARGUMENT, "output index beyond output_count");
    }
    prog->host.outputs = output_count;
    AdjointPlan plan;
    rc = make_plan(prog, atom_count, state_count, nullptr, 0, &plan);
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
    void *t1 = nullptr, *t2 = nullptr, *m0 = nullptr, *b1 = nullptr, *inv = nullptr, *seed = nullptr;
    void *ckpt = nullptr, *work = nullptr, *g = nullptr;
    if (!rc) rc = up(pointers[0], ab, &t1);
    if (!rc) rc = up(pointers[1], ab, &t2);
    if (!rc && (features & 16)) rc = up(pointers[2], ab, &m0);
    if (!rc && (features & 8)) rc = up(pointers[3], ab, &b1);
    if (!rc && (features & 32)) rc = up(pointers[6], ab, &inv);
    if (!rc) rc = up(pointers[PACKED + 1], ob, &seed);  // the imaginary seed plane acts
    if (!rc && atom_count > 0) rc = dev(size_t(plan.checkpoint_bytes), &ckpt);
    if (!rc && atom_count > 0) rc = dev(size_t(plan.workspace_bytes), &work);
    // Device gradients: 5 tissue rows of atoms, then flip and duration rows.
    const size_t gb = 5 * ab + 2 * eb;
    if (!rc) rc = dev(gb, &g);
    if (!rc) {
        cudaMemsetAsync(g, 0, gb, s);
        float* gf = static_cast<float*>(g);
        tsg_gradients grads{gf, gf + atom_count, gf + 2 * atom_count, gf + 3 * atom_count,
                            gf + 4 * atom_count, gf + 5 * atom_count,
                            gf + 5 * atom_count + train_count * event_count};
        tsg_tissue tissue{static_cast<float*>(t1), static_cast<float*>(t2), static_cast<float*>(m0),
                          static_cast<float*>(b1), static_cast<float*>(inv)};
        if (atom_count > 0 && seed) {
            rc = tsg_epg_forward_checkpointed(prog, &tissue, atom_count, state_count,
                                              TSG_LAYOUT_PLANES, nullptr, nullptr,
                                              static_cast<float*>(ckpt), plan.ops_per_checkpoint,
                                              nullptr, s);
            if (!rc)
                rc = run_adjoint(prog, &tissue, atom_count, state_count, static_cast<float*>(seed),
                                 TSG_LAYOUT_PLANES, static_cast<float*>(ckpt), plan, &grads, work, s);
        }
        if (!rc) {
            // Gradient slots: 17 tissue, then flip, phase, duration
            // (_epg_cpu.cpp:11243-11253).
            void* const* slots = pointers + PACKED + 2;
            const int tissue_slot[5] = {0, 1, 2, 3, 6};
            for (int k = 0; k < 5 && !rc; ++k)
                if (slots[tissue_slot[k]]) {
                    cudaError_t e = cudaMemcpyAsync(slots[tissue_slot[k]], gf + k * atom_count, ab,
                                                    cudaMemcpyDeviceToHost, s);
                    if (e != cudaSuccess) rc = cuda_fail(e, "cudaMemcpyAsync(D2H)");
                }
            if (!rc && slots[TISSUE + 0]) {
                cudaError_t e = cudaMemcpyAsync(slots[TISSUE + 0], gf + 5 * atom_count, eb,
                                                cudaMemcpyDeviceToHost, s);
                if (e != cudaSuccess) rc = cuda_fail(e, "cudaMemcpyAsync(D2H)");
            }
            if (!rc && slots[TISSUE + 2]) {
                cudaError_t e = cudaMemcpyAsync(slots[TISSUE + 2],
                                                gf + 5 * atom_count + train_count * event_count, eb,
                                                cudaMemcpyDeviceToHost, s);
                if (e != cudaSuccess) rc = cuda_fail(e, "cudaMemcpyAsync(D2H)");
            }
        }
    }
    for (void* p : owned) cudaFreeAsync(p, s);
    cudaError_t es = cudaStreamSynchronize(s);
    if (!rc && es != cudaSuccess) rc = cuda_fail(es, "cudaStreamSynchronize");
    if (!rc) {
        // Directions the real subspace divides out, and those not built,
        // carry no gradient here.
        void* const* slots = pointers + PACKED + 2;
        for (int k : {4, 5, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16})
            if (slots[k]) std::fill_n(static_cast<float*>(slots[k]), atom_count, 0.f);
        if (slots[TISSUE + 1])
            std::fill_n(static_cast<float*>(slots[TISSUE + 1]), train_count * event_count, 0.f);
    }
    tsg_program_destroy(prog);
    return rc;
}
