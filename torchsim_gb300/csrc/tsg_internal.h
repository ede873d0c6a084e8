// Internal definitions shared by the kernels and the C ABI layer.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/torchsim_gb300.h"

namespace tsg {

// The packed action word (src/torchsim/_epg_cpu.cpp:36-41).
constexpr uint8_t A_PRE_SHIFT = 1;
constexpr uint8_t A_POST_SHIFT = 2;
constexpr uint8_t A_INVERSION = 4;
constexpr uint8_t A_SPOIL_AFTER = 8;
constexpr uint8_t A_SHIFT_AFTER = 16;
constexpr uint8_t A_RECORD = 32;

// One op of a compiled pulse program: a fixed template of micro-steps that
// one or more consecutive events reduce to, run in this order:
//   relax(dt) | shift x n1 | rf (rotate or invert) | shift x n2 | spoil |
//   record | shift x n3 | spoil
// An MRF repetition (pulse, sample, unbalanced gradient, delay) is one op.
struct __align__(16) Op {
    float dt;        // relaxation interval in seconds (RELAX set)
    float flip;      // flip angle in radians (rotate)
    int32_t record;  // output index (RECORD set)
    uint32_t code;   // micro-step bits below
};

constexpr uint32_t OP_RELAX = 1u << 0;
constexpr uint32_t OP_SHIFT1_SHIFT = 1;   // bits 1-2
constexpr uint32_t OP_RF_SHIFT = 3;       // bits 3-4: 0 none, 1 rotate, 2 invert
constexpr uint32_t OP_SHIFT2_SHIFT = 5;   // bits 5-6
constexpr uint32_t OP_SPOIL1 = 1u << 7;
constexpr uint32_t OP_RECORD = 1u << 8;
constexpr uint32_t OP_SHIFT3_SHIFT = 9;   // bits 9-10
constexpr uint32_t OP_SPOIL2 = 1u << 11;
constexpr int RF_NONE = 0, RF_ROTATE = 1, RF_INVERT = 2;

// The op shape of an MRF repetition and of most spoiled sequences: relax,
// rotate, (record), one shift after, and nothing else. The sweeps take a
// straight-line path for it with the shift folded into the rotation.
constexpr uint32_t kFastMask = OP_RELAX | (3u << OP_SHIFT1_SHIFT) | (3u << OP_RF_SHIFT) |
                               (3u << OP_SHIFT2_SHIFT) | OP_SPOIL1 | (3u << OP_SHIFT3_SHIFT) |
                               OP_SPOIL2;
constexpr uint32_t kFastBits = OP_RELAX | (uint32_t(RF_ROTATE) << OP_RF_SHIFT) |
                               (1u << OP_SHIFT3_SHIFT);

__host__ __device__ inline int op_shift1(uint32_t c) { return (c >> OP_SHIFT1_SHIFT) & 3; }
__host__ __device__ inline int op_rf(uint32_t c) { return (c >> OP_RF_SHIFT) & 3; }
__host__ __device__ inline int op_shift2(uint32_t c) { return (c >> OP_SHIFT2_SHIFT) & 3; }
__host__ __device__ inline int op_shift3(uint32_t c) { return (c >> OP_SHIFT3_SHIFT) & 3; }

// Where each op's dt and flip came from in the event stream, for the
// per-event gradients of the adjoint and the per-event directions of a
// general tangent. -1: the op has no such step.
struct OpSource {
    int32_t dt_event;
    int32_t rf_event;
    int32_t rec_event;  // the recording (ADC) event, for its phase's gradient
};

struct HostProgram {
    int64_t trains = 0;
    int64_t events = 0;
    int64_t ops = 0;       // per train (trains padded to the longest)
    int64_t outputs = 0;   // recorded samples per train
    bool sequential_records = true;  // records appear as 0,1,2,... in op order
    std::vector<Op> op;              // [train][ops]
    std::vector<OpSource> src;       // [train][ops]
    // With event phases (the complex path): per op the phase of its pulse
    // and of its receiver, [train][ops] (radians; 0 where absent).
    std::vector<float2> phase;
};

}  // namespace tsg

struct tsg_program {
    tsg::HostProgram host;
    tsg::Op* d_ops = nullptr;
    tsg::OpSource* d_src = nullptr;
    float2* d_phase = nullptr;  // null unless built with event phases
    int device = 0;
    // A view (tsg_program_view) borrows its template's source map and phases
    // and the caller's op array; destroying it frees none of them.
    bool view = false;
};

namespace tsg {

// Sets the thread's last error and returns code.
int fail(int code, const std::string& message);
int cuda_fail(cudaError_t err, const char* where);
#define TSG_CUDA(call)                                   \
    do {                                                 \
        cudaError_t _e = (call);                         \
        if (_e != cudaSuccess) return ::tsg::cuda_fail(_e, #call); \
    } while (0)

// Compiles an event stream and copies it to the current device (the phases
// nullable; with them, the complex path's per-op phases).
int create_program(const float* duration_s, const int32_t* kind, const float* flip_rad,
                   const float* phase_rad, const uint8_t* action, const int32_t* output_index,
                   int64_t train_count, int64_t event_count, int unmerged,
                   const float* duration_tangent, tsg_program** out);

int compile_program(const float* duration, const int32_t* kind, const float* flip,
                    const uint8_t* action, const int32_t* output_index, int64_t trains,
                    int64_t events, bool unmerged, const float* duration_tangent,
                    HostProgram* out, const float* phase = nullptr);

// Arguments of one sweep launch (forward, fused tangents, general tangent).
struct SweepArgs {
    const Op* ops;
    const float2* op_dir;  // general tangent: (d dt, d flip) per op, [train][ops]
    int n_ops;
    int64_t atoms;
    int states;
    int outputs;
    const float* t1;
    const float* t2;
    const float* m0;
    const float* b1;
    const float* inv;
    const float* g_t1;
    const float* g_t2;
    const float* g_m0;
    const float* g_b1;
    const float* g_inv;
    int layout;
    float* sig_a;
    float* sig_b;
    float* jac_a;
    float* jac_b;
    int jac_cols;
    int col_t1, col_t2, col_b1, col_inv, col_m0, col_gen;
    // Optional state checkpoints for the adjoint: every ckpt_every ops the
    // state entering that op is stored, [train][k][plane][order][atom] with
    // plane F+, F-, Z and `states` orders (atoms innermost: coalesced).
    float* ckpt;
    int ckpt_every;
    int ckpt_count;
    // Optional trajectory for the adjoint (forward sweeps only): every op's
    // entry state as order pairs, tiled by 32 atoms,
    // [train][atom / 32][op][plane][pair][atom % 32] float2 with
    // (states + 1) / 2 pairs, and every recorded F+[0], [train][output][atom].
    float2* traj;
    float* traj_rec;
    // Trajectory layout: 0 order pairs (2j, 2j+1) in float2 [.. pair][32];
    // 1 the one-lane sweep's own strided pairs (k, k + RP) two at a time in
    // float4 granules [.. granule][32] (trajectory_strided_orders).
    int traj_strided;
    // Gauss-Newton accumulation (GN sweeps): the measured samples (complex64
    // of the API signal) at row measured_rows[atom] (or atom when null), and
    // per voxel: cost, J^T J (6, upper triangle by rows) and J^T r (3) of the
    // natural parameters (T1, T2, M0), written as 10 doubles.
    const float2* measured;
    const int64_t* measured_rows;
    double* gn_out;
};

using SweepLaunch = void (*)(const SweepArgs&, dim3 grid, dim3 block, size_t smem,
                             cudaStream_t stream);

// Kernel families (which tangent systems a sweep carries).
enum SweepMode : int {
    MODE_FORWARD = 0,   // primal only
    MODE_T12 = 3,       // T1, T2
    MODE_T12B = 7,      // T1, T2, B1
    MODE_T12BI = 15,    // T1, T2, B1, inversion
    MODE_GENERAL = 16,  // one general direction
    MODE_GN = 35,       // T1, T2 (+ free M0) reduced to Gauss-Newton normal equations
};

struct SweepEntry {
    int mode;
    int orders_per_lane;  // R
    int lanes_per_voxel;  // L
    SweepLaunch launch;
    int min_blocks;       // register-budget variant (0: default budget)
};

// Tables defined by the per-mode translation units.
extern const SweepEntry kSweepForward[];
extern const int kSweepForwardCount;
extern const SweepEntry kSweepT12[];
extern const int kSweepT12Count;
extern const SweepEntry kSweepT12B[];
extern const int kSweepT12BCount;
extern const SweepEntry kSweepT12BI[];
extern const int kSweepT12BICount;
extern const SweepEntry kSweepGeneral[];
extern const int kSweepGeneralCount;
extern const SweepEntry kSweepGN[];
extern const int kSweepGNCount;

constexpr int kOpChunk = 1024;  // ops staged in shared memory at a time

// Arguments of the checkpointed reverse sweep.
struct AdjointArgs {
    const Op* ops;
    int n_ops;
    int64_t atoms;
    int states;
    int outputs;
    const float* t1;
    const float* t2;
    const float* m0;
    const float* b1;
    const float* inv;
    // Cotangent of the recorded samples: the imaginary plane (layout PLANES)
    // or the complex64 gradient of 1j*signal (layout COMPLEX_IJ).
    const float* seed;
    int seed_layout;
    const float* ckpt;   // [train][k][3][states][atom], written by a forward sweep
    const float2* traj;  // trajectory mode: [train][atom/32][op][3][(states+1)/2][atom%32] float2
    const float* traj_rec;  // trajectory mode: recorded F+[0], [train][output][atom]
    int ckpt_every;      // ops per segment (C)
    int ckpt_count;      // segments per row
    float2* event_partial;   // [train][warp][op]: (flip, duration) gradient partials
    int64_t warps_per_train;
    float* tissue_partial;   // [train][atom][5]: t1, t2, m0, b1, inversion
};

using AdjointLaunch = void (*)(const AdjointArgs&, dim3 grid, dim3 block, size_t smem,
                               cudaStream_t stream);

struct AdjointEntry {
    int orders_per_lane;
    int lanes_per_voxel;
    int warps;  // warps per block (compile-time in the kernel)
    AdjointLaunch launch;
    const void* kernel;  // for the shared-memory attribute
};

// The reverse-sweep kernels built for `warps` warps per block (2 or 4),
// checkpointed or trajectory; null with *count = 0 for any other block size.
const AdjointEntry* adjoint_table(int warps, bool trajectory, int* count);
// The one-lane reverse sweep over the strided trajectory layout, for R
// orders (10 or 20) and 2 or 4 warps per block; null if none.
const AdjointEntry* adjoint_strided_entry(int orders, int warps);

// Trajectory-mode reverse sweep: ops per event-gradient reduction, ops in
// flight per lane (ring slots in shared memory), and the longest program it
// keeps in shared memory.
// Threads of the event-gradient reductions (one block per op and train).
constexpr int kEventReduceThreads = 128;
constexpr int kTrajChunk = 32;
constexpr int kTrajRing = 4;
constexpr int kTrajMaxOps = 2048;

// Bytes of the adjoint's trajectory mode: entry states (whole tiles of 32
// atoms) and recorded F+[0].
// Trajectory mode up to 20 states runs one voxel per lane on both sides and
// stores the entry state of every other op (ops 0, 2, 4, ...; the reverse
// sweep re-runs each odd op from the even one before it) in the sweep's own
// register order: R orders (10 up to 10 states, else 20) as strided pairs
// (k, k + R/2), two pairs per 16-byte granule,
// [train][atom/32][op/2][plane][granule][atom%32] float4, so the forward
// stores and the reverse sweep copies whole registers. More states keep the
// contiguous pair layout of every op. Returns R, or 0 for the latter.
inline int trajectory_strided_orders(int64_t states) {
    return states <= 10 ? 10 : (states <= 20 ? 20 : 0);
}
inline int trajectory_granules(int orders) { return (orders / 2 + 1) / 2; }

inline int64_t trajectory_state_bytes(int64_t trains, int64_t ops, int64_t atoms, int64_t states) {
    const int orders = trajectory_strided_orders(states);
    if (orders > 0)
        return trains * ((atoms + 31) / 32) * ((ops + 1) / 2) * 3 * trajectory_granules(orders) *
               32 * int64_t(sizeof(float4));
    return trains * ((atoms + 31) / 32) * ops * 3 * ((states + 1) / 2) * 32 * int64_t(sizeof(float2));
}
inline int64_t trajectory_record_bytes(int64_t trains, int64_t outputs, int64_t atoms) {
    return trains * outputs * atoms * int64_t(sizeof(float));
}
inline int64_t align256(int64_t bytes) { return (bytes + 255) / 256 * 256; }

}  // namespace tsg
