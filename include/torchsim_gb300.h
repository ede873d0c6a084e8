/*
 * torchsim_gb300 — C ABI of the GB300 (sm_103a) extended-phase-graph kernels.
 *
 * Two families of entry points:
 *
 *  1. Drop-ins for the reference's own native boundary, the CPython functions
 *     of src/torchsim/_epg_cpu.cpp (module table at :11757). They take the
 *     same pointer sequences in the same order — the packed buffers of
 *     sequence/_parameters.py:105-195, then the output/tangent/gradient
 *     slots — as HOST pointers, copy to the device, run, and copy back before
 *     returning, so a caller that binds _epg_cpu.simulate can bind these
 *     instead. Only the real-subspace, single-pool, instant-RF subset is
 *     served (real_axis == 1; no pools, tables, per-voxel pulses, diffusion,
 *     flow); anything else returns TSG_ERR_UNSUPPORTED.
 *
 *  2. Device-resident entry points used by the Python package: a compiled
 *     pulse program (tsg_program) plus DEVICE pointers and a CUDA stream.
 *     They are stream-ordered and do not synchronise the host.
 *
 * Every function returns TSG_OK (0) or a negative TSG_ERR_* code; the message
 * of the last failure on the calling thread is tsg_last_error().
 */
#ifndef TORCHSIM_GB300_H
#define TORCHSIM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    TSG_OK = 0,
    TSG_ERR_ARGUMENT = -1,    /* bad sizes or null pointers: the reference's ValueError */
    TSG_ERR_UNSUPPORTED = -2, /* outside the served subset (single pool, instant RF) */
    TSG_ERR_CUDA = -3,        /* a CUDA runtime call failed */
    TSG_ERR_CAPACITY = -4     /* a size beyond a stated maximum */
};

/* Output layouts of the device entry points. */
enum {
    /* Two float planes (real, imaginary) as the reference's kernels write
     * them: real plane 0, imaginary plane m0*F+[0] (_epg_cpu.cpp:3111-3115). */
    TSG_LAYOUT_PLANES = 0,
    /* One interleaved complex64 array holding 1j * signal, which is what
     * MRFSimulator.evaluate returns (simulators/mrf.py:84): (-m0*F+[0], 0). */
    TSG_LAYOUT_COMPLEX_IJ = 1,
    /* One interleaved complex64 array holding the signal as the reference's
     * runs return it, complex(real plane, imaginary plane) = (0, m0*F+[0])
     * (sequence/_accelerators.py:3449). */
    TSG_LAYOUT_COMPLEX = 2
};

/* Structured forward-mode directions the fused kernel carries in one pass. */
enum {
    TSG_TANGENT_T1 = 1,
    TSG_TANGENT_T2 = 2,
    TSG_TANGENT_B1 = 4,
    TSG_TANGENT_INVERSION = 8
};

/* Per-voxel tissue, DEVICE pointers, atom_count floats each. m0, b1 and
 * inversion may be null for their identity value 1, as the reference's
 * feature mask leaves an undeclared property out (_epg_cpu.cpp:91-104). */
typedef struct {
    const float* t1_ms;
    const float* t2_ms;
    const float* m0;
    const float* b1;
    const float* inversion;
} tsg_tissue;

/* Per-voxel transmit phase (radians) and off-resonance (Hz) of the complex
 * path; each nullable (zero), the reference's B1phase and B0 buffers
 * (sequence/_parameters.py:234-241). */
typedef struct {
    const float* b1_phase_rad;
    const float* b0_hz;
} tsg_offaxis;

/* One general forward-mode direction (DEVICE pointers, all nullable):
 * per atom t1/t2/m0/b1/inversion, per (train, event) duration/flip. The
 * same directions simulate_real_jvp_range follows (_epg_cpu.cpp:3136-3285). */
typedef struct {
    const float* t1_ms;
    const float* t2_ms;
    const float* m0;
    const float* b1;
    const float* inversion;
    const float* duration_s;
    const float* flip_rad;
} tsg_direction;

/* The complex path's further forward-mode directions (DEVICE pointers,
 * nullable): per atom the transmit phase (radians) and off-resonance (Hz),
 * per (train, event) the phase (of a pulse, or of an ADC's receiver). The
 * reference's b1_phase, b0 and phase tangent slots (_epg_cpu.cpp:11071). */
typedef struct {
    const float* b1_phase_rad;
    const float* b0_hz;
    const float* phase_rad;
} tsg_offaxis_direction;

/* The complex path's further gradients (DEVICE pointers, nullable): per
 * atom the transmit phase and off-resonance, per (train, event) the phase
 * (of a pulse, or of an ADC's receiver). */
typedef struct {
    float* b1_phase_rad;
    float* b0_hz;
    float* phase_rad;
} tsg_offaxis_gradients;

/* Gradients the adjoint adds into (DEVICE pointers, nullable). Per atom:
 * t1/t2/m0/b1/inversion; per (train, event): flip and duration. The slots
 * simulate_real_vjp_range fills (_epg_cpu.cpp:6223-6231, 6180, 6217). */
typedef struct {
    float* t1_ms;
    float* t2_ms;
    float* m0;
    float* b1;
    float* inversion;
    float* flip_rad;
    float* duration_s;
} tsg_gradients;

/* Launch shape. Zero fields are chosen by the built-in heuristic.
 * lanes_per_voxel spreads the F+/F-/Z orders of one voxel over that many warp
 * lanes; orders_per_lane is how many orders each lane keeps in registers
 * (even for the sweeps); warps_per_block sets the voxels per CTA;
 * min_blocks_per_sm selects a register-budget variant compiled to keep that
 * many 128-thread blocks resident per SM (0: the default budget). */
typedef struct {
    int lanes_per_voxel;
    int orders_per_lane;
    int warps_per_block;
    int min_blocks_per_sm;
} tsg_launch;

typedef struct tsg_program tsg_program;

/* ---- diagnostics ------------------------------------------------------- */

const char* tsg_last_error(void);
int tsg_version(void);

/* Launches an FP32 FMA-throughput probe (blocks x threads, each running
 * eight independent FMA chains for 32*iters steps) on `stream`, and reports
 * the FLOPs it performs; timed by the caller with events, it gives the
 * FP32 CUDA-core peak that bounds the sweep kernels. `out` (blocks floats,
 * device) is written only to keep the chains live. No reference
 * counterpart: a measurement aid. */
int tsg_probe_fp32(int64_t blocks, int threads, int iters, float* out, void* stream,
                   double* flops);
/* The same probe written with paired FP32 FMAs (__ffma2_rn): four chains of
 * float2 per thread, the same FLOPs per launch. */
int tsg_probe_fp32x2(int64_t blocks, int threads, int iters, float* out, void* stream,
                     double* flops);

/* ---- pulse programs ---------------------------------------------------- */

/* Compiles the reference's packed event stream (HOST pointers) into a device
 * pulse program. Layout as _pack_events writes it (sequence/_accelerators.py:
 * 913-1170): duration_s and flip_rad are (train_count, event_count); kind,
 * action and output_index are (event_count). Events with zero duration are
 * folded into the op before them (exact: exp(0) = 1). unmerged != 0 keeps one
 * op per event with its relaxation step, which the per-event duration
 * gradients of tsg_epg_simulate_vjp need. duration_tangent (nullable, HOST,
 * train_count*event_count) keeps an op boundary wherever a zero-duration
 * event carries a duration direction. Allocates device memory. */
int tsg_program_create(const float* duration_s, const int32_t* kind, const float* flip_rad,
                       const uint8_t* action, const int32_t* output_index,
                       int64_t train_count, int64_t event_count, int unmerged,
                       const float* duration_tangent, tsg_program** out);
/* The same compilation keeping each event's phase (train_count*event_count,
 * radians): the program then also serves tsg_epg_forward_complex. Replaces
 * the phase buffer the reference's complex kernel reads per event
 * (_epg_cpu.cpp:4513-4532). */
int tsg_program_create_phased(const float* duration_s, const int32_t* kind, const float* flip_rad,
                              const float* phase_rad, const uint8_t* action,
                              const int32_t* output_index, int64_t train_count,
                              int64_t event_count, tsg_program** out);
int tsg_program_destroy(tsg_program* program);
/* The same compilation on the host only, for inspection: writes the op
 * count per train, the output count and up to `capacity` ops (all trains,
 * train-major) as dt, flip, record index and micro-step code words (bit
 * layout: relax 0, shifts-before-RF 1-2, RF kind 3-4 (1 rotate, 2 invert),
 * shifts-after-RF 5-6, spoil 7, record 8, shifts-after-record 9-10,
 * spoil 11). Needs no GPU. */
int tsg_program_plan(const float* duration_s, const int32_t* kind, const float* flip_rad,
                     const uint8_t* action, const int32_t* output_index, int64_t train_count,
                     int64_t event_count, int unmerged, const float* duration_tangent,
                     int64_t* op_count, int64_t* output_count, float* dt_out, float* flip_out,
                     int32_t* record_out, uint32_t* code_out, int64_t capacity);
/* op_count: ops per train; output_count: recorded samples per train. */
int tsg_program_info(const tsg_program* program, int64_t* train_count, int64_t* op_count,
                     int64_t* output_count, int64_t* event_count);

/* Rebinding a compiled program to new event values on the device, with no
 * host round trip (the role of the reference's affine rebinding of packed
 * buffers, model/_binding.py:94-268, for the pulse program): every op of
 * `program` takes its relaxation dt and its rotation flip from its source
 * events in `duration_s` and `flip_rad` (DEVICE, train_count*event_count),
 * and is written, with the template's micro-step codes and records, to
 * `device_ops` (DEVICE, train_count*op_count ops of 16 bytes). The new
 * durations must be zero wherever the template's were (those events were
 * folded into the op before them); a zero where the template had a
 * relaxation is exact, since a zero-length relaxation is the identity.
 * Stream-ordered. */
int tsg_program_rebind(const tsg_program* program, const float* duration_s,
                       const float* flip_rad, void* device_ops, void* stream);
/* A program handle over `device_ops` (rebound by tsg_program_rebind) that
 * borrows the template's structure and event source map; it must not
 * outlive the template or the op array, and tsg_program_destroy frees only
 * the handle. Allocates no device memory. */
int tsg_program_view(const tsg_program* program, void* device_ops, tsg_program** out);
/* out[i] = x[0] + ... + x[i], added left to right in float32 with one
 * rounding per addition (DEVICE buffers, one thread): the reference's
 * sequential float32 clock cursor (simulators/mrf.py:46-77) on the device. */
int tsg_sequential_sum(const float* x, int64_t n, float* out, void* stream);

/* ---- device-resident kernels ------------------------------------------- */

/* Complex forward (one pool, instant RF): RF and receiver phases of the
 * events, per-voxel transmit phase and off-resonance. Replaces the complex
 * kernel simulate_range<INSTANT, ONE> (_epg_cpu.cpp:4216-4566) that
 * _epg_cpu.simulate runs when real_axis != 1 (_epg_cpu.cpp:10860-10900).
 * `program` must come from tsg_program_create_phased. Outputs as for
 * tsg_epg_forward: PLANES = the reference's (real, imag) planes of the
 * recorded sample, COMPLEX_IJ = 1j times it, COMPLEX = it interleaved. */
int tsg_epg_forward_complex(const tsg_program* program, const tsg_tissue* tissue,
                            const tsg_offaxis* offaxis, int64_t atom_count, int64_t state_count,
                            int layout, float* out_a, float* out_b, const tsg_launch* launch,
                            void* stream);

/* The complex forward with its Jacobian columns in the same pass: T1, T2 and
 * B1 tangents (TSG_TANGENT_* bits; no inversion column) and the free M0
 * column, laid out as tsg_epg_forward_tangents lays them out. Replaces the
 * complex forward-mode kernel simulate_jvp_range (_epg_cpu.cpp:2470-3005)
 * that Simulator.jacobian runs off the real subspace, one tangent per pass. */
int tsg_epg_forward_tangents_complex(const tsg_program* program, const tsg_tissue* tissue,
                                     const tsg_offaxis* offaxis, int64_t atom_count,
                                     int64_t state_count, unsigned tangent_mask,
                                     const int32_t* columns, int32_t column_count, int layout,
                                     float* sig_a, float* sig_b, float* jac_a, float* jac_b,
                                     const tsg_launch* launch, void* stream);

/* Forward. Signal layout (train, atom, output); see TSG_LAYOUT_*. For
 * TSG_LAYOUT_PLANES out_b is the imaginary plane; for COMPLEX_IJ out_b is
 * unused. Follows simulate_real_range (_epg_cpu.cpp:3041-3128). */
int tsg_epg_forward(const tsg_program* program, const tsg_tissue* tissue, int64_t atom_count,
                    int64_t state_count, int layout, float* out_a, float* out_b,
                    const tsg_launch* launch, void* stream);

/* Fused forward plus structured tangents in ONE pass (replaces the
 * reference's k x (forward + jvp) launches of model/_signal.py:233-268).
 * tangent_mask: TSG_TANGENT_* bits. columns[5]: Jacobian column of the T1, T2,
 * B1, inversion and M0 derivatives (-1 = not stored); column_count = K. The
 * signal goes to sig_a/sig_b (nullable), the Jacobian to jac_a/jac_b as
 * (train, atom, K, output). */
int tsg_epg_forward_tangents(const tsg_program* program, const tsg_tissue* tissue,
                             int64_t atom_count, int64_t state_count, unsigned tangent_mask,
                             const int32_t* columns, int32_t column_count, int layout,
                             float* sig_a, float* sig_b, float* jac_a, float* jac_b,
                             const tsg_launch* launch, void* stream);

/* One general direction (the reference's simulate_jvp): writes the tangent
 * of the recorded samples only, planes layout, (train, atom, output). The
 * program must have been compiled with this direction's duration tangent. */
int tsg_epg_tangent(const tsg_program* program, const tsg_tissue* tissue, int64_t atom_count,
                    int64_t state_count, const tsg_direction* direction, float* out_real,
                    float* out_imag, const tsg_launch* launch, void* stream);

/* Forward (as tsg_epg_forward; outputs nullable) that also stores the state
 * entering every ops_per_checkpoint-th op into `checkpoints` (DEVICE,
 * train x ceil(ops/ops_per_checkpoint) x 3 x state_count x atom floats, atoms
 * innermost), the input of tsg_epg_adjoint. */
int tsg_epg_forward_checkpointed(const tsg_program* program, const tsg_tissue* tissue,
                                 int64_t atom_count, int64_t state_count, int layout, float* out_a,
                                 float* out_b, float* checkpoints, int ops_per_checkpoint,
                                 const tsg_launch* launch, void* stream);

/* Sizes for tsg_epg_adjoint: the segment length it will use (ops between
 * checkpoints; 0 = as long as the per-block shared-memory budget allows),
 * and the checkpoint and workspace bytes the caller allocates. */
int tsg_epg_adjoint_plan(const tsg_program* program, int64_t atom_count, int64_t state_count,
                         const tsg_launch* launch, int ops_per_checkpoint,
                         int* resolved_ops_per_checkpoint, int64_t* checkpoint_bytes,
                         int64_t* workspace_bytes);

/* Checkpointed first-order adjoint (the reference's simulate_real_vjp_range,
 * _epg_cpu.cpp:5985-6232): reverse sweep over segments of
 * ops_per_checkpoint ops re-run from the checkpoints of
 * tsg_epg_forward_checkpointed. `seed` is the cotangent of the recorded
 * samples: the imaginary plane (TSG_LAYOUT_PLANES) or the complex64 gradient
 * of 1j*signal (TSG_LAYOUT_COMPLEX_IJ). Gradients ADD into `gradients`
 * (nullable slots). `workspace` holds per-warp event partials and per-train
 * tissue partials, summed in a fixed order afterwards (deterministic). */
int tsg_epg_adjoint(const tsg_program* program, const tsg_tissue* tissue, int64_t atom_count,
                    int64_t state_count, const float* seed, int seed_layout,
                    const float* checkpoints, int ops_per_checkpoint,
                    const tsg_gradients* gradients, void* workspace, int64_t workspace_bytes,
                    const tsg_launch* launch, void* stream);

/* Size of the static scratch array behind tsg_epg_adjoint_noalloc. */
#define TSG_STATIC_SCRATCH_BYTES (32LL * 1024 * 1024)

/* The checkpointed adjoint for callers that cannot allocate device memory:
 * a service that plans all its memory at start-up, a framework whose caching
 * allocator owns the GPU, or a code path where an allocation would
 * synchronise the device. It has no counterpart in the reference, whose
 * adjoint allocates its trajectory per call. Inputs and outputs as for
 * tsg_epg_adjoint (gradients ADD into the given slots), but the checkpoints
 * and gradient partials live in one static device array of
 * TSG_STATIC_SCRATCH_BYTES (32 MiB) that every GPU loading this library holds
 * until the process exits; the entry point calls no cudaMalloc, cudaFree or
 * other allocating routine. A problem whose scratch exceeds the array is
 * rejected with TSG_ERR_CAPACITY (tsg_epg_adjoint_plan gives the sizes).
 * The first call on a device (and the first after the device's context is
 * replaced, e.g. by cudaDeviceReset) resolves the array's device address in
 * the current context (cudaGetSymbolAddress); make that first call before
 * any stream capture. All calls share the one array: calls whose work overlaps on the
 * GPU (other streams, other host threads) race on it and must be ordered by
 * the caller. Nothing a previous call left in it is read. */
int tsg_epg_adjoint_noalloc(const tsg_program* program, const tsg_tissue* tissue,
                            int64_t atom_count, int64_t state_count, const float* seed,
                            int seed_layout, const tsg_gradients* gradients,
                            const tsg_launch* launch, void* stream);
/* TSG_STATIC_SCRATCH_BYTES, as built into the library. */
int64_t tsg_static_scratch_bytes(void);

/* One general forward-mode direction on the complex path: the tangent of
 * the recorded sample along per-atom T1, T2, M0, B1, inversion (direction),
 * B1phase and B0 (offaxis_direction) and per-event duration, flip
 * (direction) and phase (offaxis_direction) at once. Replaces the complex
 * simulate_jvp_range (_epg_cpu.cpp:2470-3005) for one pool and instant RF.
 * A direction along a property the tissue does not declare (a null m0, b1,
 * inversion, B1phase or B0 map) is ignored, as the reference's feature mask
 * has it. Output layouts as tsg_epg_forward_complex. `program` from
 * tsg_program_create_phased. Stream-ordered; up to 128 states. */
int tsg_epg_tangent_complex(const tsg_program* program, const tsg_tissue* tissue,
                            const tsg_offaxis* offaxis, int64_t atom_count, int64_t state_count,
                            const tsg_direction* direction,
                            const tsg_offaxis_direction* offaxis_direction, int layout,
                            float* out_a, float* out_b, const tsg_launch* launch, void* stream);

/* ---- the complex path's first-order adjoint ----------------------------- */

/* Sizes of the complex adjoint's trajectory (every op's entry state: six
 * real planes; and every recorded F+[0]) and workspace. */
int tsg_epg_complex_adjoint_plan(const tsg_program* program, int64_t atom_count,
                                 int64_t state_count, const tsg_launch* launch,
                                 int64_t* trajectory_bytes, int64_t* workspace_bytes);

/* The complex forward (as tsg_epg_forward_complex; the output nullable) that
 * also stores the trajectory tsg_epg_adjoint_complex reads. The program is
 * built with event phases (tsg_program_create_phased). */
int tsg_epg_forward_complex_trajectory(const tsg_program* program, const tsg_tissue* tissue,
                                       const tsg_offaxis* offaxis, int64_t atom_count,
                                       int64_t state_count, int layout, float* out_a,
                                       float* out_b, void* trajectory, const tsg_launch* launch,
                                       void* stream);

/* First-order adjoint of the complex path (the reference's complex
 * simulate_vjp_range, _epg_cpu.cpp:4840-5985): `seed` is the complex
 * cotangent of the samples, two planes (TSG_LAYOUT_PLANES: seed_a real,
 * seed_b imaginary) or interleaved complex64 (TSG_LAYOUT_COMPLEX). Adds the
 * gradients of T1, T2, M0, B1, the inversion efficiency, flip and duration
 * into `gradients`, and of B1phase, B0 and the event phases into
 * `offaxis_gradients` (each nullable). Deterministic. */
int tsg_epg_adjoint_complex(const tsg_program* program, const tsg_tissue* tissue,
                            const tsg_offaxis* offaxis, int64_t atom_count, int64_t state_count,
                            const float* seed_a, const float* seed_b, int seed_layout,
                            const void* trajectory, const tsg_gradients* gradients,
                            const tsg_offaxis_gradients* offaxis_gradients, void* workspace,
                            int64_t workspace_bytes, const tsg_launch* launch, void* stream);

/* ---- second order: the adjoint of the tangent sweep --------------------- */

/* Sizes for the second-order sweeps along direction_count (1-3) directions:
 * the trajectory (every op's entry state of the signal state and of each
 * tangent, and every recorded F+[0]) and the workspace the caller allocates.
 * event_directions: whether any direction has duration or flip tangents. */
int tsg_epg_second_plan(const tsg_program* program, int64_t atom_count, int64_t state_count,
                        int direction_count, int event_directions, const tsg_launch* launch,
                        int64_t* trajectory_bytes, int64_t* workspace_bytes);

/* Forward of the signal and its derivatives along `directions` (DEVICE
 * pointers, tsg_direction per direction) in one pass, storing the trajectory
 * the reverse sweep reads. Signal (train, atom, output) and derivatives
 * (train, atom, K + with_m0, output) in `layout` (nullable); with with_m0 the
 * last column is the derivative along M0 (F+[0] itself), which needs no
 * tangent state. The program must have been compiled with every direction's
 * duration tangent (or unmerged). */
int tsg_epg_second_forward(const tsg_program* program, const tsg_tissue* tissue,
                           int64_t atom_count, int64_t state_count,
                           const tsg_direction* directions, int direction_count, int with_m0,
                           int layout,
                           float* sig_a, float* sig_b, float* jac_a, float* jac_b,
                           void* trajectory, void* workspace, const tsg_launch* launch,
                           void* stream);

/* The reverse sweep of that forward for the loss
 *   L = <seed_signal, s> + sum_k <seed_derivatives[k], J d_k>
 * (seeds as tsg_epg_adjoint takes them; seed_signal nullable, the
 * derivative seeds laid out as the forward writes the derivatives, with the
 * M0 column's when with_m0). Adds dL/d(inputs) into
 * `curvature` (for seed_signal alone this is the first-order adjoint, for the
 * derivative seeds the second-order term) and, into values[k], dL/d(d_k):
 * J^T seed_k over the tissue directions, and for a single direction also its
 * duration and flip. The reference's forward over reverse
 * (simulate_real_vjp_jvp_range, _epg_cpu.cpp:7028-7330) does one direction
 * per call; this sweep takes up to three. Deterministic (fixed-order sums). */
int tsg_epg_second_reverse(const tsg_program* program, const tsg_tissue* tissue,
                           int64_t atom_count, int64_t state_count,
                           const tsg_direction* directions, int direction_count, int with_m0,
                           const float* seed_signal, const float* seed_derivatives,
                           int seed_layout, const void* trajectory,
                           const tsg_gradients* curvature, const tsg_gradients* values,
                           void* workspace, int64_t workspace_bytes, const tsg_launch* launch,
                           void* stream);

/* The same two sweeps for a design cost: the directions are the unit
 * tangents of the properties in tangent_mask (TSG_TANGENT_T1 | T2 | B1, in
 * that order; the Jacobian columns a Cramer-Rao bound differentiates), so
 * the kernels carry no per-voxel or per-event direction and leave the terms
 * those directions zero out. The reverse writes the curvature only. */
int tsg_epg_design_plan(const tsg_program* program, int64_t atom_count, int64_t state_count,
                        unsigned tangent_mask, const tsg_launch* launch,
                        int64_t* trajectory_bytes, int64_t* workspace_bytes);
int tsg_epg_design_forward(const tsg_program* program, const tsg_tissue* tissue,
                           int64_t atom_count, int64_t state_count, unsigned tangent_mask,
                           int with_m0, int layout, float* sig_a, float* sig_b, float* jac_a,
                           float* jac_b, void* trajectory, const tsg_launch* launch,
                           void* stream);
int tsg_epg_design_reverse(const tsg_program* program, const tsg_tissue* tissue,
                           int64_t atom_count, int64_t state_count, unsigned tangent_mask,
                           int with_m0, const float* seed_signal, const float* seed_derivatives,
                           int seed_layout, const void* trajectory,
                           const tsg_gradients* curvature, void* workspace,
                           int64_t workspace_bytes, const tsg_launch* launch, void* stream);

/* ---- many sequences in one persistent launch ---------------------------- */

/* One sequence of a batch. Its ops are op_count consecutive entries of the
 * concatenated op array (16-byte ops as tsg_program_plan describes them:
 * float dt, float flip, int32 record, uint32 code); its voxels are
 * voxel_count consecutive entries of the tissue arrays from voxel_offset; its
 * samples are voxel_count x outputs complex64 from output_offset.
 * lanes_per_voxel = ceil(states / orders_per_lane) <= 32. */
typedef struct {
    int32_t op_offset;
    int32_t op_count;
    int32_t states;
    int32_t lanes_per_voxel;
    int32_t outputs;
    int32_t voxel_count;
    int64_t voxel_offset;
    int64_t output_offset;
} tsg_batch_sequence;

/* One unit of work: voxel_count voxels of a sequence from voxel_begin (at
 * most warps_per_block * floor(32 / lanes_per_voxel)). */
typedef struct {
    int32_t sequence;
    int32_t voxel_begin;
    int32_t voxel_count;
    int32_t reserved;
} tsg_batch_unit;

/* Forward of every unit in ONE persistent launch of `blocks` CTAs that take
 * units from `counter` (DEVICE int32, reset here with a memset on `stream`)
 * in list order; put the largest units first. All pointers are DEVICE
 * pointers. The output is TSG_LAYOUT_COMPLEX. orders_per_lane: 2, 4 or 8.
 * Capturable in a CUDA graph (a memset node and a kernel node). No
 * counterpart in the reference, which launches one kernel per sequence
 * (sequence/_epg_triton.py:17120-17300). */
int tsg_epg_batched_forward(const void* ops, const tsg_batch_sequence* sequences,
                            const tsg_batch_unit* units, int64_t unit_count, int32_t* counter,
                            const tsg_tissue* tissue, void* out, int orders_per_lane,
                            int warps_per_block, int blocks, void* stream);

/* ---- Gauss-Newton mapping ---------------------------------------------- */

/* One fused evaluation of Gauss-Newton normal equations (one train only):
 * forward plus the T1 and T2 tangents at the tissue given (natural T1, T2, M0,
 * and B1), reduced against the measured complex64 samples of the API signal
 * (row measured_rows[voxel], or the voxel's own row when null) to 10 doubles
 * per voxel: cost sum|s - y|^2, the upper triangle of J^T J by rows (T1T1,
 * T1T2, T1M0, T2T2, T2M0, M0M0) and sum dv*(v + Re y) (= J_s^T r), all in
 * natural parameters. Replaces the reference's forward + one forward+JVP pass
 * per column and the Jacobian blocks it stores (recon/_gauss_newton.py:
 * 633-651). */
int tsg_gn_evaluate(const tsg_program* program, const tsg_tissue* tissue, int64_t atom_count,
                    int64_t state_count, const void* measured, const int64_t* measured_rows,
                    double* normal_equations, const tsg_launch* launch, void* stream);

enum { TSG_GN_FIRST = 0, TSG_GN_LIVE = 1, TSG_GN_DONE = 2 };

/* Device-resident per-voxel Levenberg-Marquardt state (all DEVICE arrays of
 * voxel_count rows): free variables u (3), candidate (3), cost, accepted
 * normal equations (10, as tsg_gn_evaluate writes them), the candidate's
 * (10), damping, its rising factor, the predicted decrease, status
 * (TSG_GN_*), step flags (bit 0 short, bit 1 singular), steps taken, and the
 * candidate's natural T1, T2, M0 (float) for the next evaluation. */
typedef struct {
    double* u;
    double* cand;
    double* cost;
    double* normal;
    double* trial;
    double* damping;
    double* rising;
    double* predicted;
    int32_t* status;
    int32_t* flags;
    int32_t* iterations;
    float* t1;
    float* t2;
    float* m0;
} tsg_gn_state;

/* Bounds (low/high per T1, T2, M0; +-inf for none), TrustRegion tau, the
 * gradient and step tolerances and the step limit (GaussNewton's knobs,
 * recon/_gauss_newton.py:445-473). */
typedef struct {
    double low[3];
    double high[3];
    double tau;
    double gradient_tolerance;
    double step_tolerance;
    int32_t max_iterations;
} tsg_gn_config;

/* Retires flat voxels, solves the damped step (FP64 3x3 Cholesky) and writes
 * the candidate's natural parameters; FIRST voxels are evaluated where they
 * stand. */
int tsg_gn_step(const tsg_gn_state* state, int64_t voxel_count, const tsg_gn_config* config,
                void* stream);
/* After tsg_gn_evaluate at the candidates: the gain test and Nielsen damping
 * update of TrustRegion.judge (recon/_gauss_newton.py:395-411), acceptance,
 * and retirement on a short step or the step limit. */
int tsg_gn_judge(const tsg_gn_state* state, int64_t voxel_count, const tsg_gn_config* config,
                 void* stream);
/* Natural parameters (voxel_count x 3 floats) of free variables. */
int tsg_gn_natural(const double* free_variables, int64_t voxel_count, const tsg_gn_config* config,
                   float* natural, void* stream);

/* ---- dictionary matching (tensor cores) -------------------------------- */

/* Screens every voxel against every atom on the tensor cores and writes each
 * voxel's best tsg_match_candidates() atoms by |<s, d>|^2, best first.
 * queries: fp16 (query_rows x k), two rows per voxel whose products with an
 * atom row are Re and Im of <s, d>; atoms: fp16 (tsg_match_screen_rows(atom_count)
 * x k, rows permuted as described there); k a
 * multiple of 8; both 16-byte aligned, DEVICE. candidate_scores / _index:
 * (query_rows / 2) x candidates. `error` (device int, zero on entry) is set
 * if a pipeline wait ran out. Replaces the chunked FP32 products and top-k of
 * DictionaryMatcher._match_here (estimators/_dictionary.py:329-382). */
int tsg_match_screen(const void* queries, int64_t query_rows, const void* atoms,
                     int64_t atom_count, int64_t k, float* candidate_scores,
                     int32_t* candidate_index, int* error, void* stream);
/* Exact FP32 |<s, d>| of each voxel's candidates against the normalized
 * complex64 signals (voxels x samples) and atoms (atom_count x samples);
 * writes the best top_k (1..8) scores and atom indices, best
 * first. DEVICE pointers. */
int tsg_match_rescore(const void* signals, int64_t voxels, const void* atoms, int64_t atom_count,
                      int64_t samples, const int32_t* candidate_index, int top_k, float* scores,
                      int64_t* index, void* stream);
/* Candidates the screen keeps per voxel (32). */
int tsg_match_candidates(void);
/* Rows of the atom matrix tsg_match_screen reads for atom_count atoms (a
 * multiple of 64): atom i sits at row (i & 1) | ((i >> 1) & 1) << 5 |
 * ((i >> 2) & 15) << 1 | (i & ~63); the other rows are zero. */
int tsg_match_screen_rows(int64_t atom_count);

/* ---- drop-ins for the reference's native boundary (HOST pointers) ------ */

/* _epg_cpu.simulate (src/torchsim/_epg_cpu.cpp:10740-10926): pointers holds
 * the 26 packed buffers, the two output planes and the 13 tail slots (41
 * entries, :10794). real_axis == 1 runs the real-subspace kernel; any other
 * value the complex one (event phases, B1phase, B0), as the reference
 * switches between simulate_real_range and simulate_range. Synchronous. */
int tsg_epg_simulate(void* const* pointers, int64_t pointer_count, int64_t atom_count,
                     int64_t train_count, int64_t event_count, int64_t state_count,
                     int64_t output_count, int real_axis, int features);

/* _epg_cpu.simulate_jvp (src/torchsim/_epg_cpu.cpp:11017-11148): 26 packed
 * buffers, 20 tangents (the differentiable inputs, FLOAT_INPUTS order of
 * sequence/_parameters.py:206: 17 tissue, then duration, flip, phase), two
 * output planes, 13 tail slots (61). real_axis == 1 runs the real-subspace
 * tangent (simulate_real_jvp_range); any other value the complex one
 * (tsg_epg_tangent_complex, simulate_jvp_range), which also follows the
 * B1phase, B0 and event phase directions. Synchronous. */
int tsg_epg_simulate_jvp(void* const* pointers, int64_t pointer_count, int64_t atom_count,
                         int64_t train_count, int64_t event_count, int64_t state_count,
                         int64_t output_count, int real_axis, int features);

/* _epg_cpu.simulate_vjp (src/torchsim/_epg_cpu.cpp:11150-11400): 26 packed
 * buffers, two seed planes, 20 gradient slots (17 tissue, then flip, phase,
 * duration, the order of :11243-11253), 13 tail slots (61). The program is
 * compiled unmerged so that every event's duration gradient is formed.
 * Gradients are written (not accumulated). real_axis == 1 runs the real
 * subspace (only the imaginary seed plane acts; phase, B1phase and B0 are
 * written as zero); any other value the complex adjoint (both seed planes;
 * phase, B1phase and B0 gradients formed). Synchronous. */
int tsg_epg_simulate_vjp(void* const* pointers, int64_t pointer_count, int64_t atom_count,
                         int64_t train_count, int64_t event_count, int64_t state_count,
                         int64_t output_count, int real_axis, int features);

/* _epg_cpu.simulate_vjp_jvp (src/torchsim/_epg_cpu.cpp:11572-11760): 26
 * packed buffers, 20 tangents, two seed planes, 20 value gradients and 20
 * curvature gradients (each 17 tissue, then duration, flip, phase), 13 tail
 * slots (101). The value side is J^T seed, the curvature side the gradient
 * of <seed, J tangent> with respect to the inputs. Compiled unmerged;
 * gradients are written (not accumulated); phase and the tissue directions
 * the real subspace divides out are written as zero. Synchronous. */
int tsg_epg_simulate_vjp_jvp(void* const* pointers, int64_t pointer_count, int64_t atom_count,
                             int64_t train_count, int64_t event_count, int64_t state_count,
                             int64_t output_count, int real_axis, int features);

#ifdef __cplusplus
}
#endif

#endif /* TORCHSIM_GB300_H */
