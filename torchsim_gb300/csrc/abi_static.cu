// The adjoint for callers that cannot allocate device memory.
//
// Some callers own every byte of device memory themselves: a reconstruction
// service that plans its memory once at start-up and must not allocate in its
// steady state, a host framework whose caching allocator owns the GPU (an
// allocation from outside it fragments that pool or fails against its
// reservation), or a code path where a cudaMalloc would synchronise the
// device. tsg_epg_adjoint asks them for checkpoint and workspace buffers;
// this entry point takes the same inputs and outputs but keeps its scratch
// (the state checkpoints and the per-warp gradient partials) in one
// file-scope device array of fixed size, so it calls no cudaMalloc,
// cudaFree or allocating routine of any library.
#include <cuda.h>

#include <mutex>

#include "tsg_internal.h"

extern "C" int tsg_epg_forward_checkpointed(const tsg_program*, const tsg_tissue*, int64_t, int64_t,
                                            int, float*, float*, float*, int, const tsg_launch*,
                                            void*);
extern "C" int tsg_epg_adjoint_plan(const tsg_program*, int64_t, int64_t, const tsg_launch*, int,
                                    int*, int64_t*, int64_t*);
extern "C" int tsg_epg_adjoint(const tsg_program*, const tsg_tissue*, int64_t, int64_t,
                               const float*, int, const float*, int, const tsg_gradients*, void*,
                               int64_t, const tsg_launch*, void*);

namespace tsg {
namespace {

constexpr int64_t kStaticScratchBytes = TSG_STATIC_SCRATCH_BYTES;

// The scratch itself. In host code this name is only a host-side stand-in
// for the array; its device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;

// The array's address as resolved in one context of a device. A module (and
// so the array) lives in a context: after cudaDeviceReset, or in another
// context on the same device, the array is loaded again elsewhere, so an
// address is reused only while the context it was resolved in is current.
struct Resolved {
    CUcontext context;
    void* address;
};
Resolved g_resolved[kMaxDevices] = {};

using CtxGetCurrent = CUresult (*)(CUcontext*);

// The driver's cuCtxGetCurrent, through the runtime's entry-point query (the
// library links only the CUDA runtime).
CtxGetCurrent context_query() {
    static CtxGetCurrent fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault,
                                             &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return CtxGetCurrent(nullptr);
        return reinterpret_cast<CtxGetCurrent>(p);
    }();
    return fn;
}

// Resolves the array's address for the current device and context, once per
// context (cudaGetSymbolAddress also makes the device's primary context
// current on a thread that has none yet).
int scratch_address(void** out) {
    int device = 0;
    TSG_CUDA(cudaGetDevice(&device));
    if (device < 0 || device >= kMaxDevices) return fail(TSG_ERR_CAPACITY, "device index beyond 64");
    CtxGetCurrent query = context_query();
    if (query == nullptr) return fail(TSG_ERR_CUDA, "cuCtxGetCurrent is unavailable");
    std::lock_guard<std::mutex> guard(g_setup_mutex);
    CUcontext context = nullptr;
    if (query(&context) != CUDA_SUCCESS) return fail(TSG_ERR_CUDA, "cuCtxGetCurrent failed");
    Resolved& slot = g_resolved[device];
    if (context == nullptr || slot.address == nullptr || slot.context != context) {
        void* ptr = nullptr;
        cudaError_t err = cudaGetSymbolAddress(&ptr, g_scratch);
        if (err != cudaSuccess) return cuda_fail(err, "cudaGetSymbolAddress(scratch)");
        if (query(&context) != CUDA_SUCCESS || context == nullptr)
            return fail(TSG_ERR_CUDA, "no current context after resolving the scratch array");
        slot = Resolved{context, ptr};
    }
    *out = slot.address;
    return TSG_OK;
}

}  // namespace
}  // namespace tsg

using namespace tsg;

extern "C" int64_t tsg_static_scratch_bytes(void) { return kStaticScratchBytes; }

extern "C" int tsg_epg_adjoint_noalloc(const tsg_program* program, const tsg_tissue* tissue,
                                       int64_t atom_count, int64_t state_count, const float* seed,
                                       int seed_layout, const tsg_gradients* gradients,
                                       const tsg_launch* launch, void* stream) {
    int ops_per_checkpoint = 0;
    int64_t ckpt_bytes = 0, work_bytes = 0;
    int rc = tsg_epg_adjoint_plan(program, atom_count, state_count, launch, 0, &ops_per_checkpoint,
                                  &ckpt_bytes, &work_bytes);
    if (rc) return rc;
    const int64_t ckpt_span = (ckpt_bytes + 255) / 256 * 256;
    if (ckpt_span + work_bytes > kStaticScratchBytes)
        return fail(TSG_ERR_CAPACITY,
                    "the no-allocation adjoint needs " + std::to_string(ckpt_span + work_bytes) +
                        " bytes of scratch; its static array holds " +
                        std::to_string(kStaticScratchBytes) + " (use tsg_epg_adjoint)");
    if (atom_count == 0) return TSG_OK;
    void* base = nullptr;
    rc = scratch_address(&base);
    if (rc) return rc;
    // Checkpoints first, then the gradient partials. The forward writes every
    // checkpoint the reverse reads and the reverse writes every partial the
    // reductions read, so nothing left by an earlier call is ever read.
    float* ckpt = static_cast<float*>(base);
    void* work = static_cast<unsigned char*>(base) + ckpt_span;
    rc = tsg_epg_forward_checkpointed(program, tissue, atom_count, state_count, TSG_LAYOUT_PLANES,
                                      nullptr, nullptr, ckpt, ops_per_checkpoint, launch, stream);
    if (rc) return rc;
    return tsg_epg_adjoint(program, tissue, atom_count, state_count, seed, seed_layout, ckpt,
                           ops_per_checkpoint, gradients, work, work_bytes, launch, stream);
}
