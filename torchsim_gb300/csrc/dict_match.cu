// Dictionary matching on the 5th-generation tensor cores.
//
// The reference's DictionaryMatcher (estimators/_dictionary.py:52-420) scores
// every normalized measurement against every normalized atom by |<s, d>|
// through chunked FP32 matrix products (_grouped.py:212-240) and keeps the
// top k. Here one kernel does the product and the selection without ever
// writing the score matrix: queries (two rows per voxel) and atoms are fp16
// K-major tiles brought by TMA into a 4-stage shared-memory ring;
// `tcgen05.mma` (issued by one thread) accumulates a 128 x 256 tile in tensor
// memory, double-buffered so the epilogue of one atom tile overlaps the MMAs of
// the next; eight epilogue warps (two per TMEM lane quarter, each taking every
// other 32-column chunk) read the accumulator with `tcgen05.ld`. The two lanes
// holding a voxel's rows exchange one value per pair of atoms; each (warp,
// lane) keeps its best kScreen atoms of one (chunk parity, column parity)
// class, so a voxel keeps kCand = 32; the atoms are stored permuted so that
// neighbouring atoms land in different classes. A chunk of atoms whose best
// does not beat a lane's current last place costs no insertion work. A second kernel rescores
// those candidates exactly in FP32 against the complex signals and atoms and
// keeps the top k, so the fp16 screen decides only which few atoms are
// compared exactly.
//
// Rows of the query matrix: voxel v owns rows 2v and 2v+1. For real atoms
// (an SSFP fingerprint) they are (Re s_v, Im s_v) against the atom; for
// complex atoms (Re s, Im s) and (Im s, -Re s) against (Re d, Im d), whose
// products are the real and imaginary parts of <s, d>.
//
// Waits on mbarriers are bounded: a wait that runs out sets the error word
// and the kernel winds down instead of hanging.
#include <cuda.h>

#include "tsg_internal.h"

namespace tsg {

namespace {

constexpr int BM = 128, BN = 256, BK = 64, STAGES = 4;
constexpr int kScreen = 8;           // per lane
constexpr int kHalves = 2;            // epilogue warps per TMEM lane quarter
constexpr int kCand = 2 * kHalves * kScreen;  // per voxel
constexpr int SMEM_A = BM * BK * 2;
constexpr int SMEM_B = BN * BK * 2;
constexpr int STAGE_BYTES = SMEM_A + SMEM_B;
constexpr int TMEM_COLS = 2 * BN;
constexpr int kEpilogueThreads = 128 * kHalves;
// warp 0 TMA, warp 1 MMA + TMEM, warps 2.. epilogue (each lane quarter twice:
// one warp per half of the accumulator's columns).
constexpr int kThreads = 64 + kEpilogueThreads;
constexpr long long kWaitLimit = 1LL << 24;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ bool wait_parity(uint32_t bar, uint32_t parity) {
    for (long long i = 0; i < kWaitLimit; ++i) {
        uint32_t ok;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            "selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

// The screen matrix stores atom i at row pos(i), which moves bit 1 of i to
// bit 5 and bits 2-5 down by one, within blocks of 64: consecutive atoms then
// alternate in column parity and in 32-column chunk parity, so they fall in
// four different candidate lists of the voxel (dictionaries put neighbouring
// atoms next to each other). This is the inverse: the atom at row `pos`.
__host__ __device__ __forceinline__ int stored_atom(int pos) {
    return (pos & 1) | (((pos >> 5) & 1) << 1) | (((pos >> 1) & 15) << 2) | (pos & ~63);
}

__device__ __forceinline__ void arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// Shared-memory matrix descriptor of a K-major 16-bit tile with 128-byte
// swizzle: 8-row groups 1024 bytes apart, rows of 128 bytes.
__device__ __forceinline__ uint64_t tile_desc(uint32_t addr) {
    uint64_t d = 0;
    d |= uint64_t((addr & 0x3FFFF) >> 4);
    d |= uint64_t(16 >> 4) << 16;
    d |= uint64_t(1024 >> 4) << 32;
    d |= uint64_t(1) << 46;
    d |= uint64_t(2) << 61;
    return d;
}

// kind::f16 instruction descriptor: FP32 accumulate, fp16 A and B (format
// 0), both K-major, M = BM, N = BN.
constexpr uint32_t kInstr = (1u << 4) | (uint32_t(BN >> 3) << 17) | (uint32_t(BM >> 4) << 24);

struct ScreenShared {
    uint64_t full[STAGES];
    uint64_t empty[STAGES];
    uint64_t tfull[2];
    uint64_t tempty[2];
    uint32_t tmem_base;
    int abort;
};

#define TSG_LD32(r, taddr)                                                                         \
    asm volatile(                                                                                  \
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14," \
        "%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"             \
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),      \
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),  \
          "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),            \
          "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),            \
          "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])             \
        : "r"(taddr))

__global__ void __launch_bounds__(kThreads, 1)
    screen_kernel(const __grid_constant__ CUtensorMap qmap, const __grid_constant__ CUtensorMap amap,
                  int64_t rows, int64_t atoms, int64_t stored_rows, int k_tiles, float* cand_score,
                  int32_t* cand_index, int* error) {
    extern __shared__ uint8_t s_raw[];
    uint8_t* tiles = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(s_raw) + 1023) & ~uintptr_t(1023));
    ScreenShared* sh = reinterpret_cast<ScreenShared*>(tiles + STAGES * STAGE_BYTES);
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int64_t row0 = int64_t(blockIdx.x) * BM;
    const int n_tiles = int((stored_rows + BN - 1) / BN);

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&sh->full[s])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&sh->empty[s])));
        }
        for (int b = 0; b < 2; ++b) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&sh->tfull[b])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&sh->tempty[b])),
                         "r"(kEpilogueThreads));
        }
        sh->abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&sh->tmem_base)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = sh->tmem_base;
    volatile int* abort = &sh->abort;

    if (warp == 0) {
        if (lane == 0) {
            // TMA producer.
            int it = 0;
            for (int n = 0; n < n_tiles && !*abort; ++n) {
                for (int kt = 0; kt < k_tiles; ++kt, ++it) {
                    const int s = it % STAGES;
                    const uint32_t ph = (it / STAGES) & 1;
                    if (!wait_parity(smem_u32(&sh->empty[s]), ph ^ 1)) {
                        *abort = 1;
                        atomicExch(error, 1);
                        break;
                    }
                    const uint32_t full = smem_u32(&sh->full[s]);
                    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(full),
                                 "r"(STAGE_BYTES)
                                 : "memory");
                    const uint32_t a_dst = smem_u32(tiles + s * STAGE_BYTES);
                    const uint32_t b_dst = a_dst + SMEM_A;
                    asm volatile(
                        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes "
                        "[%0], [%1, {%2, %3}], [%4];" ::"r"(a_dst),
                        "l"(reinterpret_cast<uint64_t>(&qmap)), "r"(kt * BK), "r"(int(row0)), "r"(full)
                        : "memory");
                    asm volatile(
                        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes "
                        "[%0], [%1, {%2, %3}], [%4];" ::"r"(b_dst),
                        "l"(reinterpret_cast<uint64_t>(&amap)), "r"(kt * BK), "r"(n * BN), "r"(full)
                        : "memory");
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // MMA issuer.
            int it = 0;
            for (int n = 0; n < n_tiles && !*abort; ++n) {
                const int b = n & 1;
                const uint32_t use = uint32_t(n >> 1);
                if (!wait_parity(smem_u32(&sh->tempty[b]), (use & 1) ^ 1)) {
                    *abort = 1;
                    atomicExch(error, 2);
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t d = tmem + uint32_t(b * BN);
                for (int kt = 0; kt < k_tiles; ++kt, ++it) {
                    const int s = it % STAGES;
                    const uint32_t ph = (it / STAGES) & 1;
                    if (!wait_parity(smem_u32(&sh->full[s]), ph)) {
                        *abort = 1;
                        atomicExch(error, 3);
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t a_addr = smem_u32(tiles + s * STAGE_BYTES);
                    const uint32_t b_addr = a_addr + SMEM_A;
#pragma unroll
                    for (int j = 0; j < BK / 16; ++j) {
                        const uint64_t adesc = tile_desc(a_addr + j * 32);
                        const uint64_t bdesc = tile_desc(b_addr + j * 32);
                        const uint32_t acc = (kt > 0 || j > 0) ? 1u : 0u;
                        asm volatile(
                            "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
                            "l"(adesc), "l"(bdesc), "r"(kInstr), "r"(acc)
                            : "memory");
                    }
                    asm volatile(
                        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                            smem_u32(&sh->empty[s]))
                        : "memory");
                }
                if (*abort) break;
                asm volatile(
                    "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                        smem_u32(&sh->tfull[b]))
                    : "memory");
            }
        }
    } else {
        // Epilogue: warp w reads TMEM lanes 32 (w % 4) .. +31 = tile rows, in
        // the columns of its half of the accumulator. A voxel's rows sit on
        // lanes 2i (Re) and 2i+1 (Im); lane parity p scores the atoms of
        // column parity p.
        const int quarter = warp & 3;
        const int half = (warp - 2) / 4;
        const int r = quarter * 32 + lane;
        const int parity = lane & 1;
        float best_s[kScreen];
        int best_i[kScreen];
#pragma unroll
        for (int k = 0; k < kScreen; ++k) {
            best_s[k] = -1.f;
            best_i[k] = -1;
        }
        for (int n = 0; n < n_tiles && !*abort; ++n) {
            const int b = n & 1;
            const uint32_t use = uint32_t(n >> 1);
            if (!wait_parity(smem_u32(&sh->tfull[b]), use & 1)) {
                *abort = 1;
                atomicExch(error, 4);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll 1
            for (int cc = 0; cc < BN / 64; ++cc) {
                // The warp of half h takes the 32-column chunks of parity h.
                const int c = 2 * cc + half;
                uint32_t v[32];
                const uint32_t taddr = tmem + (uint32_t(quarter * 32) << 16) + uint32_t(b * BN + c * 32);
                TSG_LD32(v, taddr);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                float sc[16];
                float chunk_best = -1.f;
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const float x0 = __uint_as_float(v[2 * j]), x1 = __uint_as_float(v[2 * j + 1]);
                    // Send the partner the value of its column; keep our own.
                    const float mine = parity ? x1 : x0;
                    const float other = __shfl_xor_sync(0xffffffffu, parity ? x0 : x1, 1);
                    sc[j] = fmaf(mine, mine, other * other);
                    chunk_best = fmaxf(chunk_best, sc[j]);
                }
                if (chunk_best > best_s[kScreen - 1]) {
                    const int pos0 = n * BN + c * 32 + parity;
#pragma unroll 1
                    for (int j = 0; j < 16; ++j) {
                        const int atom = stored_atom(pos0 + 2 * j);
                        const float score = sc[j];
                        if (atom < atoms && score > best_s[kScreen - 1]) {
                            best_s[kScreen - 1] = score;
                            best_i[kScreen - 1] = atom;
#pragma unroll
                            for (int k = kScreen - 1; k > 0; --k) {
                                if (best_s[k] > best_s[k - 1]) {
                                    const float ts = best_s[k];
                                    best_s[k] = best_s[k - 1];
                                    best_s[k - 1] = ts;
                                    const int ti = best_i[k];
                                    best_i[k] = best_i[k - 1];
                                    best_i[k - 1] = ti;
                                }
                            }
                        }
                    }
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            arrive(smem_u32(&sh->tempty[b]));
        }
        const int64_t row = row0 + (r & ~1);
        if (row < rows) {
            const int64_t voxel = row >> 1;
#pragma unroll
            for (int k = 0; k < kScreen; ++k) {
                cand_score[voxel * kCand + (half * 2 + parity) * kScreen + k] = best_s[k];
                cand_index[voxel * kCand + (half * 2 + parity) * kScreen + k] = best_i[k];
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (*abort) {
        // Let copies and products in flight land before the memory goes away.
        for (int i = 0; i < 64; ++i) __nanosleep(1000);
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(TMEM_COLS));
}

// Exact FP32 rescoring of each voxel's screened candidates against the complex
// normalized signal and atoms; keeps the best `top_k` in descending order.
// One warp per voxel: lanes stride over the samples.
__global__ void rescore_kernel(const float2* __restrict__ signals, const float2* __restrict__ atoms,
                               int64_t voxels, int64_t samples, const int32_t* __restrict__ cand,
                               int top_k, float* __restrict__ scores, int64_t* __restrict__ index) {
    const int64_t voxel = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (voxel >= voxels) return;
    const float2* s = signals + voxel * samples;
    float best_s[kCand];
    int best_i[kCand];
#pragma unroll 4
    for (int k = 0; k < kCand; ++k) {
        const int a = cand[voxel * kCand + k];
        float re = 0.f, im = 0.f;
        if (a >= 0) {
            const float2* d = atoms + int64_t(a) * samples;
            for (int64_t p = lane; p < samples; p += 32) {
                const float2 x = s[p], y = d[p];
                // s * conj(d)
                re = fmaf(x.x, y.x, fmaf(x.y, y.y, re));
                im = fmaf(x.y, y.x, fmaf(-x.x, y.y, im));
            }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            re += __shfl_xor_sync(0xffffffffu, re, off);
            im += __shfl_xor_sync(0xffffffffu, im, off);
        }
        best_s[k] = a >= 0 ? sqrtf(re * re + im * im) : -1.f;
        best_i[k] = a;
    }
    if (lane != 0) return;
    // Descending by score, ties to the lower atom index.
    for (int k = 0; k < top_k; ++k) {
        int pick = k;
        for (int j = k + 1; j < kCand; ++j) {
            const bool better = best_s[j] > best_s[pick] ||
                                (best_s[j] == best_s[pick] && best_i[j] >= 0 &&
                                 (best_i[pick] < 0 || best_i[j] < best_i[pick]));
            if (better) pick = j;
        }
        const float ts = best_s[k];
        best_s[k] = best_s[pick];
        best_s[pick] = ts;
        const int ti = best_i[k];
        best_i[k] = best_i[pick];
        best_i[pick] = ti;
        scores[voxel * top_k + k] = best_s[k];
        index[voxel * top_k + k] = best_i[k];
    }
}

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                 const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                 const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                 CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn() {
    static EncodeTiled fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return EncodeTiled(nullptr);
        return reinterpret_cast<EncodeTiled>(p);
    }();
    return fn;
}

int tile_map(CUtensorMap* map, const void* base, int64_t rows, int64_t k, int box_rows) {
    EncodeTiled fn = encode_fn();
    if (!fn) return fail(TSG_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");
    const cuuint64_t dims[2] = {cuuint64_t(k), cuuint64_t(rows)};
    const cuuint64_t strides[1] = {cuuint64_t(k) * 2};
    const cuuint32_t box[2] = {cuuint32_t(BK), cuuint32_t(box_rows)};
    const cuuint32_t elem[2] = {1, 1};
    const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void*>(base), dims,
                          strides, box, elem, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(TSG_ERR_ARGUMENT, "tensor map rejected the matrix");
    return TSG_OK;
}

}  // namespace

}  // namespace tsg

using namespace tsg;

extern "C" int tsg_match_screen_rows(int64_t atom_count) {
    return int((atom_count + 63) / 64 * 64);
}

extern "C" int tsg_match_screen(const void* queries, int64_t query_rows, const void* atoms,
                                int64_t atom_count, int64_t k, float* candidate_scores,
                                int32_t* candidate_index, int* error, void* stream) {
    if (query_rows < 0 || atom_count < 0 || k < 1)
        return fail(TSG_ERR_ARGUMENT, "invalid matching dimensions");
    if (query_rows % 2) return fail(TSG_ERR_ARGUMENT, "queries come as two rows per voxel");
    if (k % 8) return fail(TSG_ERR_ARGUMENT, "the inner dimension must be a multiple of 8 (16 bytes)");
    if (query_rows == 0) return TSG_OK;
    if (!queries || !atoms || !candidate_scores || !candidate_index || !error)
        return fail(TSG_ERR_ARGUMENT, "null matching buffer");
    if ((reinterpret_cast<uintptr_t>(queries) | reinterpret_cast<uintptr_t>(atoms)) & 15)
        return fail(TSG_ERR_ARGUMENT, "matrices must be 16-byte aligned");
    if (atom_count == 0) return fail(TSG_ERR_ARGUMENT, "empty dictionary");
    if (query_rows > (int64_t(1) << 31) || atom_count > (int64_t(1) << 31) - BN)
        return fail(TSG_ERR_CAPACITY, "matrix too large");
    CUtensorMap qmap, amap;
    const int64_t stored_rows = (atom_count + 63) / 64 * 64;
    int rc = tile_map(&qmap, queries, query_rows, k, BM);
    if (!rc) rc = tile_map(&amap, atoms, stored_rows, k, BN);
    if (rc) return rc;
    const size_t smem = 1024 + STAGES * STAGE_BYTES + sizeof(ScreenShared);
    TSG_CUDA(cudaFuncSetAttribute(screen_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    const int k_tiles = int((k + BK - 1) / BK);
    const unsigned blocks = unsigned((query_rows + BM - 1) / BM);
    screen_kernel<<<blocks, kThreads, smem, static_cast<cudaStream_t>(stream)>>>(
        qmap, amap, query_rows, atom_count, stored_rows, k_tiles, candidate_scores,
        candidate_index, error);
    TSG_CUDA(cudaGetLastError());
    return TSG_OK;
}

extern "C" int tsg_match_rescore(const void* signals, int64_t voxels, const void* atoms,
                                 int64_t atom_count, int64_t samples,
                                 const int32_t* candidate_index, int top_k, float* scores,
                                 int64_t* index, void* stream) {
    if (voxels < 0 || atom_count < 1 || samples < 1 || top_k < 1 || top_k > 8)
        return fail(TSG_ERR_ARGUMENT, "invalid rescoring dimensions (top_k must be 1..8)");
    if (voxels == 0) return TSG_OK;
    if (!signals || !atoms || !candidate_index || !scores || !index)
        return fail(TSG_ERR_ARGUMENT, "null rescoring buffer");
    const int64_t threads = voxels * 32;
    const unsigned blocks = unsigned((threads + 255) / 256);
    rescore_kernel<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const float2*>(signals), static_cast<const float2*>(atoms), voxels, samples,
        candidate_index, top_k, scores, index);
    TSG_CUDA(cudaGetLastError());
    return TSG_OK;
}

extern "C" int tsg_match_candidates(void) { return kCand; }
