// check_noalloc.cu -- the allocation-invariant check without any allocation.
//
// pbm_check_ids needs scratch memory: one "seen" bit per page to catch a page
// handed to two requesters, plus a few counters.  It takes that scratch from
// its pool, which was set up with cudaMalloc.  Some callers cannot call
// cudaMalloc at all: a database engine that hands every byte of device
// memory to its own buffer pool up front, or a process that must not grow
// its device footprint after start-up (a cudaMalloc there either fails or
// takes memory the engine has already promised elsewhere).  For them,
// pbm_check_ids_noalloc works on buffers the caller already has (the bitmap
// and the id list) and keeps its scratch in the static array below, which
// exists once per GPU that loads this library and stays allocated until the
// process exits.
//
// Limits and sharing rules:
//   * at most kNoAllocMaxPages pages (8,388,608 pages: 1 MiB of seen bits);
//     larger pools are rejected with PBM_ERR_INVALID, and so are id lists
//     longer than INT32_MAX (ids are int32 page numbers);
//   * every call uses the same scratch array.  Each call clears it before use,
//     but two calls whose work overlaps on the GPU (different streams, or
//     different host threads) race on it and give wrong counts: serialise them;
//   * the call waits for its stream before it returns (it reads the counters
//     back to the host);
//   * the first call on a device (in each CUDA context of that device) looks
//     up the array's device address with cudaGetSymbolAddress, a set-up step
//     that is not a stream operation, so make that first call before any
//     stream capture starts.
#include <mutex>

#include "internal.cuh"

namespace pbm {
namespace {

constexpr uint64_t kNoAllocMaxPages = 1ull << 23;
constexpr size_t kSeenWords = (size_t)(kNoAllocMaxPages / 32);   // 32-bit words
constexpr size_t kCounterWords = 2 * 8;                         // 8 64-bit counters
constexpr int kMaxDevices = 64;

// The scratch: seen bits first, then the counters (64-bit aligned).
static __device__ __align__(256) uint32_t g_noalloc_scratch[kSeenWords + kCounterWords];

struct Counters {
    unsigned long long ok, failed, out_of_range, duplicates, not_marked, used, pad0, pad1;
};

std::mutex g_setup_mu;
struct ScratchSlot {
    unsigned long long ctx_id;   // the context the address belongs to (0: not looked up yet)
    uint32_t* ptr;
};
ScratchSlot g_scratch[kMaxDevices] = {};

// Identity of the current CUDA context, from the driver's cuCtxGetCurrent and
// cuCtxGetId (reached through the runtime's entry-point query, so the library
// does not link libcuda).  A device reset makes a new context with a new id,
// and the array's address is then looked up again.  Returns 0 if unknown.
unsigned long long current_context_id() {
    using GetCurrent = int (*)(void**);
    using GetId = int (*)(void*, unsigned long long*);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        cudaDriverEntryPointQueryResult q1, q2;
        void* f1 = nullptr;
        void* f2 = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
            q1 == cudaDriverEntryPointSuccess && q2 == cudaDriverEntryPointSuccess) {
            get_current = (GetCurrent)f1;
            get_id = (GetId)f2;
        }
        cudaGetLastError();
    }
    void* ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
    return id;
}

// Device address of the scratch on the current device, looked up once per
// device and context with that device current.  Host code must not use the
// symbol g_noalloc_scratch itself as an address: on the host it is a stand-in.
int scratch_address(uint32_t** out) {
    int dev = 0;
    PBM_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return PBM_ERR_INVALID;
    const unsigned long long ctx = current_context_id();   // 0 before the context exists
    std::lock_guard<std::mutex> lk(g_setup_mu);
    ScratchSlot& slot = g_scratch[dev];
    if (!slot.ptr || ctx == 0 || slot.ctx_id != ctx) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            std::fprintf(stderr, "[pbm] cudaGetSymbolAddress(no-alloc scratch) failed: %s\n",
                         cudaGetErrorString(e));
            cudaGetLastError();
            return PBM_ERR_CUDA;
        }
        slot.ptr = (uint32_t*)p;
        slot.ctx_id = current_context_id();   // the lookup has made the context current
    }
    *out = slot.ptr;
    return PBM_OK;
}

__device__ __forceinline__ unsigned long long warp_sum(unsigned long long v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_down_sync(0xffffffffu, v, d);
    return v;
}

__global__ void __launch_bounds__(256) k_noalloc_check(const uint32_t* words, uint64_t n_pages,
                                                       const int32_t* ids, uint32_t n, uint32_t* seen,
                                                       Counters* out) {
    unsigned long long ok = 0, failed = 0, oor = 0, dup = 0, unmarked = 0;
    const uint64_t n_round = ((uint64_t)n + 31u) & ~31ull;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_round; i += (uint64_t)gridDim.x * blockDim.x) {
        if (i >= n) continue;
        int32_t id = ids[i];
        if (id == -1) { ++failed; continue; }
        if (id < 0 || (uint64_t)id >= n_pages) { ++oor; continue; }
        ++ok;
        uint32_t w = (uint32_t)id >> 5, bit = 1u << ((uint32_t)id & 31u);
        if (atomicOr(seen + w, bit) & bit) ++dup;
        if (!(__ldcg(words + w) & bit)) ++unmarked;
    }
    ok = warp_sum(ok);
    failed = warp_sum(failed);
    oor = warp_sum(oor);
    dup = warp_sum(dup);
    unmarked = warp_sum(unmarked);
    if ((threadIdx.x & 31u) == 0) {
        if (ok) atomicAdd(&out->ok, ok);
        if (failed) atomicAdd(&out->failed, failed);
        if (oor) atomicAdd(&out->out_of_range, oor);
        if (dup) atomicAdd(&out->duplicates, dup);
        if (unmarked) atomicAdd(&out->not_marked, unmarked);
    }
}

// Held pages among the first n_pages bits (padding bits are not counted).
__global__ void __launch_bounds__(256) k_noalloc_used(const uint32_t* words, uint64_t n_pages, Counters* out) {
    const uint32_t full = (uint32_t)(n_pages / 32u);
    const uint32_t tail = (uint32_t)(n_pages % 32u);
    unsigned long long c = 0;
    const uint32_t total = full + (tail ? 1u : 0u);
    const uint64_t n_round = ((uint64_t)total + 31u) & ~31ull;
    for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w < n_round; w += (uint64_t)gridDim.x * blockDim.x) {
        if (w >= total) continue;
        uint32_t v = __ldcg(words + w);
        if (w == full) v &= (1u << tail) - 1u;
        c += (unsigned long long)__popc(v);
    }
    c = warp_sum(c);
    if ((threadIdx.x & 31u) == 0 && c) atomicAdd(&out->used, c);
}

}  // namespace
}  // namespace pbm

using namespace pbm;

extern "C" int pbm_check_ids_noalloc(const uint32_t* d_bitmap, uint64_t n_pages, const int32_t* d_ids,
                                     uint32_t n, pbm_check_result* h_out, void* stream) {
    if (!d_bitmap || !h_out || (n && !d_ids) || n_pages == 0) return PBM_ERR_INVALID;
    if (n > (uint32_t)INT32_MAX) {
        std::fprintf(stderr, "[pbm] pbm_check_ids_noalloc: %u ids exceed INT32_MAX\n", n);
        return PBM_ERR_INVALID;
    }
    if (n_pages > kNoAllocMaxPages) {
        std::fprintf(stderr,
                     "[pbm] pbm_check_ids_noalloc: %llu pages exceed the no-alloc limit of %llu pages\n",
                     (unsigned long long)n_pages, (unsigned long long)kNoAllocMaxPages);
        return PBM_ERR_INVALID;
    }
    cudaStream_t s = (cudaStream_t)stream;
    uint32_t* scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc) return rc;
    uint32_t* seen = scratch;
    Counters* ctr = reinterpret_cast<Counters*>(scratch + kSeenWords);
    // the scratch keeps the previous call's contents: clear what this call uses
    const size_t seen_bytes = (size_t)((n_pages + 31u) / 32u) * 4u;
    PBM_CUDA_TRY(cudaMemsetAsync(seen, 0, seen_bytes, s));
    PBM_CUDA_TRY(cudaMemsetAsync(ctr, 0, sizeof(Counters), s));
    const int sms = sm_count();
    if (n) {
        int blocks = (int)((n + 255u) / 256u);
        if (blocks > sms * 8) blocks = sms * 8;
        k_noalloc_check<<<blocks, 256, 0, s>>>(d_bitmap, n_pages, d_ids, n, seen, ctr);
        PBM_LAUNCH_CHECK();
    }
    {
        uint32_t nw = (uint32_t)((n_pages + 31u) / 32u);
        int blocks = (int)((nw + 255u) / 256u);
        if (blocks > sms * 4) blocks = sms * 4;
        if (blocks < 1) blocks = 1;
        k_noalloc_used<<<blocks, 256, 0, s>>>(d_bitmap, n_pages, ctr);
        PBM_LAUNCH_CHECK();
    }
    Counters h{};
    PBM_CUDA_TRY(cudaMemcpyAsync(&h, ctr, sizeof(h), cudaMemcpyDeviceToHost, s));
    PBM_CUDA_TRY(cudaStreamSynchronize(s));
    h_out->n_ok = (int64_t)h.ok;
    h_out->n_failed = (int64_t)h.failed;
    h_out->n_out_of_range = (int64_t)h.out_of_range;
    h_out->n_duplicates = (int64_t)h.duplicates;
    h_out->n_not_marked = (int64_t)h.not_marked;
    h_out->used_pages = (int64_t)h.used;
    return (h.out_of_range || h.duplicates || h.not_marked) ? PBM_ERR_CORRUPT : PBM_OK;
}
