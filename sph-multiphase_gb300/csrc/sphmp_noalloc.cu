// sphmp_noalloc.cu — the cell sort (what GetGridListCUDA computes) into buffers
// the caller owns, with no device allocation at all.
//
// Some callers cannot let a library allocate device memory: a host application
// that owns the whole device through its own memory pool, a frame loop where the
// implicit device synchronisation of cudaMalloc/cudaFree is not acceptable, or
// an FFI caller that wants no library-held allocations to outlive the call.
// sphmp_sort_cells_noalloc serves them: its only scratch is the file-scope
// static device array below, fixed at load time, whose address is looked up once
// per CUDA context. It calls no cudaMalloc/cudaFree and no allocating library.
//
// Limits: n <= SPHMP_NOALLOC_MAX_PARTICLES, gridtotal <= SPHMP_NOALLOC_MAX_CELLS
// and at most kNaMaxCellMembers particles in one cell; larger inputs are
// rejected with an error before anything runs (cell occupancy: after the sort,
// from a device flag).
//
// The scratch address is looked up once per CUDA context (the device's primary
// context, or a context the caller made current), by the first call made in
// that context, and kept with the context's unique id: after a
// cudaDeviceReset the next call sees a new id and looks the address up again.
// Every call copies the error word to the host and synchronises `stream`, so no
// call can be made while the stream is being captured into a CUDA graph.
//
// Every call clears, on the stream, the scratch that has to start at zero (the
// per-cell counters, the scatter cursors, the per-chunk out-of-grid counts and
// the error word) before using it; nothing relies on the array's zero
// initialisation. All calls on one device share the one scratch array, so calls
// that overlap in time (two streams, two host threads) race on it and give wrong
// results: serialise them on one stream or synchronise between them.
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "sphmp.h"
#include "sphmp_internal.h"

namespace sphmp {
namespace {

constexpr uint32_t kNaUndef = 0xFFFFFFFFu;
constexpr int kNaThreads = 256;
constexpr int kNaMaxParticles = SPHMP_NOALLOC_MAX_PARTICLES;
constexpr int kNaMaxCells = SPHMP_NOALLOC_MAX_CELLS;
constexpr int kNaMaxCellMembers = 4096;
constexpr int kNaChunks = (kNaMaxParticles + kNaThreads - 1) / kNaThreads;
constexpr uint32_t kNaErrKey = 1u;       // a key that is neither a cell id nor GRID_UNDEF
constexpr uint32_t kNaErrCellSize = 2u;  // a cell above kNaMaxCellMembers

// Scratch layout (32-bit words):
//   count [G + 1]   particles per cell; entry G is cleared and never counted
//                   into (out-of-grid keys are counted per chunk instead), so
//                   that start[G] is the in-grid total, where the out-of-grid
//                   tail begins
//   start [G + 2]   exclusive prefix of count; start[G + 1] = n
//   cursor[G + 1]   scatter cursors
//   chunk [kNaChunks] out-of-grid keys per 256-key chunk, then its exclusive prefix
//   sidx  [n]       particle indices scattered by cell (unordered inside a cell)
//   err   [1]       kNaErr* bits
constexpr size_t kNaWords = (size_t)(kNaMaxCells + 1) + (kNaMaxCells + 2) + (kNaMaxCells + 1) + kNaChunks +
                            kNaMaxParticles + 1;

static __device__ __align__(256) uint32_t g_na_scratch[kNaWords];

struct NaScratch {
    uint32_t *count, *start, *cursor, *chunk, *sidx, *err;
};

NaScratch carve(uint32_t* base, int G) {
    NaScratch S;
    S.count = base;
    S.start = S.count + (G + 1);
    S.cursor = S.start + (G + 2);
    S.chunk = S.cursor + (G + 1);
    S.sidx = S.chunk + kNaChunks;
    S.err = S.sidx + kNaMaxParticles;
    return S;
}

__global__ void k_na_clear(NaScratch S, int G) {
    const int i = blockIdx.x * kNaThreads + threadIdx.x;
    if (i <= G) S.count[i] = 0;
    if (i < kNaChunks) S.chunk[i] = 0;
    if (i == 0) *S.err = 0;
}

// Cell counts; out-of-grid keys are counted per 256-key chunk as well.
__global__ void k_na_count(const uint32_t* __restrict__ key, int n, int G, NaScratch S) {
    const int i = blockIdx.x * kNaThreads + threadIdx.x;
    bool undef = false;
    if (i < n) {
        const uint32_t k = key[i];
        if (k == kNaUndef) {
            undef = true;
        } else if (k < (uint32_t)G) {
            atomicAdd(&S.count[k], 1u);
        } else {
            atomicOr(S.err, kNaErrKey);
        }
    }
    const unsigned b = __ballot_sync(0xffffffffu, undef);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(&S.chunk[blockIdx.x], (uint32_t)__popc(b));
}

// One block: exclusive prefix of the cell counts (start, cursor, the reference's
// mgridoff / mgridcnt) and of the out-of-grid chunk counts.
__global__ void __launch_bounds__(1024) k_na_scan(int n, int G, NaScratch S, int32_t* __restrict__ gridoff,
                                                  int32_t* __restrict__ gridcnt) {
    __shared__ uint32_t part[32];
    __shared__ uint32_t carry;
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base <= G; base += 1024) {
        const int c = base + (int)threadIdx.x;
        const uint32_t v = c <= G ? S.count[c] : 0u;
        uint32_t inc = v;
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t o = __shfl_up_sync(0xffffffffu, inc, d);
            if ((int)lane >= d) inc += o;
        }
        if (lane == 31) part[warp] = inc;
        __syncthreads();
        if (warp == 0) {
            uint32_t p = part[lane];
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t o = __shfl_up_sync(0xffffffffu, p, d);
                if ((int)lane >= d) p += o;
            }
            part[lane] = p;
        }
        __syncthreads();
        const uint32_t excl = carry + (warp > 0 ? part[warp - 1] : 0u) + inc - v;
        if (c <= G) {
            S.start[c] = excl;
            S.cursor[c] = excl;
            if (c < G) {
                gridcnt[c] = (int32_t)v;
                gridoff[c] = v ? (int32_t)excl : 0;  // empty cells keep 0, as after the reference's memset
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) carry += part[31];
        __syncthreads();
    }
    if (threadIdx.x == 0) S.start[G + 1] = (uint32_t)n;
    // out-of-grid chunk counts -> exclusive prefix (serial over at most kNaChunks)
    if (threadIdx.x == 0) {
        uint32_t run = 0;
        const int nch = (n + kNaThreads - 1) / kNaThreads;
        for (int k = 0; k < nch; k++) {
            const uint32_t v = S.chunk[k];
            S.chunk[k] = run;
            run += v;
        }
    }
}

// In-grid keys go to their cell's range in any order (fixed by k_na_order);
// out-of-grid keys go straight to their final place after all cells, in index
// order.
__global__ void k_na_scatter(const uint32_t* __restrict__ key, int n, int G, NaScratch S,
                             uint32_t* __restrict__ midsort, uint32_t* __restrict__ mgndx) {
    const int i = blockIdx.x * kNaThreads + threadIdx.x;
    const uint32_t k = i < n ? key[i] : 0u;
    const bool undef = i < n && k == kNaUndef;
    const unsigned b = __ballot_sync(0xffffffffu, undef);
    __shared__ uint32_t wsum[kNaThreads / 32];
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) wsum[warp] = (uint32_t)__popc(b);
    __syncthreads();
    if (i >= n) return;
    if (undef) {
        uint32_t r = (uint32_t)__popc(b & ((1u << lane) - 1u));
        for (unsigned w = 0; w < warp; w++) r += wsum[w];
        const uint32_t d = S.start[G] + S.chunk[blockIdx.x] + r;
        midsort[d] = (uint32_t)i;
        mgndx[d] = kNaUndef;
    } else if (k < (uint32_t)G) {
        S.sidx[atomicAdd(&S.cursor[k], 1u)] = (uint32_t)i;
    }
}

// Stable order inside each cell: a member's place is the number of members of
// its cell with a smaller particle index (the stable sort keeps index order).
__global__ void k_na_order(const uint32_t* __restrict__ key, int G, NaScratch S, uint32_t* __restrict__ midsort,
                           uint32_t* __restrict__ mgndx) {
    const uint32_t d = blockIdx.x * kNaThreads + threadIdx.x;
    if (d >= S.start[G]) return;
    const uint32_t i = S.sidx[d];
    const uint32_t k = key[i];
    const uint32_t s0 = S.start[k], s1 = S.start[k + 1];
    if (s1 - s0 > (uint32_t)kNaMaxCellMembers) {
        atomicOr(S.err, kNaErrCellSize);
        return;
    }
    uint32_t r = 0;
    for (uint32_t e = s0; e < s1; e++) r += S.sidx[e] < i ? 1u : 0u;
    midsort[s0 + r] = i;
    mgndx[s0 + r] = r;
}

// Scratch addresses by CUDA context: the context's unique id (cuCtxGetId, never
// reused inside a process) and the address of g_na_scratch in it.
struct NaEntry {
    unsigned long long ctx_id;
    uint32_t* ptr;
};
constexpr int kNaCacheSize = 64;
std::mutex g_na_mutex;
NaEntry g_na_cache[kNaCacheSize] = {};
int g_na_next = 0;

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

// Id of the context current on this thread; false if none is current. Called
// with g_na_mutex held.
bool current_ctx_id(unsigned long long* id) {
    if (!g_ctx_get_current || !g_ctx_get_id) {
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaDriverEntryPointQueryResult q1, q2;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
            q1 != cudaDriverEntryPointSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
            q2 != cudaDriverEntryPointSuccess)
            return false;
        g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
        g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f2);
    }
    CUcontext ctx = nullptr;
    if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx) return false;
    return g_ctx_get_id(ctx, id) == CUDA_SUCCESS;
}

// The scratch address in the current context, looked up (cudaGetSymbolAddress,
// which also makes the device's primary context current when none is) the first
// time a context calls. Called with g_na_mutex held.
cudaError_t scratch_address(uint32_t** out) {
    unsigned long long id = 0;
    if (current_ctx_id(&id)) {
        for (const NaEntry& e : g_na_cache)
            if (e.ptr && e.ctx_id == id) {
                *out = e.ptr;
                return cudaSuccess;
            }
    }
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_na_scratch);
    if (e != cudaSuccess) return e;
    if (!current_ctx_id(&id)) return cudaErrorContextIsDestroyed;  // no context current after the lookup
    g_na_cache[g_na_next] = NaEntry{id, static_cast<uint32_t*>(p)};
    g_na_next = (g_na_next + 1) % kNaCacheSize;
    *out = static_cast<uint32_t*>(p);
    return cudaSuccess;
}

}  // namespace
}  // namespace sphmp

using namespace sphmp;

extern "C" sphmp_status sphmp_sort_cells_noalloc(const uint32_t* cell, int32_t n, int32_t gridtotal,
                                                 uint32_t* midsort, uint32_t* mgndx, int32_t* gridoff,
                                                 int32_t* gridcnt, void* stream) {
    if (n < 0 || n > kNaMaxParticles)
        return record_error(SPHMP_ERR_CAPACITY, "sphmp_sort_cells_noalloc: n must be in [0, 262144]");
    if (gridtotal < 1 || gridtotal > kNaMaxCells)
        return record_error(SPHMP_ERR_CAPACITY, "sphmp_sort_cells_noalloc: gridtotal must be in [1, 262144]");
    if ((n > 0 && (!cell || !midsort || !mgndx)) || !gridoff || !gridcnt)
        return record_error(SPHMP_ERR_INVALID_ARG, "sphmp_sort_cells_noalloc: NULL buffer");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return record_error(SPHMP_ERR_NO_DEVICE, cudaGetErrorString(e));
    uint32_t* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_na_mutex);
        e = scratch_address(&base);
    }
    if (e != cudaSuccess) return record_error(SPHMP_ERR_CUDA, cudaGetErrorString(e));
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int G = gridtotal;
    const NaScratch S = carve(base, G);
    const int gclear = (G + 1 > kNaChunks ? G + 1 : kNaChunks) / kNaThreads + 1;
    const int gn = n > 0 ? (n + kNaThreads - 1) / kNaThreads : 1;
    k_na_clear<<<gclear, kNaThreads, 0, s>>>(S, G);
    k_na_count<<<gn, kNaThreads, 0, s>>>(cell, n, G, S);
    k_na_scan<<<1, 1024, 0, s>>>(n, G, S, gridoff, gridcnt);
    k_na_scatter<<<gn, kNaThreads, 0, s>>>(cell, n, G, S, midsort, mgndx);
    k_na_order<<<gn, kNaThreads, 0, s>>>(cell, G, S, midsort, mgndx);
    e = cudaGetLastError();
    if (e != cudaSuccess) return record_error(SPHMP_ERR_CUDA, cudaGetErrorString(e));
    uint32_t err = 0;
    e = cudaMemcpyAsync(&err, S.err, sizeof(err), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return record_error(SPHMP_ERR_CUDA, cudaGetErrorString(e));
    if (err & kNaErrKey)
        return record_error(SPHMP_ERR_INVALID_ARG, "sphmp_sort_cells_noalloc: a key is neither a cell id nor GRID_UNDEF");
    if (err & kNaErrCellSize)
        return record_error(SPHMP_ERR_CELL_OVERFLOW, "sphmp_sort_cells_noalloc: a cell holds more than 4096 particles");
    return SPHMP_OK;
}
