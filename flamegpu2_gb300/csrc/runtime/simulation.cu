// CUDASimulation on GB300.
//
// Per step, in layer order and for each agent function (the reference's
// CUDASimulation::stepLayer, src/flamegpu/simulation/CUDASimulation.cu:644-1109):
//   1. automatic spatial sort of the agent list if the function reads a
//      spatial message (fg_spatial_sort_agents; :670-681)
//   2. spatial index build of the input message list if it changed
//      (fg_spatial_build; CUDAMessage::buildIndex :864)
//   3. the agent function kernel (templated in the model's translation unit)
//   4. birth/death compaction (fg_compact_agents; processDeath/scatterNew :1064-1081)
// Everything is issued on one stream without host synchronisation: counts
// stay on the device, grids are sized by capacity. The whole step is captured
// once into a CUDA graph per "buffer parity" state (sorts and compactions
// ping-pong each agent list between two buffers) and replayed. The host
// synchronises only when a population might outgrow its buffers (births) or
// when data is read back.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <limits>
#include <mutex>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <random>
#include <set>
#include <string>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "flamegpu/detail/launch.cuh"
#include "flamegpu/simulation/CUDASimulation.h"
#include "flamegpu_gb300/fg_capi.h"
#include "runtime/internal.h"
#include "runtime/json.h"

namespace flamegpu {
namespace detail {

using exception::format;

#define FG_CUDA(call)                                                                                      \
    do {                                                                                                   \
        const cudaError_t _e = (call);                                                                     \
        if (_e != cudaSuccess)                                                                             \
            THROW exception::CUDAError(format("%s failed: %s (%s:%d)", #call, cudaGetErrorString(_e), __FILE__, __LINE__)); \
    } while (0)

#define FG_CAPI(call)                                                                                      \
    do {                                                                                                   \
        const int _r = (call);                                                                             \
        if (_r != FG_OK) THROW exception::CUDAError(format("%s returned %d (%s:%d)", #call, _r, __FILE__, __LINE__)); \
    } while (0)

namespace {

// End of a step in one launch: the message counts of the non-persistent
// lists are cleared (CUDASimulation.cu:619-625) and the step counter advances.
constexpr uint32_t kStepEndClears = 16;
constexpr uint32_t kStepEndCounts = 32;
struct StepEnd {
    uint32_t* clear[kStepEndClears];
    uint32_t nclear;
    uint32_t* d_step;
    // agent-steps: acc[0] += acc[1] (the agents that entered this step), then
    // acc[1] = the agents of every list now (those entering the next one)
    const uint32_t* counts[kStepEndCounts];
    uint32_t ncounts;
    unsigned long long* acc;
};
__global__ void k_step_end(const __grid_constant__ StepEnd e) {
    grid_dependency_enter();
    if (threadIdx.x < e.nclear) *e.clear[threadIdx.x] = 0u;
    if (threadIdx.x == 0) *e.d_step += 1u;
    if (e.acc && threadIdx.x < 32) {
        unsigned long long c = threadIdx.x < e.ncounts ? *e.counts[threadIdx.x] : 0ull;
        for (int d = 16; d > 0; d >>= 1) c += __shfl_xor_sync(0xFFFFFFFFu, c, d);
        if (threadIdx.x == 0) {
            e.acc[0] += e.acc[1];
            e.acc[1] = c;
        }
    }
}
// acc[1] = the agents of every list (after a population was set from the host)
__global__ void k_recount(const __grid_constant__ StepEnd e) {
    grid_dependency_enter();
    if (threadIdx.x < 32) {
        unsigned long long c = threadIdx.x < e.ncounts ? *e.counts[threadIdx.x] : 0ull;
        for (int d = 16; d > 0; d >>= 1) c += __shfl_xor_sync(0xFFFFFFFFu, c, d);
        if (threadIdx.x == 0) e.acc[1] = c;
    }
}
// *base = the list's messages so far this step, or 0 if none has been output
// by a launch with agents yet (the appending output then truncates it)
__global__ void k_append_base(uint32_t* base, const uint32_t* count, const uint32_t* filled) {
    grid_dependency_enter();
    *base = *filled ? *count : 0u;
}
__global__ void k_max_u32(uint32_t* p, uint32_t v) {
    grid_dependency_enter();
    *p = *p > v ? *p : v;
}

// Array message build (MessageArray2D.cu:69-101 and CUDAScatter's
// arrayMessageReorder): the array's columns and claim words were cleared
// before this launch; every message output this step (valid, its index set)
// is copied to its index. An index outside the array, or a second message at
// one index, is a device error (the message is dropped).
constexpr uint32_t kArrayCols = 32;
constexpr uint32_t kArrayWriteConflict = 0xA77A0001u;  // the error's name-hash word: raised by the build
struct ArrayScatter {
    const char* src[kArrayCols];
    char* dst[kArrayCols];
    uint32_t bytes[kArrayCols];  // per column, a multiple of 4
    uint32_t ncols;
    const uint32_t* index;       // the ___INDEX column (output rows)
    const uint32_t* valid;       // 1 where the row set its index
    const uint32_t* d_count;     // rows output this step
    uint32_t max_n;
    uint32_t length;             // elements of the array
    uint32_t* claim;             // per array element
    uint32_t* error;             // [code, hash, index, count]
};
__global__ void k_array_scatter(const __grid_constant__ ArrayScatter a) {
    grid_dependency_enter();
    const uint32_t n = min(*a.d_count, a.max_n);
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        if (!a.valid[r]) continue;
        const uint32_t at = a.index[r];
        if (at >= a.length || atomicAdd(a.claim + at, 1u) != 0u) {
            if (atomicCAS(&a.error[0], 0u, static_cast<uint32_t>(kDevArrayMessage)) == 0u) {
                a.error[1] = kArrayWriteConflict;
                a.error[2] = r;
            }
            atomicAdd(&a.error[3], 1u);
            continue;
        }
        for (uint32_t c = 0; c < a.ncols; ++c) {
            const uint32_t* s = reinterpret_cast<const uint32_t*>(a.src[c] + static_cast<size_t>(r) * a.bytes[c]);
            uint32_t* d = reinterpret_cast<uint32_t*>(a.dst[c] + static_cast<size_t>(at) * a.bytes[c]);
            for (uint32_t w = 0; w < a.bytes[c] / 4u; ++w) d[w] = s[w];
        }
    }
}

// HostAgentAPI::sort (HostAgentAPI.cuh:856-1017, a radix sort of (key, row)
// pairs, then every column gathered): a least-significant-digit radix sort
// of 8-bit digits. Keys are the variable's bits made order-preserving as
// unsigned integers (sign bit flipped for signed integers; for floating
// point, all bits of negatives and the sign bit of the rest), inverted for a
// descending sort, cut to bits [begin, end). Each pass: per 2,048-row tile
// the digit counts (digit-major, so that one scan gives every tile's start
// for every digit), then each tile writes its rows in row order: within a
// round of 256 rows a row's place is the rows of its digit in earlier rounds,
// in lower warps of this round and in lower lanes of its warp. Stable, so a
// second key sorts ties of the first.
constexpr uint32_t kSortTile = 2048;
__global__ void k_hsort_keys(const char* col, uint32_t kind, uint32_t bytes, uint32_t invert, uint32_t begin,
                             uint32_t bits, uint32_t n, uint64_t* keys, uint32_t* rows) {
    grid_dependency_enter();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint64_t u = 0;
        const char* p = col + static_cast<size_t>(i) * bytes;
        switch (bytes) {
            case 1: u = *reinterpret_cast<const uint8_t*>(p); break;
            case 2: u = *reinterpret_cast<const uint16_t*>(p); break;
            case 4: u = *reinterpret_cast<const uint32_t*>(p); break;
            default: u = *reinterpret_cast<const uint64_t*>(p); break;
        }
        const uint32_t w = 8u * bytes;
        const uint64_t sign = 1ull << (w - 1u);
        const uint64_t all = w == 64u ? ~0ull : ((1ull << w) - 1ull);
        if (kind == 1u) u ^= sign;                                // signed integer
        else if (kind == 2u) u ^= (u & sign) ? all : sign;        // floating point
        if (invert) u = ~u & all;
        u >>= begin;
        if (bits < 64u) u &= (1ull << bits) - 1ull;
        keys[i] = u;
        rows[i] = i;
    }
}
__global__ void __launch_bounds__(256) k_hsort_counts(const uint64_t* keys, uint32_t n, uint32_t shift, uint32_t ntiles,
                                                     uint32_t* counts) {
    grid_dependency_enter();
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0u;
    __syncthreads();
    const uint32_t base = blockIdx.x * kSortTile;
    for (uint32_t r = 0; r < kSortTile / 256u; ++r) {
        const uint32_t row = base + r * 256u + threadIdx.x;
        if (row < n) atomicAdd(&h[(keys[row] >> shift) & 255u], 1u);
    }
    __syncthreads();
    counts[threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}
__global__ void __launch_bounds__(256) k_hsort_scatter(const uint64_t* keys_in, const uint32_t* rows_in, uint64_t* keys_out,
                                                      uint32_t* rows_out, uint32_t n, uint32_t shift, uint32_t ntiles,
                                                      const uint32_t* starts) {
    grid_dependency_enter();
    __shared__ uint32_t run[256];      // the tile's next place per digit
    __shared__ uint32_t wc[8][256];    // this round's rows per warp and digit
    const uint32_t t = threadIdx.x, lane = t & 31u, warp = t >> 5;
    run[t] = starts[t * ntiles + blockIdx.x];
    const uint32_t base = blockIdx.x * kSortTile;
    for (uint32_t r = 0; r < kSortTile / 256u; ++r) {
        for (uint32_t w = 0; w < 8u; ++w) wc[w][t] = 0u;
        __syncthreads();
        const uint32_t row = base + r * 256u + t;
        const bool act = row < n;
        const uint64_t key = act ? keys_in[row] : 0ull;
        const uint32_t d = act ? static_cast<uint32_t>((key >> shift) & 255u) : 256u + lane;
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
        const uint32_t rank = __popc(peers & ((1u << lane) - 1u));
        if (act && lane == static_cast<uint32_t>(__ffs(peers) - 1)) wc[warp][d] = __popc(peers);
        __syncthreads();
        if (act) {
            uint32_t at = run[d] + rank;
            for (uint32_t w = 0; w < warp; ++w) at += wc[w][d];
            keys_out[at] = key;
            rows_out[at] = rows_in[row];
        }
        __syncthreads();
        uint32_t tot = 0;
        for (uint32_t w = 0; w < 8u; ++w) tot += wc[w][t];
        run[t] += tot;
        __syncthreads();
    }
}
// every column's rows gathered in sorted order: out[p] = in[rows[p]]
__global__ void k_hsort_gather(const char* in, char* out, uint32_t bytes, const uint32_t* rows, uint32_t n) {
    grid_dependency_enter();
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const char* s = in + static_cast<size_t>(rows[p]) * bytes;
        char* o = out + static_cast<size_t>(p) * bytes;
        if ((bytes & 3u) == 0u) {
            for (uint32_t b = 0; b < bytes; b += 4) *reinterpret_cast<uint32_t*>(o + b) = *reinterpret_cast<const uint32_t*>(s + b);
        } else {
            for (uint32_t b = 0; b < bytes; ++b) o[b] = s[b];
        }
    }
}

// Bucket message build (MessageBucket.cu:98-137): each message output this
// step (valid, its key set) gets the sort key key - lower and is counted in
// its bucket; every other row of the list's capacity gets the key `buckets`
// (past the last bucket, so it sorts after every message). The stable sort
// of the rows by key then orders the messages by bucket, in output order.
__global__ void k_bucket_keys(const int32_t* key_col, const uint32_t* valid, const uint32_t* d_count, uint32_t cap,
                              int32_t lower, uint32_t buckets, uint64_t* keys, uint32_t* rows, uint32_t* hist) {
    grid_dependency_enter();
    const uint32_t n = min(*d_count, cap);
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < cap; r += gridDim.x * blockDim.x) {
        uint32_t k = buckets;
        if (r < n && valid[r]) {
            const int64_t d = static_cast<int64_t>(key_col[r]) - lower;
            if (d >= 0 && d < static_cast<int64_t>(buckets)) {
                k = static_cast<uint32_t>(d);
                atomicAdd(hist + k, 1u);
            }
        }
        keys[r] = k;
        rows[r] = r;
    }
}

// Population columns between the device and page-locked host memory in one
// launch (the host buffers read or written by the kernel through their
// mapped device addresses) instead of one copy per column: the set and get
// of a small population cost a launch and a wait, not a dozen copies.
constexpr int kHostXferCols = 32;
constexpr int kHostXferWords = 24;
struct HostXfer {
    const char* src[kHostXferCols];
    char* dst[kHostXferCols];
    uint32_t elem_bytes[kHostXferCols];
    uint32_t ncols;
    uint32_t rows;             // rows to copy (at most, with d_rows)
    const uint32_t* d_rows;    // device row count (get), or null (set: rows)
    uint32_t* rows_out;        // set: the list's device count (= rows); get: a host word for the count
    uint32_t* max_target;      // set: next id, raised to max_value and past every id of column id_col
    uint32_t max_value;
    int32_t id_col;            // set: the id column, checked here (16-byte path only); -1: none
    uint32_t* id_unset;        // set: a host word raised when an id of id_col is unset (0)
    const uint32_t* word_src[kHostXferWords];  // get: status words copied to word_dst
    uint32_t* word_dst[kHostXferWords];
    uint32_t nwords;
    // set: acc[1] = the sum of every list's count (rows_out's new value among
    // them), as k_recount does after a population is set; acc null: none
    const uint32_t* counts[kStepEndCounts];
    uint32_t ncounts;
    unsigned long long* acc;
};

__global__ void k_host_xfer(const __grid_constant__ HostXfer x) {
    grid_dependency_enter();
    const uint32_t rows = x.d_rows ? min(*x.d_rows, x.rows) : x.rows;
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x, nthreads = gridDim.x * blockDim.x;
    if (tid == 0) {
        if (x.rows_out) *x.rows_out = x.d_rows ? *x.d_rows : rows;
        if (x.max_target && x.max_value) atomicMax(x.max_target, x.max_value);
        if (x.acc) {  // after rows_out: the same thread's store is visible to its loads
            unsigned long long c = 0;
            for (uint32_t k = 0; k < x.ncounts; ++k) c += *x.counts[k];
            x.acc[1] = c;
        }
    }
    if (tid < x.nwords) *x.word_dst[tid] = *x.word_src[tid];
    // columns eight at a time: the 16-byte pieces of all eight are loaded
    // before any is stored, so one round trip to host memory (set) covers
    // every column instead of one per column. The ids of column id_col are
    // checked on the way (the host does not read them again).
    uint32_t id_max = 0, id_unset = 0;
    for (uint32_t c0 = 0; c0 < x.ncols; c0 += 8) {
        const uint32_t nc = min(8u, x.ncols - c0);
        size_t n16[8];
        size_t most = 0;
#pragma unroll
        for (uint32_t j = 0; j < 8; ++j) {
            n16[j] = 0;
            if (j < nc) {
                const size_t bytes = static_cast<size_t>(rows) * x.elem_bytes[c0 + j];
                const uintptr_t a = reinterpret_cast<uintptr_t>(x.src[c0 + j]) | reinterpret_cast<uintptr_t>(x.dst[c0 + j]);
                if (((a | bytes) & 15) == 0) n16[j] = bytes / 16;
                most = n16[j] > most ? n16[j] : most;
            }
        }
        for (size_t k = tid; k < most; k += nthreads) {
            uint4 v[8];
#pragma unroll
            for (uint32_t j = 0; j < 8; ++j)
                if (k < n16[j]) v[j] = reinterpret_cast<const uint4*>(x.src[c0 + j])[k];
#pragma unroll
            for (uint32_t j = 0; j < 8; ++j)
                if (k < n16[j]) reinterpret_cast<uint4*>(x.dst[c0 + j])[k] = v[j];
#pragma unroll
            for (uint32_t j = 0; j < 8; ++j)
                if (static_cast<int32_t>(c0 + j) == x.id_col && k < n16[j]) {
                    id_max = max(max(max(id_max, v[j].x), max(v[j].y, v[j].z)), v[j].w);
                    id_unset |= (v[j].x == 0u) | (v[j].y == 0u) | (v[j].z == 0u) | (v[j].w == 0u);
                }
        }
    }
    if (x.id_col >= 0) {
        id_max = __reduce_max_sync(0xFFFFFFFFu, id_max);
        id_unset = __reduce_or_sync(0xFFFFFFFFu, id_unset);
        if ((threadIdx.x & 31u) == 0) {
            if (id_max && x.max_target) atomicMax(x.max_target, id_max + 1u);
            if (id_unset) *x.id_unset = 1u;
        }
    }
    // the columns not 16-byte aligned: word or byte copies
    for (uint32_t c = 0; c < x.ncols; ++c) {
        const size_t bytes = static_cast<size_t>(rows) * x.elem_bytes[c];
        const char* s = x.src[c];
        char* d = x.dst[c];
        if (((reinterpret_cast<uintptr_t>(s) | reinterpret_cast<uintptr_t>(d) | bytes) & 15) == 0) {
            continue;  // copied above
        } else if (((reinterpret_cast<uintptr_t>(s) | reinterpret_cast<uintptr_t>(d) | bytes) & 3) == 0) {
            const uint32_t* s1 = reinterpret_cast<const uint32_t*>(s);
            uint32_t* d1 = reinterpret_cast<uint32_t*>(d);
            for (size_t k = tid; k < bytes / 4; k += nthreads) d1[k] = s1[k];
        } else {
            for (size_t k = tid; k < bytes; k += nthreads) d[k] = s[k];
        }
    }
}

// One 16-byte unit of each column per thread (host memory is far: keep
// every copy in flight at once), at most four blocks of 256 per SM.
inline unsigned int host_xfer_grid(const HostXfer& x, int sms) {
    size_t bytes = 0;
    for (uint32_t c = 0; c < x.ncols; ++c) bytes = std::max(bytes, static_cast<size_t>(x.rows) * x.elem_bytes[c]);
    const size_t blocks = (bytes + 256 * 16 - 1) / (256 * 16);
    return static_cast<unsigned int>(std::max<size_t>(1, std::min<size_t>(blocks, 4u * static_cast<unsigned int>(sms))));
}

// The device address of page-locked host memory, or null (pageable memory,
// or not addressable from the device): such buffers take the copy path.
inline void* host_mapped(const void* p) {
    if (!p) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// Device buffers of one simulation, taken stream-ordered from the device's
// default memory pool: a finished simulation returns its memory without
// stalling the other simulations of the process (cudaFree would wait for the
// whole device), and a later one reuses it without a new mapping.
struct DevMem {
    std::vector<void*> ptrs;
    cudaStream_t stream = nullptr;  // the owning simulation's stream
    static void keep_pool(int device) {
        static std::once_flag once[64];
        if (device < 0 || device >= 64) return;
        std::call_once(once[device], [device] {
            cudaMemPool_t pool;
            if (cudaDeviceGetDefaultMemPool(&pool, device) != cudaSuccess) return;
            uint64_t keep = ~0ull;  // freed blocks stay in the pool for the next simulation
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        });
    }
    void* alloc(size_t bytes, bool zero = true) {
        void* p = nullptr;
        const size_t n = std::max<size_t>(bytes, 256);
        FG_CUDA(cudaMallocAsync(&p, n, stream));
        ptrs.push_back(p);
        if (zero) FG_CUDA(cudaMemsetAsync(p, 0, n, stream));
        // host copies into the buffer may follow on other streams
        FG_CUDA(cudaStreamSynchronize(stream));
        return p;
    }
    void release(void* p) {
        if (!p) return;
        auto it = std::find(ptrs.begin(), ptrs.end(), p);
        if (it != ptrs.end()) {
            cudaFreeAsync(p, stream);  // after the stream's pending work on it
            ptrs.erase(it);
        }
    }
    void release_all() {
        for (void* p : ptrs) cudaFreeAsync(p, stream);
        ptrs.clear();
    }
    ~DevMem() { release_all(); }
};

uint32_t round4(uint32_t b) { return (b + 3u) & ~3u; }

int sm_count(int dev) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    return v > 0 ? v : 132;
}

}  // namespace

VarTable make_table(const std::vector<TableEntry>& e, const char* what) {
    VarTable t;
    std::memset(&t, 0, sizeof(t));
    const uint32_t n = static_cast<uint32_t>(e.size());
    uint32_t size = 2;
    while (size < n) size <<= 1;
    std::mt19937 rng(12345u);
    for (; size <= static_cast<uint32_t>(kMaxVarSlots); size <<= 1) {
        uint32_t bits = 0;
        while ((1u << bits) < size) ++bits;
        const uint32_t shift = 32u - bits;
        for (int attempt = 0; attempt < 200000; ++attempt) {
            const uint32_t mult = attempt == 0 ? 1u : (rng() | 1u);
            uint64_t used = 0;
            bool ok = true;
            for (const auto& x : e) {
                const uint32_t s = table_slot(mult, shift, x.hash);
                if (used & (1ull << s)) {
                    ok = false;
                    break;
                }
                used |= 1ull << s;
            }
            if (!ok) continue;
            t.mult = mult;
            t.shift = shift;
            t.count = n;
            for (const auto& x : e) {
                VarSlot& s = t.slot[table_slot(mult, shift, x.hash)];
                s.ptr = x.ptr;
                s.stride = x.stride;
                s.hash = x.hash;
                s.elem_bytes = x.elem_bytes;
                s.elements = x.elements;
            }
            return t;
        }
    }
    THROW exception::InvalidArgument(format("Too many variables (%u) in one %s for the lookup table", n, what));
}

SpatialRecordLayout spatial_record_layout(const std::vector<std::pair<uint32_t, uint32_t>>& vars, int dims,
                                          const char* what) {
    static const uint32_t loc[3] = {fnv1a32("x", 1), fnv1a32("y", 1), fnv1a32("z", 1)};
    if (vars.size() < static_cast<size_t>(dims))
        THROW exception::InvalidMessage(format("Spatial message '%s' has no location", what));
    for (int d = 0; d < dims; ++d)
        if (vars[d].first != loc[d] || vars[d].second != 4u)
            THROW exception::InvalidMessage(format("Spatial message '%s' does not start with its location", what));
    SpatialRecordLayout L;
    std::vector<TableEntry> pay;
    uint32_t stride = 4;
    for (size_t v = dims; v < vars.size(); ++v) {
        pay.push_back({vars[v].first, nullptr, 0, 4, 1});
        stride = std::max(stride, vars[v].second);
    }
    const VarTable t = make_table(pay, what);
    uint32_t slots = 0;
    for (const auto& x : pay) slots = std::max(slots, table_slot(t.mult, t.shift, x.hash) + 1u);
    L.pay_mult = t.mult;
    L.pay_shift = t.shift;
    L.pay_stride = stride;
    for (size_t v = 0; v < vars.size(); ++v)
        L.field_word.push_back(v < static_cast<size_t>(dims)
                                   ? static_cast<uint32_t>(v)
                                   : static_cast<uint32_t>(dims) + table_slot(t.mult, t.shift, vars[v].first) * (stride / 4u));
    const uint32_t words = static_cast<uint32_t>(dims) + slots * (stride / 4u);
    L.record_words = std::max(4u, (words + 3u) & ~3u);
    if (L.record_words > FG_MAX_RECORD_WORDS)
        THROW exception::InvalidMessage(format("Message '%s' is larger than %d bytes", what, FG_MAX_RECORD_WORDS * 4));
    return L;
}

struct AgentList {
    AgentData* agent = nullptr;
    std::string state;
    uint32_t capacity = 0;
    std::vector<std::array<void*, 2>> cols;  // per agent variable, ping-pong buffers
    int parity = 0;
    uint32_t* d_count = nullptr;
    uint32_t bound = 0;                       // host upper bound of the device count
    std::map<const void*, std::pair<void*, size_t>> sort_ws;  // per sorting message grid
    void* comp_ws = nullptr;
    size_t comp_ws_bytes = 0;
    int var_index(const std::string& n) const {
        for (size_t v = 0; v < agent->variables.size(); ++v)
            if (agent->variables[v].name == n) return static_cast<int>(v);
        return -1;
    }
};

struct MsgList {
    MessageData* msg = nullptr;
    uint32_t capacity = 0;
    std::vector<uint32_t> slot_bytes;  // per variable, rounded up to 4 bytes
    std::vector<void*> cols;           // unsorted struct-of-arrays, written by the output function
    uint32_t* valid = nullptr;         // per-row output flags when any output is optional
    uint32_t* d_count = nullptr;
    bool optional_any = false;
    // spatial
    fg_spatial_grid grid{};
    uint32_t* pbm = nullptr;
    uint32_t pbm_alloc = 0;
    uint32_t* records = nullptr;
    uint32_t record_words = 0;
    uint32_t pay_mult = 0, pay_shift = 0, pay_stride = 0;  // record layout of the non-location fields
    std::vector<uint32_t> field_word;
    void* build_ws = nullptr;
    size_t build_ws_bytes = 0;
    // brute force with optional output: compacted copy
    std::vector<void*> bf_cols;
    uint32_t* bf_count = nullptr;
    void* bf_ws = nullptr;
    size_t bf_ws_bytes = 0;
    bool needs_build = true;
    // truncate / append (CUDASimulation.cu:598-601,874,1058): the first output
    // of a step truncates the list, later ones append after its messages
    bool written = false;            // host, while a step is being issued
    uint32_t* d_base = nullptr;      // count before an appending output (device)
    // 1 once a launch with at least one agent has output to the list this step
    // (device; cleared at every step end): until then an output truncates it,
    // and a launch over no agents leaves it as it was (CUDASimulation.cu:1050-1059)
    uint32_t* d_filled = nullptr;
    // array messages: the array (index order, one column per variable), its
    // dimensions, a claim word per element (the build's duplicate check) and
    // its length on the device (the input's message count)
    uint32_t arr_dims[3] = {1, 1, 1};
    uint32_t arr_len = 0;
    std::vector<void*> arr_cols;
    uint32_t* arr_claim = nullptr;
    uint32_t* arr_count = nullptr;
    // bucket messages: keys lower .. lower + buckets - 1; the messages sorted
    // by bucket (one column per variable), the PBM (buckets + 1 entries), the
    // bucket counts, and the radix sort's scratch (sized by the capacity)
    int32_t bk_lower = 0;
    uint32_t bk_buckets = 0;
    std::vector<void*> bk_cols;
    uint32_t* bk_pbm = nullptr;
    uint32_t* bk_hist = nullptr;
    uint64_t* bk_keys[2] = {nullptr, nullptr};
    uint32_t* bk_rows[2] = {nullptr, nullptr};
    uint32_t* bk_counts = nullptr;
    uint32_t* bk_starts = nullptr;
    void* bk_ws = nullptr;
    size_t bk_ws_bytes = 0;
    bool bucket() const { return msg->kind == MessageKind::Bucket; }
    bool array() const { return array_dims(msg->kind) != 0; }
    bool spatial() const { return msg->kind == MessageKind::Spatial2D || msg->kind == MessageKind::Spatial3D; }
};

struct FnRt {
    AgentFunctionData* fn = nullptr;
    AgentList* list = nullptr;
    MsgList* in = nullptr;
    MsgList* out = nullptr;
    bool births = false;
    // the list births go to (setAgentOutput's agent and state). Fused: it is the
    // list where the function's own agents end up (their list, or the end
    // state's), so one compaction writes survivors then births; otherwise the
    // births are appended to it after the death compaction and the transition
    AgentList* birth_list = nullptr;
    bool births_fused = false;
    uint32_t* d_launch_n = nullptr;  // rows the function ran over (unfused births)
    uint32_t* death_flags = nullptr;
    uint32_t* birth_flags = nullptr;
    std::vector<void*> birth_cols;
    void* birth_defaults = nullptr;
    std::unique_ptr<FunctionTables> tables[2];  // per buffer parity of the agent list
    bool sort_trigger = false;
    int pos_var = -1;   // a packed "xyz" / "xy" position variable the sort reads, or -1 (x, y, z)
    bool stage = false;  // spatial input and the agent has float x, y (, z): stage neighbour windows
    uint32_t* cond_fail = nullptr;  // condition result per row (1 = failed), capacity + 1 entries
    uint32_t* d_first = nullptr;    // rows that failed the condition (device)
    AgentList* end_list = nullptr;  // state transition target, or null
    // keys computed by this function's launch for what follows it (plan_keys)
    MsgList* key_msg = nullptr;  // the build of this output list
    FnRt* key_sort = nullptr;    // the agent sort before this function (same list)
    bool build_keyed = false;    // this function's input build: keys already written
    bool sort_keyed = false;     // this function's agent sort: keys already written
};

struct SimulationImpl {
    std::shared_ptr<ModelData> model;
    CUDASimulation::SimConfig config;
    CUDASimulation::Config cuda_config;
    int device = 0;
    int sms = 132;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;        // second branch of a layer (build next to sort)
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    DevMem mem;
    std::vector<std::unique_ptr<AgentList>> lists;
    std::vector<std::unique_ptr<MsgList>> msgs;
    std::vector<FnRt> fns;
    // environment
    std::vector<char> env_host;
    std::vector<size_t> env_offset;
    char* d_env = nullptr;
    bool env_dirty = true;
    // macro properties: after the plain properties in the environment buffer
    // (offsets from its start, 8-byte aligned), never uploaded from env_host;
    // the host views that are alive, by name
    std::vector<size_t> macro_offset;
    size_t macro_flags_offset = 0, macro_flag_bytes = 0;
    std::unordered_map<std::string, std::weak_ptr<HostMacroData>> macro_views;
    // misc device state
    uint32_t* d_misc = nullptr;  // [0] step, [1..4] error record, [8..] next ids per agent
    unsigned long long* d_agent_steps = nullptr;  // [0] agents summed over the steps run, [1] agents now
    unsigned long long host_agent_steps = 0;      // the same for populations that only the host changes
    CUDASimulation* owner = nullptr;  // the simulation this implements (host functions reach it)
    // HostRandom's engine: seeded with the simulation's random seed when the
    // configuration is applied (RandomManager::reseed)
    std::mt19937_64 host_rng{0};
    uint64_t host_rng_seed = 0;
    bool host_rng_applied = false;
    uint64_t host_rng_applied_seed = 0;
    // agents created by host functions (HostAgentAPI::newAgent), per (agent, state),
    // joining their populations when the host functions return
    std::map<std::pair<std::string, std::string>, std::unique_ptr<AgentVector>> host_births;
    // populations host functions read with getPopulationData, per (agent, state),
    // written back when the host functions return
    std::map<std::pair<std::string, std::string>, std::unique_ptr<AgentVector>> host_views;
    uint32_t* h_pinned = nullptr;
    uint32_t* h_pinned_dev = nullptr;  // its device address (null: not mapped)
    unsigned int step_count = 0;
    bool exit_requested = false;  // an exit condition returned EXIT in the last step
    std::vector<uint32_t> next_id;  // host mirror per agent index (valid when synced)
    bool ids_on_device = true;
    // graphs
    std::map<std::vector<int>, cudaGraphExec_t> graphs;
    unsigned long long graph_launches = 0;
    unsigned int kernels_last_step = 0;
    unsigned int kernel_counter = 0;
    bool allocated = false;
    // per-operation profile (eager mode only): label -> events
    bool profiling = false;
    std::vector<std::tuple<std::string, cudaEvent_t, cudaEvent_t>> op_events;
    std::map<std::string, std::pair<double, uint64_t>> op_totals;  // label -> (ms, count)
    // timing events captured into the step graphs (Config::time_ops_in_graphs):
    // per graph key, the event pairs around each operation, and the keys
    // replayed since the last harvest
    bool capturing = false;
    std::vector<int> capture_key;
    std::map<std::vector<int>, std::vector<std::tuple<std::string, cudaEvent_t, cudaEvent_t>>> graph_op_events;
    std::set<std::vector<int>> replayed;
    // timing
    struct StepTimer {
        cudaEvent_t e0, e1;
        unsigned int steps;  // model steps between the two events
    };
    std::vector<StepTimer> step_events;
    std::vector<double> step_ms;
    double sim_ms = 0.0;

    explicit SimulationImpl(const std::shared_ptr<ModelData>& m) : model(m) {}
    ~SimulationImpl() {
        if (stream) {
            cudaStreamSynchronize(stream);
            mem.release_all();
            cudaStreamSynchronize(stream);
        }
        for (auto& g : graphs) cudaGraphExecDestroy(g.second);
        drop_graph_op_events();
        for (auto& e : step_events) {
            cudaEventDestroy(e.e0);
            cudaEventDestroy(e.e1);
        }
        for (auto& c : count_ring)
            if (c.ev) cudaEventDestroy(c.ev);
        if (count_pinned) cudaFreeHost(count_pinned);
        if (h_pinned) cudaFreeHost(h_pinned);
        if (fork_ev) cudaEventDestroy(fork_ev);
        if (join_ev) cudaEventDestroy(join_ev);
        if (side) cudaStreamDestroy(side);
        if (stream) cudaStreamDestroy(stream);
    }

    uint32_t* d_step() const { return d_misc; }
    uint32_t* d_error() const { return d_misc + 1; }
    uint32_t* d_next_id(size_t agent_idx) const { return d_misc + 8 + agent_idx; }

    size_t agent_index(const AgentData* a) const {
        for (size_t i = 0; i < model->agents.size(); ++i)
            if (model->agents[i].get() == a) return i;
        return 0;
    }

    // The compaction workspace header's survivor word of list l (fg_compact_agents
    // reads it as d_alive_total; its last block resets it to zero).
    static uint32_t* survivors_word(const AgentList& l) { return fgi_compact_survivor_word(l.comp_ws); }
    AgentList* list_of(const std::string& agent, const std::string& state) {
        for (auto& l : lists)
            if (l->agent->name == agent && l->state == state) return l.get();
        THROW exception::InvalidAgentName(format("No agent list '%s' in state '%s'", agent.c_str(), state.c_str()));
    }
    MsgList* msg_of(const std::string& name) {
        for (auto& m : msgs)
            if (m->msg->name == name) return m.get();
        return nullptr;
    }

    // ------------------------------------------------------------- set-up

    void init() {
        FG_CUDA(cudaSetDevice(cuda_config.device_id));
        device = cuda_config.device_id;
        sms = sm_count(device);
        FG_CUDA(cudaStreamCreateWithPriority(&stream, cudaStreamNonBlocking, cuda_config.stream_priority));
        FG_CUDA(cudaStreamCreateWithPriority(&side, cudaStreamNonBlocking, cuda_config.stream_priority));
        DevMem::keep_pool(device);
        mem.stream = stream;
        FG_CUDA(cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming));
        FG_CUDA(cudaEventCreateWithFlags(&join_ev, cudaEventDisableTiming));
        FG_CUDA(cudaMallocHost(&h_pinned, 4096));
        h_pinned_dev = static_cast<uint32_t*>(host_mapped(h_pinned));
        std::memset(h_pinned, 0, 4096);
        d_misc = static_cast<uint32_t*>(mem.alloc(sizeof(uint32_t) * (8 + model->agents.size() + 8)));
        d_agent_steps = static_cast<unsigned long long*>(mem.alloc(2 * sizeof(unsigned long long)));
        next_id.assign(model->agents.size(), 1u);
        std::vector<uint32_t> init_ids(model->agents.size(), 1u);
        FG_CUDA(cudaMemcpy(d_misc + 8, init_ids.data(), sizeof(uint32_t) * init_ids.size(), cudaMemcpyHostToDevice));
        validate_model();
        // environment buffer (8-byte aligned properties)
        size_t off = 0;
        for (const auto& p : model->environment) {
            env_offset.push_back(off);
            off += (p.value.size() + 7) & ~size_t(7);
        }
        env_host.assign(std::max<size_t>(off, 8), 0);
        for (size_t i = 0; i < model->environment.size(); ++i)
            std::memcpy(env_host.data() + env_offset[i], model->environment[i].value.data(), model->environment[i].value.size());
        // one flag word per macro property (read / updated by the running agent
        // function), then the macro properties
        macro_flags_offset = env_host.size();
        macro_flag_bytes = sizeof(uint32_t) * model->macro_environment.size();
        size_t macro_end = macro_flags_offset + ((macro_flag_bytes + 7) & ~size_t(7));
        for (const auto& p : model->macro_environment) {
            macro_offset.push_back(macro_end);
            macro_end += (static_cast<size_t>(p.type_size) * p.elements() + 7) & ~size_t(7);
        }
        d_env = static_cast<char*>(mem.alloc(macro_end));  // zeroed: macro properties start at 0
        FG_CUDA(cudaMemcpy(d_env, env_host.data(), env_host.size(), cudaMemcpyHostToDevice));
        env_dirty = false;
        // agent lists (one per state)
        for (const auto& a : model->agents)
            for (const auto& s : a->states) {
                auto l = std::make_unique<AgentList>();
                l->agent = a.get();
                l->state = s;
                l->cols.resize(a->variables.size(), {nullptr, nullptr});
                l->d_count = static_cast<uint32_t*>(mem.alloc(sizeof(uint32_t)));
                lists.push_back(std::move(l));
            }
        for (const auto& m : model->messages) {
            auto ml = std::make_unique<MsgList>();
            ml->msg = m.get();
            ml->d_count = static_cast<uint32_t*>(mem.alloc(sizeof(uint32_t)));
            ml->d_base = static_cast<uint32_t*>(mem.alloc(sizeof(uint32_t)));
            ml->d_filled = static_cast<uint32_t*>(mem.alloc(sizeof(uint32_t)));  // zeroed
            for (const auto& v : m->variables) ml->slot_bytes.push_back(round4(v.bytes()));
            if (m->kind == MessageKind::Bucket) {
                if (m->bucket_upper == std::numeric_limits<int32_t>::max())
                    THROW exception::InvalidMessage(format("Bucket message '%s' has no upper bound", m->name.c_str()));
                const int64_t buckets = static_cast<int64_t>(m->bucket_upper) - m->bucket_lower + 1;
                if (buckets <= 0 || buckets > (1ll << 30))
                    THROW exception::InvalidMessage(format("Bucket message '%s' has too many keys", m->name.c_str()));
                ml->bk_lower = m->bucket_lower;
                ml->bk_buckets = static_cast<uint32_t>(buckets);
                ml->bk_pbm = static_cast<uint32_t*>(mem.alloc(sizeof(uint32_t) * (static_cast<size_t>(buckets) + 2)));
                ml->bk_hist = static_cast<uint32_t*>(mem.alloc(sizeof(uint32_t) * (static_cast<size_t>(buckets) + 2)));
            } else if (array_dims(m->kind)) {
                for (int a = 0; a < 3; ++a) ml->arr_dims[a] = a < array_dims(m->kind) ? m->dims[a] : 1u;
                const uint64_t len = static_cast<uint64_t>(ml->arr_dims[0]) * ml->arr_dims[1] * ml->arr_dims[2];
                if (len == 0 || len > 0x7FFFFFFFull)
                    THROW exception::InvalidMessage(format("Array message '%s' has unset or too large dimensions", m->name.c_str()));
                if (m->variables.size() > kArrayCols)
                    THROW exception::InvalidMessage(format("Array message '%s' has more than %u variables", m->name.c_str(), kArrayCols));
                ml->arr_len = static_cast<uint32_t>(len);
                for (uint32_t b : ml->slot_bytes) ml->arr_cols.push_back(mem.alloc(static_cast<size_t>(b) * len));
                ml->arr_claim = static_cast<uint32_t*>(mem.alloc(sizeof(uint32_t) * len));
                ml->arr_count = static_cast<uint32_t*>(mem.alloc(sizeof(uint32_t)));
                FG_CUDA(cudaMemcpy(ml->arr_count, &ml->arr_len, sizeof(uint32_t), cudaMemcpyHostToDevice));
            } else if (m->kind != MessageKind::BruteForce) {
                const int dims = m->kind == MessageKind::Spatial3D ? 3 : 2;
                FG_CAPI(fg_spatial_grid_init(&ml->grid, dims, m->min, m->max, m->radius));
                // PBM padded to a multiple of 4 entries (+4): the staging window copies 16-byte aligned slices
                ml->pbm_alloc = (ml->grid.binCount + 1u + 3u) & ~3u;
                ml->pbm = static_cast<uint32_t*>(mem.alloc(sizeof(uint32_t) * (static_cast<size_t>(ml->pbm_alloc) + 4)));
                std::vector<std::pair<uint32_t, uint32_t>> vars;
                for (size_t v = 0; v < m->variables.size(); ++v)
                    vars.emplace_back(fnv1a32(m->variables[v].name), ml->slot_bytes[v]);
                const SpatialRecordLayout L = spatial_record_layout(vars, dims, m->name.c_str());
                ml->field_word = L.field_word;
                ml->record_words = L.record_words;
                ml->pay_mult = L.pay_mult;
                ml->pay_shift = L.pay_shift;
                ml->pay_stride = L.pay_stride;
            }
            msgs.push_back(std::move(ml));
        }
        for (const auto& a : model->agents)
            for (const auto& f : a->functions) {
                FnRt r;
                r.fn = f.get();
                r.list = list_of(a->name, f->initial_state);
                if (f->initial_state != f->end_state) r.end_list = list_of(a->name, f->end_state);
                r.in = f->message_input.empty() ? nullptr : msg_of(f->message_input);
                r.out = f->message_output.empty() ? nullptr : msg_of(f->message_output);
                if (r.out && f->message_output_optional) r.out->optional_any = true;
                if (!f->agent_output.empty()) {
                    // CUDASimulation.cu:1062-1080: death compaction, then the state
                    // transition, then the births appended to the output list
                    r.births = true;
                    r.birth_list = list_of(f->agent_output, f->agent_output_state);
                    r.births_fused = r.birth_list == (r.end_list ? r.end_list : r.list);
                    if (!r.births_fused) r.d_launch_n = static_cast<uint32_t*>(mem.alloc(sizeof(uint32_t)));
                }
                // determineAgentsToSort (CUDASimulation.cu:409-461)
                if (r.in && r.in->spatial()) {
                    const int dims = r.in->msg->kind == MessageKind::Spatial3D ? 3 : 2;
                    bool ok = true;
                    const char* ax[3] = {"x", "y", "z"};
                    for (int d = 0; d < dims; ++d) {
                        const Variable* v = a->find(ax[d]);
                        ok = ok && v && v->type == std::type_index(typeid(float)) && v->elements == 1;
                    }
                    r.sort_trigger = ok;
                    r.stage = ok;
                    if (!ok) {  // or a packed position array of the message's dimensions
                        const char* packed = dims == 3 ? "xyz" : "xy";
                        for (size_t v = 0; v < a->variables.size(); ++v) {
                            const Variable& var = a->variables[v];
                            if (var.name == packed && var.type == std::type_index(typeid(float)) &&
                                var.elements == static_cast<uint32_t>(dims)) {
                                r.sort_trigger = true;
                                r.pos_var = static_cast<int>(v);
                            }
                        }
                    }
                }
                fns.push_back(std::move(r));
            }
    }

    void validate_model() {
        for (const auto& m : model->messages) {
            if (m->kind != MessageKind::Spatial2D && m->kind != MessageKind::Spatial3D) continue;
            const int dims = m->kind == MessageKind::Spatial3D ? 3 : 2;
            if (std::isnan(m->radius))
                THROW exception::InvalidMessage(format("Spatial message '%s' has no radius", m->name.c_str()));
            for (int d = 0; d < dims; ++d)
                if (std::isnan(m->min[d]) || std::isnan(m->max[d]))
                    THROW exception::InvalidMessage(format("Spatial message '%s' has unset bounds", m->name.c_str()));
        }
        for (const auto& l : model->layers)
            if (!l->host_functions.empty() && !l->functions.empty())
                THROW exception::InvalidArgument("A layer may hold agent functions or host functions, not both");
    }

    // Allocate (or grow) an agent list to `cap` rows, keeping `keep` rows.
    void ensure_capacity(AgentList& l, uint32_t cap, uint32_t keep) {
        if (cap <= l.capacity) return;
        const uint32_t old_cap = l.capacity;
        for (size_t v = 0; v < l.cols.size(); ++v) {
            const size_t b = l.agent->variables[v].bytes();
            void* n0 = mem.alloc(b * cap, false);
            void* n1 = mem.alloc(b * cap, false);
            if (l.cols[v][l.parity] && keep)
                FG_CUDA(cudaMemcpyAsync(n0, l.cols[v][l.parity], b * keep, cudaMemcpyDeviceToDevice, stream));
            mem.release(l.cols[v][0]);
            mem.release(l.cols[v][1]);
            l.cols[v] = {n0, n1};
        }
        l.parity = 0;
        l.capacity = cap;
        for (auto& s : l.sort_ws) mem.release(s.second.first);
        l.sort_ws.clear();
        mem.release(l.comp_ws);
        l.comp_ws_bytes = fg_compact_workspace_size(cap);
        l.comp_ws = mem.alloc(l.comp_ws_bytes);
        (void)old_cap;
        // dependants: message lists written by this list's functions, birth staging, flags
        for (auto& f : fns) {
            if (f.list != &l) continue;
            if (f.out) ensure_msg_capacity(*f.out, producers_capacity(*f.out));
            if (f.fn->has_agent_death) {
                mem.release(f.death_flags);
                f.death_flags = static_cast<uint32_t*>(mem.alloc(sizeof(uint32_t) * cap));
            }
            if (f.fn->condition) {
                mem.release(f.cond_fail);
                f.cond_fail = static_cast<uint32_t*>(mem.alloc(sizeof(uint32_t) * (static_cast<size_t>(cap) + 1)));
                if (!f.d_first) f.d_first = static_cast<uint32_t*>(mem.alloc(sizeof(uint32_t)));
            }
            if (f.births) {
                // staging: one row of the output agent's variables per parent row
                mem.release(f.birth_flags);
                f.birth_flags = static_cast<uint32_t*>(mem.alloc(sizeof(uint32_t) * cap));
                for (void* p : f.birth_cols) mem.release(p);
                f.birth_cols.clear();
                for (const auto& v : f.birth_list->agent->variables)
                    f.birth_cols.push_back(mem.alloc(static_cast<size_t>(v.bytes()) * cap));
            }
        }
        invalidate();
    }

    // Messages one step can put in a list: every function that outputs to it
    // may append a message per agent of its list.
    uint32_t producers_capacity(const MsgList& m) const {
        uint64_t c = 0;
        for (const auto& g : fns)
            if (g.out == &m) c += g.list->capacity;
        return static_cast<uint32_t>(std::min<uint64_t>(std::max<uint64_t>(c, 1), (1ull << 31) - 1));
    }

    void ensure_msg_capacity(MsgList& m, uint32_t cap) {
        if (cap <= m.capacity) return;
        for (void* p : m.cols) mem.release(p);
        m.cols.clear();
        for (uint32_t b : m.slot_bytes) m.cols.push_back(mem.alloc(static_cast<size_t>(b) * cap));
        if (m.optional_any || m.array() || m.bucket()) {
            mem.release(m.valid);
            m.valid = static_cast<uint32_t*>(mem.alloc(sizeof(uint32_t) * cap));
        }
        if (m.bucket()) {
            for (void* p : m.bk_cols) mem.release(p);
            m.bk_cols.clear();
            for (uint32_t b : m.slot_bytes) m.bk_cols.push_back(mem.alloc(static_cast<size_t>(b) * cap));
            for (int k = 0; k < 2; ++k) {
                mem.release(m.bk_keys[k]);
                mem.release(m.bk_rows[k]);
                m.bk_keys[k] = static_cast<uint64_t*>(mem.alloc(sizeof(uint64_t) * cap));
                m.bk_rows[k] = static_cast<uint32_t*>(mem.alloc(sizeof(uint32_t) * cap));
            }
            const uint32_t ncount = 256u * ((cap + kSortTile - 1) / kSortTile);
            mem.release(m.bk_counts);
            mem.release(m.bk_starts);
            m.bk_counts = static_cast<uint32_t*>(mem.alloc(sizeof(uint32_t) * (ncount + 4)));
            m.bk_starts = static_cast<uint32_t*>(mem.alloc(sizeof(uint32_t) * (ncount + 4)));
            mem.release(m.bk_ws);
            m.bk_ws_bytes = fg_scan_workspace_size(std::max(ncount, m.bk_buckets + 1u));
            m.bk_ws = mem.alloc(m.bk_ws_bytes);
        }
        if (m.spatial()) {
            mem.release(m.records);
            m.records = static_cast<uint32_t*>(mem.alloc(sizeof(uint32_t) * m.record_words * static_cast<size_t>(cap)));
            mem.release(m.build_ws);
            m.build_ws_bytes = fg_spatial_build_workspace_size(cap, m.grid.binCount);
            m.build_ws = mem.alloc(m.build_ws_bytes);
        } else if (m.optional_any && !m.array() && !m.bucket()) {
            for (void* p : m.bf_cols) mem.release(p);
            m.bf_cols.clear();
            for (uint32_t b : m.slot_bytes) m.bf_cols.push_back(mem.alloc(static_cast<size_t>(b) * cap));
            if (!m.bf_count) m.bf_count = static_cast<uint32_t*>(mem.alloc(sizeof(uint32_t)));
            mem.release(m.bf_ws);
            m.bf_ws_bytes = fg_compact_workspace_size(cap);
            m.bf_ws = mem.alloc(m.bf_ws_bytes);
        }
        m.capacity = cap;
        invalidate();
    }

    // Step graphs are keyed by parities, population classes, sort decisions
    // and block lengths; a long run with births can meet many keys. The cache
    // is emptied when it reaches kGraphCache entries (the graphs are captured
    // again as the keys recur).
    static constexpr size_t kGraphCache = 256;
    void trim_graph_cache() {
        if (graphs.size() < kGraphCache) return;
        FG_CUDA(cudaStreamSynchronize(stream));
        for (auto& g : graphs) cudaGraphExecDestroy(g.second);
        graphs.clear();
        drop_graph_op_events();
    }

    void invalidate() {
        for (auto& g : graphs) cudaGraphExecDestroy(g.second);
        graphs.clear();
        drop_graph_op_events();
        allocated = false;
    }

    void drop_graph_op_events() {
        for (auto& kv : graph_op_events)
            for (auto& t : kv.second) {
                cudaEventDestroy(std::get<1>(t));
                cudaEventDestroy(std::get<2>(t));
            }
        graph_op_events.clear();
        replayed.clear();
    }

    // Adds the operation times of the last replay of every graph replayed
    // since the previous call to the operation profile (waits for the stream).
    void harvest_graph_ops() {
        if (replayed.empty()) return;
        FG_CUDA(cudaStreamSynchronize(stream));
        for (const auto& key : replayed) {
            auto it = graph_op_events.find(key);
            if (it == graph_op_events.end()) continue;
            for (auto& t : it->second) {
                float ms = 0.0f;
                if (cudaEventElapsedTime(&ms, std::get<1>(t), std::get<2>(t)) != cudaSuccess) continue;
                auto& acc = op_totals[std::get<0>(t)];
                acc.first += ms;
                acc.second += 1;
            }
        }
        replayed.clear();
    }

    // Lists with no population yet still need buffers for their functions.
    void ensure_all_allocated() {
        if (allocated) return;
        for (auto& l : lists)
            if (l->capacity == 0) ensure_capacity(*l, 1024, 0);
        for (auto& m : msgs)
            if (m->capacity == 0) ensure_msg_capacity(*m, 1024);
        // sort workspaces are sized per (list, sorting message grid) up front:
        // nothing may allocate while a step is being captured
        for (auto& f : fns) {
            if (!f.sort_trigger) continue;
            AgentList& l = *f.list;
            if (l.sort_ws.count(f.in)) continue;
            const size_t b = fg_spatial_sort_workspace_size(l.capacity, &f.in->grid);
            if (!b) THROW exception::InvalidMessage("Spatial grid too large for the automatic agent sort");
            l.sort_ws.emplace(f.in, std::make_pair(mem.alloc(b), b));
        }
        for (auto& f : fns) build_tables(f);
        allocated = true;
    }

    // ------------------------------------------------------------- tables

    void build_tables(FnRt& f) {
        AgentList& l = *f.list;
        for (int par = 0; par < 2; ++par) {
            FunctionTables* T = new FunctionTables;
            std::memset(T, 0, sizeof(FunctionTables));
            std::vector<TableEntry> e;
            for (size_t v = 0; v < l.agent->variables.size(); ++v) {
                const Variable& var = l.agent->variables[v];
                e.push_back({fnv1a32(var.name), static_cast<char*>(l.cols[v][par]), var.bytes(), var.type_size, var.elements});
            }
            T->agent = make_table(e, "agent");
            if (f.out) {
                e.clear();
                for (size_t v = 0; v < f.out->msg->variables.size(); ++v) {
                    const Variable& var = f.out->msg->variables[v];
                    e.push_back({fnv1a32(var.name), static_cast<char*>(f.out->cols[v]), f.out->slot_bytes[v], var.type_size, var.elements});
                }
                T->msg_out = make_table(e, "message");
            }
            if (f.in) {
                e.clear();
                for (size_t v = 0; v < f.in->msg->variables.size(); ++v) {
                    const Variable& var = f.in->msg->variables[v];
                    char* p;
                    uint32_t stride;
                    if (f.in->spatial()) {
                        p = reinterpret_cast<char*>(f.in->records + f.in->field_word[v]);
                        stride = f.in->record_words * 4;
                    } else if (f.in->array()) {
                        p = static_cast<char*>(f.in->arr_cols[v]);
                        stride = f.in->slot_bytes[v];
                    } else if (f.in->bucket()) {
                        p = static_cast<char*>(f.in->bk_cols.empty() ? f.in->cols[v] : f.in->bk_cols[v]);
                        stride = f.in->slot_bytes[v];
                    } else {
                        p = static_cast<char*>(f.in->optional_any ? f.in->bf_cols[v] : f.in->cols[v]);
                        stride = f.in->slot_bytes[v];
                    }
                    e.push_back({fnv1a32(var.name), p, stride, var.type_size, var.elements});
                }
                T->msg_in = make_table(e, "message");
            }
            if (f.births) {
                e.clear();
                std::vector<TableEntry> d;
                std::vector<char> defaults;
                std::vector<size_t> doff;
                const AgentData* ba = f.birth_list->agent;
                for (const auto& var : ba->variables) {
                    doff.push_back(defaults.size());
                    defaults.insert(defaults.end(), var.default_value.begin(), var.default_value.end());
                    defaults.resize((defaults.size() + 7) & ~size_t(7));
                }
                if (!f.birth_defaults) f.birth_defaults = mem.alloc(defaults.size());
                FG_CUDA(cudaMemcpy(f.birth_defaults, defaults.data(), defaults.size(), cudaMemcpyHostToDevice));
                for (size_t v = 0; v < ba->variables.size(); ++v) {
                    const Variable& var = ba->variables[v];
                    e.push_back({fnv1a32(var.name), static_cast<char*>(f.birth_cols[v]), var.bytes(), var.type_size, var.elements});
                    d.push_back({fnv1a32(var.name), static_cast<char*>(f.birth_defaults) + doff[v], var.bytes(), var.type_size, var.elements});
                }
                T->birth = make_table(e, "agent");
                T->birth_def = make_table(d, "agent");
            }
            e.clear();
            for (size_t i = 0; i < model->environment.size(); ++i) {
                const EnvProperty& p = model->environment[i];
                // offsets into the environment buffer (LaunchParams::env)
                e.push_back({fnv1a32(p.name), reinterpret_cast<char*>(env_offset[i]), 0, p.type_size, p.elements});
            }
            // macro properties: the stride field holds the offset of the
            // property's flag word (never 0), which marks them as macro properties
            for (size_t i = 0; i < model->macro_environment.size(); ++i) {
                const MacroProperty& p = model->macro_environment[i];
                const uint32_t flag = static_cast<uint32_t>(macro_flags_offset + sizeof(uint32_t) * i);
                e.push_back({fnv1a32(p.name), reinterpret_cast<char*>(macro_offset[i]), flag, p.type_size, p.elements()});
            }
            T->env = make_table(e, "environment");
            f.tables[par].reset(T);
        }
    }

    // ------------------------------------------------------------- step

    uint32_t grid_for(uint32_t n, uint32_t block, int per_sm) const {
        const uint32_t need = std::max(1u, (n + block - 1) / block);
        return std::min(need, static_cast<uint32_t>(sms * per_sm));
    }

    // Capacity check before a step: births can at most double a list per
    // birth function. Synchronises only if the bound could exceed capacity.
    // Births can at most double a list per birth function and step. The check
    // starts from the newest population counts the device has already reported
    // (copied to pinned memory after every step, tagged by an event), so a
    // birth model synchronises only when even that bound could overflow.
    struct CountSlot {
        unsigned int step_after = 0;
        cudaEvent_t ev = nullptr;
        uint32_t* host = nullptr;
        bool used = false;
    };
    std::vector<CountSlot> count_ring;
    size_t count_next = 0;
    uint32_t* count_pinned = nullptr;

    // Whether some function's births are written to list l (fused births are
    // written to the function's own list first, then move with a transition).
    bool receives_births(const AgentList* l) const {
        for (const auto& f : fns)
            if (f.births && (f.birth_list == l || (f.births_fused && f.list == l))) return true;
        return false;
    }
    // Rows to allocate for a population of n: with a population limit, a list
    // that births can grow starts at the limit (the memory a served run was
    // budgeted for), so capacity checks rarely need a count from the device.
    uint32_t initial_capacity(const AgentList* l, uint32_t n) const {
        uint32_t cap = std::max<uint32_t>(1024u, n);
        if (cuda_config.max_agents && receives_births(l)) cap = std::max(cap, cuda_config.max_agents);
        return cap;
    }
    bool any_births() const {
        for (const auto& f : fns)
            if (f.births) return true;
        return false;
    }

    // Populations were replaced from the host: earlier reports no longer apply,
    // and the agents entering the next step are counted again.
    void forget_counts(bool recounted = false) {
        if (!recounted) recount();
        for (auto& c : count_ring) {
            if (c.used) cudaEventSynchronize(c.ev);
            c.used = false;
        }
    }

    void record_counts() {
        if (!any_births()) return;
        if (count_ring.empty()) {
            FG_CUDA(cudaMallocHost(&count_pinned, sizeof(uint32_t) * lists.size() * 4));
            count_ring.resize(4);
            for (size_t k = 0; k < 4; ++k) {
                FG_CUDA(cudaEventCreateWithFlags(&count_ring[k].ev, cudaEventDisableTiming));
                count_ring[k].host = count_pinned + k * lists.size();
            }
        }
        CountSlot& c = count_ring[count_next];
        count_next = (count_next + 1) % count_ring.size();
        if (c.used) FG_CUDA(cudaEventSynchronize(c.ev));  // never overwrite a copy in flight
        for (size_t i = 0; i < lists.size(); ++i)
            FG_CUDA(cudaMemcpyAsync(c.host + i, lists[i]->d_count, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
        FG_CUDA(cudaEventRecord(c.ev, stream));
        c.step_after = step_count + 1;
        c.used = true;
    }

    bool any_transitions() const {
        for (const auto& f : fns)
            if (f.end_list) return true;
        return false;
    }
    size_t list_index(const AgentList* l) const {
        for (size_t i = 0; i < lists.size(); ++i)
            if (lists[i].get() == l) return i;
        return 0;
    }
    // Upper bounds of every list's population `rounds` steps on from `bound`:
    // in layer order, a function with births adds up to its list's bound to
    // its output list, or, fused, to its own list (doubling it: survivors and
    // births share it until a transition moves them on), and a state
    // transition moves up to its list's bound into its end list (not
    // subtracted from the source, so the result stays an upper bound). Capped
    // at 2^33.
    void advance_bounds(std::vector<uint64_t>& bound, uint64_t rounds) const {
        constexpr uint64_t kMax = 1ull << 33;
        if (!any_births() && !any_transitions()) return;
        for (uint64_t r = 0; r < rounds; ++r)
            for (const auto& layer : model->layers)
                for (auto* fd : layer->functions)
                    for (const auto& f : fns) {
                        if (f.fn != fd) continue;
                        const uint64_t src = bound[list_index(f.list)];
                        if (f.births) {
                            uint64_t& t = bound[list_index(f.births_fused ? f.list : f.birth_list)];
                            t = std::min(t + src, kMax);
                        }
                        if (f.end_list) {
                            uint64_t& t = bound[list_index(f.end_list)];
                            t = std::min(t + bound[list_index(f.list)], kMax);
                        }
                    }
    }

    void prepare_capacity() {
        if (!any_births() && !any_transitions()) return;
        // newest reported counts
        const CountSlot* known = nullptr;
        for (size_t k = 0; k < count_ring.size(); ++k) {
            const CountSlot& c = count_ring[k];
            if (!c.used || (known && c.step_after <= known->step_after)) continue;
            if (cudaEventQuery(c.ev) == cudaSuccess) known = &c;
        }
        std::vector<uint64_t> bound(lists.size());
        bool over = false;
        // from the newest report: the steps issued after it, then this one
        const bool have = known && known->step_after <= step_count;
        for (size_t i = 0; i < lists.size(); ++i)
            bound[i] = have ? std::min<uint64_t>(known->host[i], lists[i]->bound) : lists[i]->bound;
        advance_bounds(bound, have ? step_count - known->step_after + 1 : 1);
        for (size_t i = 0; i < lists.size(); ++i)
            if (bound[i] > lists[i]->capacity) over = true;
        if (over) {
            // exact counts after every issued step, then grow what needs it
            sync_counts();
            for (size_t i = 0; i < lists.size(); ++i) bound[i] = lists[i]->bound;
            advance_bounds(bound, 1);
            for (size_t i = 0; i < lists.size(); ++i) {
                if (cuda_config.max_agents && bound[i] > cuda_config.max_agents)
                    THROW exception::OutOfMemory(format("Agent '%s' may reach %llu agents in the next step, above the limit of %u",
                                                        lists[i]->agent->name.c_str(), static_cast<unsigned long long>(bound[i]),
                                                        cuda_config.max_agents));
                if (bound[i] > lists[i]->capacity) {
                    if (bound[i] >= (1ull << 31)) THROW exception::OutOfMemory("Population bound exceeds 2^31 agents");
                    uint64_t want = std::max<uint64_t>(2 * bound[i], 2ull * lists[i]->capacity);
                    if (cuda_config.max_agents) want = std::min<uint64_t>(want, cuda_config.max_agents);
                    ensure_capacity(*lists[i], static_cast<uint32_t>(std::min<uint64_t>(want, (1ull << 31) - 1)), lists[i]->bound);
                }
            }
            ensure_all_allocated();
        }
        for (size_t i = 0; i < lists.size(); ++i) lists[i]->bound = static_cast<uint32_t>(std::min<uint64_t>(bound[i], 0xFFFFFFFFu));
    }

    void sync_counts() {
        FG_CUDA(cudaStreamSynchronize(stream));
        for (auto& l : lists) {
            uint32_t c = 0;
            FG_CUDA(cudaMemcpy(&c, l->d_count, sizeof(uint32_t), cudaMemcpyDeviceToHost));
            l->bound = c;
        }
    }

    std::vector<int> step_key() const {
        std::vector<int> k;
        for (const auto& l : lists) {
            k.push_back(l->parity);
            k.push_back(static_cast<int>(grid_rows(*l)));
        }
        for (const auto& layer : model->layers)
            for (auto* fd : layer->functions) {
                const unsigned p = fd->parent->sort_period;
                k.push_back(p != 0 && step_count % p == 0);
            }
        return k;
    }

    // Runs op() on the stream, bracketed by events when profiling (eager mode).
    template <typename Op>
    void timed(const std::string& label, Op&& op) {
        timed_on(stream, label, std::forward<Op>(op));
    }
    // Runs op() on stream `st`: bracketed by events when profiling (eager), or
    // by event-record nodes of the step graph being captured when
    // Config::time_ops_in_graphs is set.
    template <typename Op>
    void timed_on(cudaStream_t st, const std::string& label, Op&& op) {
        const bool in_graph =
            capturing && (cuda_config.time_ops_in_graphs ||
                          (!cuda_config.time_op_label.empty() && label == cuda_config.time_op_label));
        if (!profiling && !in_graph) {
            op();
            return;
        }
        cudaEvent_t a, b;
        FG_CUDA(cudaEventCreate(&a));
        FG_CUDA(cudaEventCreate(&b));
        if (in_graph) {
            FG_CUDA(cudaEventRecordWithFlags(a, st, cudaEventRecordExternal));
            op();
            FG_CUDA(cudaEventRecordWithFlags(b, st, cudaEventRecordExternal));
            graph_op_events[capture_key].emplace_back(label, a, b);
        } else {
            FG_CUDA(cudaEventRecord(a, st));
            op();
            FG_CUDA(cudaEventRecord(b, st));
            op_events.emplace_back(label, a, b);
        }
    }

    void resolve_profile() {
        for (auto& t : op_events) {
            float ms = 0;
            cudaEventSynchronize(std::get<2>(t));
            cudaEventElapsedTime(&ms, std::get<1>(t), std::get<2>(t));
            auto& acc = op_totals[std::get<0>(t)];
            acc.first += ms;
            acc.second += 1;
            cudaEventDestroy(std::get<1>(t));
            cudaEventDestroy(std::get<2>(t));
        }
        op_events.clear();
    }

    // Whether agent-function launches may compute the keys of the build and
    // sort after them (FLAMEGPU_FUSE_KEYS=0 turns it off).
    static bool fuse_keys_enabled() {
        static const bool on = [] {
            const char* e = std::getenv("FLAMEGPU_FUSE_KEYS");
            return !(e && e[0] == '0');
        }();
        return on;
    }

    // An agent sort and the build of the messages its function reads, both
    // keyed by the launch before, can run as one chain of paired launches
    // (fgi_spatial_sort_and_build: four kernels instead of two concurrent
    // chains of four joined before the function). Measured on the 16,384-agent
    // Boids step the paired chain took 38.0 us a step against 37.1 us for the
    // two branches (each paired launch waits for the slower of its two sorts),
    // so the branches stay the default; FLAMEGPU_PAIR_SORT_BUILD=1 pairs them.
    static bool pair_sort_build_enabled() {
        static const bool on = [] {
            const char* e = std::getenv("FLAMEGPU_PAIR_SORT_BUILD");
            return e && e[0] == '1';
        }();
        return on;
    }

    // Which launches compute the keys of the message build and the agent sort
    // that follow them, so that those pipelines skip their key kernel. A
    // launch f qualifies for the build of its spatial output list m when m is
    // not persistent, f is its only writer this step (no append), f has no
    // condition (its rows are the message rows) and a later function g reads
    // m first; and for the agent sort before g as well when the sort is due,
    // g runs on f's list and no function runs on that list between them, and
    // f neither kills, gives birth nor changes state (the rows sorted are the
    // rows f saw, with the positions f left). Layer host functions, which may
    // change agents between layers, turn it off.
    void plan_keys() {
        for (auto& f : fns) {
            f.key_msg = nullptr;
            f.key_sort = nullptr;
            f.build_keyed = f.sort_keyed = false;
        }
        if (!fuse_keys_enabled() || has_layer_host_functions()) return;
        std::map<const MsgList*, std::pair<FnRt*, int>> writers;  // last writer and writes so far
        std::map<const AgentList*, FnRt*> last_fn;                 // last function run on a list
        std::set<const MsgList*> read;                              // lists already built this step
        for (const auto& layer : model->layers)
            for (auto* fd : layer->functions)
                for (auto& g : fns) {
                    if (g.fn != fd) continue;
                    AgentList* L = g.list;
                    if (g.in && g.in->spatial() && !g.in->msg->persistent && !read.count(g.in)) {
                        read.insert(g.in);
                        const auto w = writers.find(g.in);
                        FnRt* f = w != writers.end() && w->second.second == 1 ? w->second.first : nullptr;
                        if (f && !f->fn->condition && f->list->capacity > 0) {
                            f->key_msg = g.in;
                            g.build_keyed = true;
                            const bool do_sort = g.sort_trigger && L->agent->sort_period != 0 &&
                                                 step_count % L->agent->sort_period == 0;
                            const auto lf = last_fn.find(L);
                            if (do_sort && g.pos_var < 0 && f->list == L && lf != last_fn.end() && lf->second == f &&
                                !f->fn->has_agent_death && !f->births && !f->end_list) {
                                f->key_sort = &g;
                                g.sort_keyed = true;
                            }
                        }
                    }
                    if (g.out) {
                        auto& w = writers[g.out];
                        w.first = &g;
                        ++w.second;
                    }
                    last_fn[L] = &g;
                    if (g.end_list) last_fn[g.end_list] = &g;
                }
    }

    // The key target of f's launch for the build of f.key_msg / the sort of
    // its list before f.key_sort.
    KeyTarget build_key_target(const FnRt& f) {
        MsgList& m = *f.key_msg;
        KeyTarget t;
        FG_CAPI(fgi_key_target(&m.grid, m.capacity, false, m.build_ws, m.build_ws_bytes, &t));
        t.x = static_cast<const float*>(m.cols[0]);  // x, y, z are the first message variables
        t.y = static_cast<const float*>(m.cols[1]);
        t.z = m.grid.dims == 3 ? static_cast<const float*>(m.cols[2]) : nullptr;
        return t;
    }
    KeyTarget sort_key_target(const FnRt& f) {
        const FnRt& g = *f.key_sort;
        AgentList& l = *f.list;
        const auto it = l.sort_ws.find(g.in);
        if (it == l.sort_ws.end()) THROW exception::InvalidOperation("Sort workspace missing (not allocated before capture)");
        KeyTarget t;
        FG_CAPI(fgi_key_target(&g.in->grid, l.capacity, true, it->second.first, it->second.second, &t));
        const int xi = l.var_index("x"), yi = l.var_index("y"), zi = l.var_index("z");
        t.x = static_cast<const float*>(l.cols[xi][l.parity]);
        t.y = static_cast<const float*>(l.cols[yi][l.parity]);
        t.z = g.in->grid.dims == 3 ? static_cast<const float*>(l.cols[zi][l.parity]) : nullptr;
        return t;
    }

    void enqueue_sort(FnRt& f) {
        AgentList& l = *f.list;
        const fg_spatial_grid* g = &f.in->grid;
        auto it = l.sort_ws.find(f.in);
        if (it == l.sort_ws.end()) THROW exception::InvalidOperation("Sort workspace missing (not allocated before capture)");
        std::vector<fg_column> cols(l.cols.size());
        for (size_t v = 0; v < l.cols.size(); ++v)
            cols[v] = fg_column{l.cols[v][l.parity], l.cols[v][l.parity ^ 1], l.agent->variables[v].bytes()};
        const float *px, *py, *pz;
        uint32_t stride = 1;
        if (f.pos_var >= 0) {  // packed: row i's coordinates at [dims * i + a]
            px = static_cast<const float*>(l.cols[f.pos_var][l.parity]);
            py = px + 1;
            pz = g->dims == 3 ? px + 2 : nullptr;
            stride = static_cast<uint32_t>(g->dims);
        } else {
            const int xi = l.var_index("x"), yi = l.var_index("y"), zi = l.var_index("z");
            px = static_cast<const float*>(l.cols[xi][l.parity]);
            py = static_cast<const float*>(l.cols[yi][l.parity]);
            pz = g->dims == 3 ? static_cast<const float*>(l.cols[zi][l.parity]) : nullptr;
        }
        FG_CAPI(fgi_spatial_sort_agents(g, l.capacity, l.d_count, px, py, pz, cols.data(),
                                        static_cast<uint32_t>(cols.size()), nullptr, it->second.first,
                                        it->second.second, stream, f.sort_keyed, stride));
        l.parity ^= 1;
        kernel_counter += f.sort_keyed ? 4 : 5;
    }

    // The record layout of a message list's sorted records: each record word's
    // source column, stride and word.
    static fg_record_desc record_desc_of(const MsgList& m) {
        fg_record_desc rec;
        std::memset(&rec, 0, sizeof(rec));
        rec.words = m.record_words;
        for (size_t v = 0; v < m.cols.size(); ++v) {
            const uint32_t words = m.slot_bytes[v] / 4;
            for (uint32_t k = 0; k < words; ++k) {
                const uint32_t w = m.field_word[v] + k;
                rec.src[w] = static_cast<const uint32_t*>(m.cols[v]);
                rec.src_stride[w] = words;
                rec.src_word[w] = k;
            }
        }
        return rec;
    }

    // f's agent sort and its input's build as one chain (both keyed).
    void enqueue_sort_and_build(FnRt& f) {
        AgentList& l = *f.list;
        MsgList& m = *f.in;
        auto it = l.sort_ws.find(f.in);
        if (it == l.sort_ws.end()) THROW exception::InvalidOperation("Sort workspace missing (not allocated before capture)");
        std::vector<fg_column> cols(l.cols.size());
        for (size_t v = 0; v < l.cols.size(); ++v)
            cols[v] = fg_column{l.cols[v][l.parity], l.cols[v][l.parity ^ 1], l.agent->variables[v].bytes()};
        const fg_record_desc rec = record_desc_of(m);
        FG_CAPI(fgi_spatial_sort_and_build(&m.grid, l.capacity, l.d_count, cols.data(), static_cast<uint32_t>(cols.size()),
                                           it->second.first, it->second.second, m.capacity, m.d_count, &rec, m.records,
                                           m.pbm, m.build_ws, m.build_ws_bytes, stream));
        l.parity ^= 1;
        m.needs_build = false;
        kernel_counter += 4;
    }

    void enqueue_build(MsgList& m, cudaStream_t st, bool keys_ready = false) {
        const fg_record_desc rec = record_desc_of(m);
        const int dims = m.grid.dims;
        const int xi = 0, yi = 1, zi = 2;  // x, y, z are the first message variables
        FG_CAPI(fgi_spatial_build(&m.grid, m.capacity, m.d_count, static_cast<const float*>(m.cols[xi]),
                                  static_cast<const float*>(m.cols[yi]), dims == 3 ? static_cast<const float*>(m.cols[zi]) : nullptr,
                                  m.optional_any ? m.valid : nullptr, &rec, m.records, m.pbm, m.build_ws, m.build_ws_bytes,
                                  st, keys_ready));
        m.needs_build = false;
        kernel_counter += keys_ready ? 4 : 5;
    }

    // The array of message list m from this step's output: cleared, then each
    // output message copied to its index (k_array_scatter).
    void enqueue_array_build(MsgList& m) {
        for (size_t v = 0; v < m.arr_cols.size(); ++v)
            FG_CUDA(cudaMemsetAsync(m.arr_cols[v], 0, static_cast<size_t>(m.slot_bytes[v]) * m.arr_len, stream));
        FG_CUDA(cudaMemsetAsync(m.arr_claim, 0, sizeof(uint32_t) * m.arr_len, stream));
        if (m.capacity > 0) {
            ArrayScatter a;
            std::memset(&a, 0, sizeof(a));
            int index_var = -1;
            for (size_t v = 0; v < m.msg->variables.size(); ++v) {
                if (m.msg->variables[v].name == "___INDEX") index_var = static_cast<int>(v);
                a.src[v] = static_cast<const char*>(m.cols[v]);
                a.dst[v] = static_cast<char*>(m.arr_cols[v]);
                a.bytes[v] = m.slot_bytes[v];
            }
            a.ncols = static_cast<uint32_t>(m.msg->variables.size());
            a.index = static_cast<const uint32_t*>(m.cols[index_var]);
            a.valid = m.valid;
            a.d_count = m.d_count;
            a.max_n = m.capacity;
            a.length = m.arr_len;
            a.claim = m.arr_claim;
            a.error = d_error();
            const unsigned int grid = std::max(1u, std::min((m.capacity + 255u) / 256u, static_cast<unsigned int>(sms) * 8u));
            FG_CUDA(launch_kernel(pdl_enabled(), k_array_scatter, grid, 256, 0, stream, a));
            kernel_counter += 1;
        }
        m.needs_build = false;
    }

    // The buckets of message list m from this step's output: the rows' keys
    // (k_bucket_keys), a stable radix sort of the rows by key over the list's
    // capacity (the host sort's kernels), the PBM as the exclusive scan of the
    // bucket counts, every column gathered in sorted order.
    void enqueue_bucket_build(MsgList& m) {
        FG_CUDA(cudaMemsetAsync(m.bk_hist, 0, sizeof(uint32_t) * (static_cast<size_t>(m.bk_buckets) + 2), stream));
        const uint32_t cap = m.capacity;
        if (cap == 0) {
            FG_CUDA(cudaMemsetAsync(m.bk_pbm, 0, sizeof(uint32_t) * (static_cast<size_t>(m.bk_buckets) + 2), stream));
            m.needs_build = false;
            return;
        }
        int key_var = -1;
        for (size_t v = 0; v < m.msg->variables.size(); ++v)
            if (m.msg->variables[v].name == "___KEY") key_var = static_cast<int>(v);
        const unsigned int grid = std::max(1u, std::min((cap + 255u) / 256u, static_cast<unsigned int>(sms) * 8u));
        FG_CUDA(launch_kernel(pdl_enabled(), k_bucket_keys, grid, 256, 0, stream, static_cast<const int32_t*>(m.cols[key_var]),
                              static_cast<const uint32_t*>(m.valid), static_cast<const uint32_t*>(m.d_count), cap, m.bk_lower,
                              m.bk_buckets, m.bk_keys[0], m.bk_rows[0], m.bk_hist));
        kernel_counter += 1;
        uint32_t bits = 1;
        while (bits < 32 && (1ull << bits) <= m.bk_buckets) ++bits;  // keys 0 .. buckets
        const uint32_t ntiles = (cap + kSortTile - 1) / kSortTile;
        int cur = 0;
        for (uint32_t shift = 0; shift < bits; shift += 8, cur ^= 1) {
            FG_CUDA(launch_kernel(pdl_enabled(), k_hsort_counts, ntiles, 256, 0, stream,
                                  static_cast<const uint64_t*>(m.bk_keys[cur]), cap, shift, ntiles, m.bk_counts));
            FG_CAPI(fg_exclusive_scan_u32(m.bk_counts, m.bk_starts, 256u * ntiles, m.bk_ws, m.bk_ws_bytes, stream));
            FG_CUDA(launch_kernel(pdl_enabled(), k_hsort_scatter, ntiles, 256, 0, stream,
                                  static_cast<const uint64_t*>(m.bk_keys[cur]), static_cast<const uint32_t*>(m.bk_rows[cur]),
                                  m.bk_keys[cur ^ 1], m.bk_rows[cur ^ 1], cap, shift, ntiles,
                                  static_cast<const uint32_t*>(m.bk_starts)));
            kernel_counter += 3;
        }
        FG_CAPI(fg_exclusive_scan_u32(m.bk_hist, m.bk_pbm, m.bk_buckets + 1u, m.bk_ws, m.bk_ws_bytes, stream));
        kernel_counter += 1;
        for (size_t v = 0; v < m.cols.size(); ++v) {
            FG_CUDA(launch_kernel(pdl_enabled(), k_hsort_gather, grid, 256, 0, stream, static_cast<const char*>(m.cols[v]),
                                  static_cast<char*>(m.bk_cols[v]), m.slot_bytes[v], static_cast<const uint32_t*>(m.bk_rows[cur]),
                                  cap));
            kernel_counter += 1;
        }
        m.needs_build = false;
    }

    // Rows an agent-function launch of list l covers with one block per 128
    // rows: the host's bound on its population rounded up to a power of two
    // (at least one wave of 8 blocks per SM), at most its capacity. The
    // kernels loop over the rows, so a population above this takes more rounds
    // per block, never a wrong result; a population far below its capacity
    // (a decaying birth/death run) launches few blocks. The step graphs are
    // keyed by it, so a change of class captures a graph sized for it.
    uint32_t grid_rows(const AgentList& l) const {
        uint64_t r = 1;
        while (r < l.bound) r <<= 1;
        r = std::max<uint64_t>(r, 8ull * static_cast<uint64_t>(sms) * kAgentBlock);
        return static_cast<uint32_t>(std::min<uint64_t>(r, std::max(l.capacity, 1u)));
    }
    // Threads per agent-function block: CUDAConfig::agent_block if set (32,
    // 64 or 128), else 128; FLAMEGPU_AGENT_BLOCK overrides it. Measured on
    // the 16,384-agent Boids step (one block per SM or fewer): 64 threads ran
    // as fast as 128 and 32 a third slower, since each agent's walk over its
    // neighbourhood, not the number of SMs taking part, sets the time.
    unsigned int agent_block(uint32_t) const {
        static const unsigned int env = [] {
            const char* e = std::getenv("FLAMEGPU_AGENT_BLOCK");
            const unsigned int v = e ? static_cast<unsigned int>(std::atoi(e)) : 0u;
            return (v == 32u || v == 64u || v == 128u) ? v : 0u;
        }();
        if (env) return env;
        const unsigned int c = cuda_config.agent_block;
        return (c == 32u || c == 64u || c == 128u) ? c : kAgentBlock;
    }
    unsigned int agent_grid(uint32_t rows, unsigned int block) const {
        return std::min(std::max(1u, (rows + block - 1) / block), 1u << 17);
    }

    static bool stage_window_fits(const MsgList& m, unsigned int stage_bytes, unsigned int block) {
        const double per_bin = static_cast<double>(m.capacity) / std::max<uint32_t>(m.grid.binCount, 1u);
        return detail::stage_window_fits(m.grid, per_bin, m.record_words, block, stage_bytes);
    }

    void enqueue_function(FnRt& f) {
        AgentList& l = *f.list;
        bool do_sort = false;
        if (f.sort_trigger && l.agent->sort_period != 0 && step_count % l.agent->sort_period == 0)
            do_sort = true;
        const bool do_build = f.in && f.in->spatial() && f.in->needs_build;
        if (do_sort && do_build && f.sort_keyed && f.build_keyed && pair_sort_build_enabled()) {
            timed("sort+build:" + l.agent->name + "/" + f.in->msg->name, [&] { enqueue_sort_and_build(f); });
        } else if (do_sort && do_build && cuda_config.inLayerConcurrency && !profiling) {
            // the agent sort and the message index build touch disjoint buffers:
            // two branches of the step graph (fork/join through events)
            FG_CUDA(cudaEventRecord(fork_ev, stream));
            FG_CUDA(cudaStreamWaitEvent(side, fork_ev, 0));
            timed_on(side, "build:" + f.in->msg->name, [&] { enqueue_build(*f.in, side, f.build_keyed); });
            timed_on(stream, "sort:" + l.agent->name, [&] { enqueue_sort(f); });
            FG_CUDA(cudaEventRecord(join_ev, side));
            FG_CUDA(cudaStreamWaitEvent(stream, join_ev, 0));
        } else {
            if (do_sort) timed("sort:" + l.agent->name, [&] { enqueue_sort(f); });
            if (do_build) timed("build:" + f.in->msg->name, [&] { enqueue_build(*f.in, stream, f.build_keyed); });
        }
        if (f.in && f.in->array() && f.in->needs_build)
            timed("build:" + f.in->msg->name, [&] { enqueue_array_build(*f.in); });
        if (f.in && f.in->bucket() && f.in->needs_build)
            timed("build:" + f.in->msg->name, [&] { enqueue_bucket_build(*f.in); });
        const bool append = f.out && f.out->written;
        if (f.out) {
            f.out->written = true;
            // the base of an appending output: the messages so far this step,
            // none if no launch with agents has output yet (the list is truncated)
            if (append) {
                FG_CUDA(launch_kernel(pdl_enabled(), k_append_base, 1, 1, 0, stream, f.out->d_base,
                                      static_cast<const uint32_t*>(f.out->d_count),
                                      static_cast<const uint32_t*>(f.out->d_filled)));
                kernel_counter += 1;
            }
        }
        if (f.fn->condition) {
            // FLAMEGPU_AGENT_FUNCTION_CONDITION, then the failing agents to the
            // front of the list and the others after them
            // (CUDASimulation.cu:820-836, CUDAFatAgent.cu:186-236)
            LaunchParams C;
            std::memset(&C, 0, sizeof(C));
            C.T = *f.tables[l.parity];
            C.max_n = l.capacity;
            C.d_n = l.d_count;
            C.cond_fail = f.cond_fail;
            C.d_step = d_step();
            C.seed = config.random_seed;
            C.fn_uid = f.fn->uid;
            C.agent_hash = fnv1a32(l.agent->name);
            C.state_hash = fnv1a32(f.fn->initial_state);
            C.error = d_error();
            C.env = d_env;
            cudaError_t ce = cudaSuccess;
            timed("cond:" + f.fn->name, [&] {
                ce = f.fn->condition(C, agent_grid(grid_rows(l) + 1, kAgentBlock), kAgentBlock, 0, stream,
                                     detail::pdl_enabled());
            });
            if (ce != cudaSuccess)
                THROW exception::CUDAError(format("Launch of the condition of '%s' failed: %s", f.fn->name.c_str(), cudaGetErrorString(ce)));
            std::vector<fg_column> pc(l.cols.size());
            for (size_t v = 0; v < l.cols.size(); ++v)
                pc[v] = fg_column{l.cols[v][l.parity], l.cols[v][l.parity ^ 1], l.agent->variables[v].bytes()};
            timed("partition:" + l.agent->name, [&] {
                FG_CAPI(fg_partition_agents(l.capacity, l.d_count, f.cond_fail, pc.data(), static_cast<uint32_t>(pc.size()),
                                            f.d_first, l.comp_ws, l.comp_ws_bytes, stream));
            });
            l.parity ^= 1;
            kernel_counter += 3;
        }
        LaunchParams P;
        std::memset(&P, 0, sizeof(P));
        P.T = *f.tables[l.parity];
        P.max_n = l.capacity;
        P.d_n = l.d_count;
        P.d_first = f.fn->condition ? f.d_first : nullptr;
        if (f.out) {
            // an array message is output where its agent set the index
            // an array or bucket message is output where its agent set the index or key
            const bool placed = f.out->array() || f.out->bucket();
            P.msg_out_valid = (f.out->optional_any || placed) ? f.out->valid : nullptr;
            P.msg_out_always = (f.fn->message_output_optional || placed) ? 0 : 1;
            for (int a = 0; a < 3; ++a) P.out_dims[a] = f.out->arr_dims[a];
            P.out_key_lo = f.out->bk_lower;
            P.out_key_hi = static_cast<int32_t>(static_cast<int64_t>(f.out->bk_lower) + f.out->bk_buckets);
            P.msg_out_count = f.out->d_count;
            P.msg_out_base = append ? f.out->d_base : nullptr;
            P.msg_out_filled = f.out->d_filled;
            P.msg_out_enabled = 1;
        }
        if (f.in) {
            if (f.in->spatial()) {
                P.in_grid = f.in->grid;
                P.in_pbm = f.in->pbm;
                P.in_count = f.in->pbm + f.in->grid.binCount;
                P.in_records = reinterpret_cast<const char*>(f.in->records);
                P.in_record_bytes = f.in->record_words * 4u;
                P.in_pay_mult = f.in->pay_mult;
                P.in_pay_shift = f.in->pay_shift;
                P.in_pay_stride = f.in->pay_stride;
                P.in_pbm_alloc = f.in->pbm_alloc;
                if (f.stage && cuda_config.message_stage_bytes >= 1024u &&
                    stage_window_fits(*f.in, cuda_config.message_stage_bytes, agent_block(grid_rows(l))))
                    P.stage_bytes = (cuda_config.message_stage_bytes + 15u) & ~15u;
            } else if (f.in->array()) {
                P.in_count = f.in->arr_count;
                for (int a = 0; a < 3; ++a) P.in_dims[a] = f.in->arr_dims[a];
            } else if (f.in->bucket()) {
                P.in_pbm = f.in->bk_pbm;
                P.in_count = f.in->bk_pbm + f.in->bk_buckets;
                P.in_key_lo = f.in->bk_lower;
                P.in_key_hi = static_cast<int32_t>(static_cast<int64_t>(f.in->bk_lower) + f.in->bk_buckets);
            } else {
                P.in_count = f.in->optional_any ? f.in->bf_count : f.in->d_count;
            }
        }
        P.birth_flags = f.births ? f.birth_flags : nullptr;
        P.birth_next_id = f.births ? d_next_id(agent_index(f.birth_list->agent)) : nullptr;
        P.death_flags = f.fn->has_agent_death ? f.death_flags : nullptr;
        // the survivors are counted by the launch itself into the compaction
        // workspace's header (the compaction then reads them there, and its
        // last block resets the word): no counting kernel before it
        P.alive_count = f.fn->has_agent_death ? survivors_word(l) : nullptr;
        P.d_step = d_step();
        P.seed = config.random_seed;
        P.fn_uid = f.fn->uid;
        P.agent_hash = fnv1a32(l.agent->name);
        P.state_hash = fnv1a32(f.fn->initial_state);
        P.error = d_error();
        P.env = d_env;
        if (f.key_msg) P.keyed[0] = build_key_target(f);
        if (f.key_sort) P.keyed[1] = sort_key_target(f);
        cudaError_t e = cudaSuccess;
        const unsigned int smem = P.stage_bytes ? P.stage_bytes + static_cast<unsigned int>(sizeof(StageHeader)) : 0u;
        // one block per 128 rows (no grid-stride reuse): blocks stay short, so
        // kernels of other simulations on the device (a server's other runs,
        // higher-priority streams) get SMs between them
        timed("fn:" + f.fn->name, [&] {
            const unsigned int block = agent_block(grid_rows(l));
            e = f.fn->launcher(P, agent_grid(grid_rows(l), block), block, smem, stream, detail::pdl_enabled());
        });
        if (e != cudaSuccess)
            THROW exception::CUDAError(format("Launch of agent function '%s' failed: %s", f.fn->name.c_str(), cudaGetErrorString(e)));
        kernel_counter += 1;
        if (f.out) {
            f.out->needs_build = true;
            if (!f.out->spatial() && !f.out->array() && !f.out->bucket() && f.out->optional_any) {
                // brute-force optional output: stable compaction of the message rows
                std::vector<fg_column> cols(f.out->cols.size());
                for (size_t v = 0; v < cols.size(); ++v) cols[v] = fg_column{f.out->cols[v], f.out->bf_cols[v], f.out->slot_bytes[v]};
                FG_CAPI(fg_compact_agents(f.out->capacity, f.out->d_count, f.out->valid, nullptr, cols.data(), nullptr,
                                          static_cast<uint32_t>(cols.size()), -1, nullptr, nullptr, f.out->bf_count,
                                          f.out->capacity, f.out->bf_ws, f.out->bf_ws_bytes, stream));
                kernel_counter += 2;
            }
        }
        // births into another list: the rows the function ran over, before the
        // death compaction and transition change the list's count
        const bool fused = f.births && f.births_fused;
        if (f.births && !fused) {
            FG_CUDA(cudaMemcpyAsync(f.d_launch_n, l.d_count, sizeof(uint32_t), cudaMemcpyDeviceToDevice, stream));
        }
        if (f.fn->has_agent_death || fused) {
            std::vector<fg_column> cols(l.cols.size()), bcols(l.cols.size());
            int id_col = -1;
            for (size_t v = 0; v < l.cols.size(); ++v) {
                const uint32_t b = l.agent->variables[v].bytes();
                cols[v] = fg_column{l.cols[v][l.parity], l.cols[v][l.parity ^ 1], b};
                bcols[v] = fg_column{fused ? f.birth_cols[v] : l.cols[v][l.parity], l.cols[v][l.parity ^ 1], b};
                if (l.agent->variables[v].name == "_id") id_col = static_cast<int>(v);
            }
            // survivors: counted by the function's launch (death), else all n
            const uint32_t* survivors = f.fn->has_agent_death ? survivors_word(l) : l.d_count;
            timed("compact:" + l.agent->name, [&] {
                FG_CAPI(fg_compact_agents(l.capacity, l.d_count, f.fn->has_agent_death ? f.death_flags : nullptr,
                                          fused ? f.birth_flags : nullptr, cols.data(), bcols.data(),
                                          static_cast<uint32_t>(cols.size()), fused ? id_col : -1,
                                          fused ? d_next_id(agent_index(l.agent)) : nullptr, survivors, l.d_count,
                                          l.capacity, l.comp_ws, l.comp_ws_bytes, stream));
            });
            l.parity ^= 1;
            kernel_counter += 1;
        }
        if (f.end_list) {
            // state transition (CUDAFatAgent.cu:139-184): the agents that ran the
            // function (and their births) are appended, in order, to the end
            // state's list; the list keeps the agents that failed the condition
            AgentList& E = *f.end_list;
            std::vector<fg_column> tc(l.cols.size());
            for (size_t v = 0; v < l.cols.size(); ++v)
                tc[v] = fg_column{l.cols[v][l.parity], E.cols[v][E.parity], l.agent->variables[v].bytes()};
            timed("transition:" + l.agent->name, [&] {
                FG_CAPI(fg_append_rows(tc.data(), static_cast<uint32_t>(tc.size()), l.capacity,
                                       f.fn->condition ? f.d_first : nullptr, l.d_count, E.d_count, E.capacity, E.comp_ws,
                                       E.comp_ws_bytes, stream));
            });
            kernel_counter += 2;
        }
        if (f.births && !fused) {
            // CUDAAgent::scatterNew (CUDAAgent.cu:427-450): the new agents are
            // appended after the output list's agents, in parent order
            AgentList& B = *f.birth_list;
            std::vector<fg_column> bc(B.cols.size());
            int id_col = -1;
            for (size_t v = 0; v < B.cols.size(); ++v) {
                bc[v] = fg_column{f.birth_cols[v], B.cols[v][B.parity], B.agent->variables[v].bytes()};
                if (B.agent->variables[v].name == "_id") id_col = static_cast<int>(v);
            }
            timed("birth:" + B.agent->name, [&] {
                FG_CAPI(fg_append_births(l.capacity, f.d_launch_n, f.birth_flags, bc.data(), static_cast<uint32_t>(bc.size()),
                                         id_col, d_next_id(agent_index(B.agent)), B.d_count, B.capacity, l.comp_ws,
                                         l.comp_ws_bytes, stream));
            });
            kernel_counter += 1;
        }
        // every agent function starts with its macro properties neither read nor updated
        if (macro_flag_bytes) FG_CUDA(cudaMemsetAsync(d_env + macro_flags_offset, 0, macro_flag_bytes, stream));
    }

    // populations no kernel changes: the agents of the step being issued
    void count_host_step() {
        if (counts_on_device()) return;
        for (const auto& l : lists) host_agent_steps += l->bound;
    }

    void enqueue_step() {
        kernel_counter = 0;
        for (auto& m : msgs) {
            if (!m->msg->persistent) m->needs_build = true;
            m->written = false;
        }
        plan_keys();
        for (const auto& layer : model->layers) {
            for (auto* fd : layer->functions)
                for (auto& f : fns)
                    if (f.fn == fd) enqueue_function(f);
        }
        enqueue_step_end();
        kernel_counter += 1;
    }

    // non-persistent messages are cleared at the end of the step
    // (CUDASimulation.cu:619-625), then the step counter advances
    void enqueue_step_end() {
        StepEnd e{};
        auto clear = [&](uint32_t* p) {
            if (e.nclear < kStepEndClears)
                e.clear[e.nclear++] = p;
            else
                FG_CUDA(cudaMemsetAsync(p, 0, sizeof(uint32_t), stream));
        };
        for (auto& m : msgs) {
            if (!m->msg->persistent) {
                clear(m->d_count);
                if (m->bf_count) clear(m->bf_count);
            }
            clear(m->d_filled);  // the next step's first output truncates the list
        }
        e.d_step = d_step();
        count_targets(e);
        FG_CUDA(launch_kernel(pdl_enabled(), k_step_end, 1, 32, 0, stream, e));
    }

    // Every list's count, for the agent-step accumulator (models of at most
    // kStepEndCounts agent lists; beyond that, no count is kept). Only models
    // whose populations change on the device (birth, death, state
    // transitions) count there; the others' counts are the host's (host_steps).
    bool counts_on_device() const {
        if (any_births() || any_transitions()) return true;
        for (const auto& f : fns)
            if (f.fn->has_agent_death) return true;
        return false;
    }
    void count_targets(StepEnd& e) const {
        if (lists.size() > kStepEndCounts || !counts_on_device()) return;
        for (const auto& l : lists) e.counts[e.ncounts++] = l->d_count;
        e.acc = d_agent_steps;
    }
    // After a population is set from the host: the agents entering the next step.
    void recount() {
        StepEnd e{};
        count_targets(e);
        if (e.acc) FG_CUDA(launch_kernel(pdl_enabled(), k_recount, 1, 32, 0, stream, e));
    }

    bool has_layer_host_functions() const {
        for (const auto& l : model->layers)
            if (!l->host_functions.empty()) return true;
        return false;
    }

    // Agents created by host functions join their populations (after the
    // existing agents, in creation order, with fresh ids), as the reference adds
    // them when the host function returns (HostAgentAPI::newAgent).
    // A host function's population view reaches the device before a device
    // reduction or sort of that population reads it, and a sort reorders it
    // (the reference's DeviceAgentVector synchronisation).
    void sync_host_view(const std::string& a, const std::string& s) {
        auto it = host_views.find({a, s});
        if (it != host_views.end() && it->second) owner->setPopulationData(*it->second, s);
    }
    void refresh_host_view(const std::string& a, const std::string& s) {
        auto it = host_views.find({a, s});
        if (it != host_views.end() && it->second) owner->getPopulationData(*it->second, s);
    }

    void flush_host_births() {
        for (auto& kv : host_views)
            if (kv.second) owner->setPopulationData(*kv.second, kv.first.second);
        host_views.clear();
        for (auto& kv : host_births) {
            AgentVector& add = *kv.second;
            if (add.empty()) continue;
            AgentVector pop(AgentDescription(model, const_cast<AgentData*>(add.getAgentData())));
            owner->getPopulationData(pop, kv.first.second);
            const flamegpu::size_type n = pop.size(), k = add.size();
            pop.resize(n + k);
            const auto& vars = add.getAgentData()->variables;
            for (size_t v = 0; v < vars.size(); ++v) {
                const size_t b = vars[v].bytes();
                std::memcpy(pop.columns()[v].data() + n * b, add.columns()[v].data(), k * b);
            }
            owner->setPopulationData(pop, kv.first.second);
            add.clear();
        }
    }

    void run_host_layer(LayerData* layer, HostAPI& api) {
        FG_CUDA(cudaStreamSynchronize(stream));
        for (auto fn : layer->host_functions) fn(&api);
        flush_host_births();
        upload_env_if_dirty();
    }

    void upload_env_if_dirty() {
        if (!env_dirty) return;
        FG_CUDA(cudaMemcpyAsync(d_env, env_host.data(), env_host.size(), cudaMemcpyHostToDevice, stream));
        FG_CUDA(cudaStreamSynchronize(stream));
        env_dirty = false;
    }

    void step_once(CUDASimulation* owner) {
        ensure_all_allocated();
        prepare_capacity();
        upload_env_if_dirty();
        cudaEvent_t e0, e1;
        FG_CUDA(cudaEventCreate(&e0));
        FG_CUDA(cudaEventCreate(&e1));
        FG_CUDA(cudaEventRecord(e0, stream));
        profiling = cuda_config.profile_ops;
        if (has_layer_host_functions() || !cuda_config.use_graphs || profiling) {
            HostAPI api(this);
            kernel_counter = 0;
            for (auto& m : msgs) {
                if (!m->msg->persistent) m->needs_build = true;
                m->written = false;
            }
            plan_keys();
            for (const auto& layer : model->layers) {
                if (!layer->host_functions.empty()) {
                    run_host_layer(layer.get(), api);
                    continue;
                }
                for (auto* fd : layer->functions)
                    for (auto& f : fns)
                        if (f.fn == fd) enqueue_function(f);
            }
            enqueue_step_end();
            kernels_last_step = kernel_counter + 1;
        } else {
            const std::vector<int> key = step_key();
            std::vector<int> parity_before;
            for (auto& l : lists) parity_before.push_back(l->parity);
            auto it = graphs.find(key);
            if (it == graphs.end()) {
                cudaGraph_t g;
                FG_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
                capturing = true;
                capture_key = key;
                try {
                    enqueue_step();
                } catch (...) {
                    capturing = false;
                    cudaStreamEndCapture(stream, &g);
                    throw;
                }
                capturing = false;
                FG_CUDA(cudaStreamEndCapture(stream, &g));
                cudaGraphExec_t ge;
                FG_CUDA(cudaGraphInstantiate(&ge, g, 0));
                cudaGraphDestroy(g);
                trim_graph_cache();
                it = graphs.emplace(key, ge).first;
                kernels_last_step = kernel_counter;
            } else {
                // replay: apply the host-side effects of the step (buffer parities)
                for (size_t i = 0; i < lists.size(); ++i) lists[i]->parity = parity_before[i];
                simulate_parity_flips();
            }
            FG_CUDA(cudaGraphLaunch(it->second, stream));
            ++graph_launches;
            if (cuda_config.time_ops_in_graphs || !cuda_config.time_op_label.empty()) replayed.insert(key);
        }
        FG_CUDA(cudaEventRecord(e1, stream));
        step_events.push_back({e0, e1, 1u});
        record_counts();
        count_host_step();
        // step functions, then exit conditions, see the step that is ending;
        // the counter advances after them (CUDASimulation.cu:612-637)
        exit_requested = false;
        if (!model->step_functions.empty() || !model->exit_conditions.empty()) {
            FG_CUDA(cudaStreamSynchronize(stream));
            HostAPI api(this);
            for (auto fn : model->step_functions) fn(&api);
            for (auto fn : model->exit_conditions)
                if (fn(&api) == EXIT) {
                    exit_requested = true;
                    break;
                }
            flush_host_births();
            upload_env_if_dirty();
        }
        ++step_count;
        if (cuda_config.check_each_step) owner->synchronize();
        owner->processStepLog(-1.0);
    }

    // Whether steps may be replayed several per graph: no host work between
    // steps (host layers, step functions, step log), no state transitions
    // (their capacity is checked on the host each step), graphs on, no
    // per-operation timing or per-step checks. Births are allowed: a block
    // is only as long as the worst-case growth keeps within capacity.
    bool multi_step_ok(bool step_log) const {
        return cuda_config.use_graphs && !cuda_config.profile_ops && !cuda_config.time_ops_in_graphs &&
               !cuda_config.check_each_step && !step_log && !has_layer_host_functions() &&
               model->step_functions.empty() && model->exit_conditions.empty() && !any_transitions();
    }

    // Up to Smax steps as one captured graph, cached by the buffer parities
    // and population classes at its start and every step's sort decisions.
    // With births, the block ends where the population bound (doubling per
    // birth function and step) could pass a list's capacity. Returns the
    // steps run.
    unsigned int step_block(unsigned int Smax) {
        ensure_all_allocated();
        prepare_capacity();  // room for one step; bounds after it
        upload_env_if_dirty();
        // the block ends before a step whose population bound could pass a
        // list's capacity; `after` holds the bounds after its last step
        unsigned int S = 1;
        std::vector<uint64_t> after(lists.size());
        for (size_t i = 0; i < lists.size(); ++i) after[i] = lists[i]->bound;
        while (S < Smax) {
            std::vector<uint64_t> next = after;
            advance_bounds(next, 1);
            bool fits = true;
            for (size_t i = 0; i < lists.size(); ++i) {
                uint64_t cap = lists[i]->capacity;
                if (cuda_config.max_agents) cap = std::min<uint64_t>(cap, cuda_config.max_agents);
                fits = fits && next[i] <= cap;
            }
            if (!fits) break;
            after.swap(next);
            ++S;
        }
        const unsigned int first = step_count;
        std::vector<int> key{-static_cast<int>(S)};
        std::vector<int> parity_before;
        for (auto& l : lists) {
            key.push_back(l->parity);
            key.push_back(static_cast<int>(grid_rows(*l)));
            parity_before.push_back(l->parity);
        }
        for (unsigned int j = 0; j < S; ++j)
            for (const auto& layer : model->layers)
                for (auto* fd : layer->functions) {
                    const unsigned p = fd->parent->sort_period;
                    key.push_back(p != 0 && (first + j) % p == 0);
                }
        cudaEvent_t e0, e1;
        FG_CUDA(cudaEventCreate(&e0));
        FG_CUDA(cudaEventCreate(&e1));
        FG_CUDA(cudaEventRecord(e0, stream));
        profiling = false;
        auto it = graphs.find(key);
        if (it == graphs.end()) {
            cudaGraph_t g;
            FG_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
            capturing = true;
            capture_key = key;
            try {
                for (unsigned int j = 0; j < S; ++j, ++step_count) enqueue_step();
            } catch (...) {
                step_count = first;
                capturing = false;
                cudaStreamEndCapture(stream, &g);
                throw;
            }
            step_count = first;
            capturing = false;
            FG_CUDA(cudaStreamEndCapture(stream, &g));
            cudaGraphExec_t ge;
            FG_CUDA(cudaGraphInstantiate(&ge, g, 0));
            cudaGraphDestroy(g);
            trim_graph_cache();
            it = graphs.emplace(key, ge).first;
        } else {
            for (size_t i = 0; i < lists.size(); ++i) lists[i]->parity = parity_before[i];
            for (unsigned int j = 0; j < S; ++j, ++step_count) simulate_parity_flips();
            step_count = first;
        }
        kernels_last_step = kernel_counter;
        FG_CUDA(cudaGraphLaunch(it->second, stream));
        ++graph_launches;
        if (!cuda_config.time_op_label.empty()) replayed.insert(key);
        FG_CUDA(cudaEventRecord(e1, stream));
        step_events.push_back({e0, e1, S});
        for (unsigned int j = 0; j < S; ++j) count_host_step();
        for (size_t i = 0; i < lists.size(); ++i)  // bounds after the block's S steps
            lists[i]->bound = static_cast<uint32_t>(std::min<uint64_t>(after[i], 0xFFFFFFFFu));
        step_count += S - 1;
        record_counts();  // the counts after the block, for later bounds
        ++step_count;
        return S;
    }

    // The parity changes a step makes, replayed on the host for a cached graph.
    void simulate_parity_flips() {
        for (const auto& layer : model->layers)
            for (auto* fd : layer->functions)
                for (auto& f : fns) {
                    if (f.fn != fd) continue;
                    AgentList& l = *f.list;
                    if (f.sort_trigger && l.agent->sort_period != 0 && step_count % l.agent->sort_period == 0) l.parity ^= 1;
                    if (f.fn->condition) l.parity ^= 1;
                    if (f.fn->has_agent_death || (f.births && f.births_fused)) l.parity ^= 1;
                }
    }

    // The error record and every workspace's status word, read with one batch
    // of async copies into pinned memory and one wait (check_errors), or as
    // part of a caller's batch (enqueue_status_reads, its wait, raise_status).
    void resolve_step_timers();  // step_events -> step_ms (their steps have completed)
    using StatusList = std::vector<std::pair<void*, std::string>>;
    // the workspaces whose status word a read checks
    StatusList status_sources() const {
        StatusList ws;
        for (auto& m : msgs)
            if (m->build_ws) ws.emplace_back(m->build_ws, format("Message '%s' index build", m->msg->name.c_str()));
        for (auto& l : lists)
            if (l->comp_ws) ws.emplace_back(l->comp_ws, format("Compaction of agent '%s'", l->agent->name.c_str()));
        return ws;
    }
    StatusList enqueue_status_reads() {
        uint32_t* hp = h_pinned + 64;
        const uint32_t cap = 1024 - 64;
        FG_CUDA(cudaMemcpyAsync(hp, d_error(), 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
        const StatusList ws = status_sources();
        for (size_t k = 0; k < ws.size() && 4 + k < cap; ++k)
            FG_CUDA(cudaMemcpyAsync(hp + 4 + k, ws[k].first, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
        return ws;
    }
    void check_errors() {
        const StatusList ws = enqueue_status_reads();
        FG_CUDA(cudaStreamSynchronize(stream));
        raise_status(ws);
    }
    void raise_status(const StatusList& ws) {
        uint32_t* hp = h_pinned + 64;
        const uint32_t cap = 1024 - 64;
        uint32_t err[4] = {hp[0], hp[1], hp[2], hp[3]};
        for (size_t k = 0; k < ws.size() && 4 + k < cap; ++k) {
            const int st = static_cast<int>(static_cast<int32_t>(hp[4 + k]));
            if (st != FG_OK) {
                FG_CUDA(cudaMemsetAsync(ws[k].first, 0, sizeof(uint32_t), stream));
                FG_CUDA(cudaStreamSynchronize(stream));
                THROW exception::DeviceError(format("%s reported status %d", ws[k].second.c_str(), st));
            }
        }
        if (err[0] != 0) {
            FG_CUDA(cudaMemset(d_error(), 0, sizeof(err)));
            static const char* names[] = {"ok", "unknown variable name", "variable type mismatch", "array index out of bounds",
                                          "wrapped iterator location outside the environment bounds",
                                          "spatial radius is not a factor of the environment width (wrapped iterator)",
                                          "agent death is not enabled for this function",
                                          "agent output is not enabled for this function", "reserved variable name",
                                          "unsupported device call", "message output is not enabled for this function",
                                          "a neighbourhood staging wait gave up (bounded wait)",
                                          "AgentRandom::uniform() with min > max",
                                          "array message index or search radius out of range, or two messages output to one index",
                                          "bucket message key outside the bounds",
                                          "environment macro property both read and updated in one agent function"};
            if (err[0] == kDevArrayMessage && err[1] == kArrayWriteConflict)
                THROW exception::ArrayMessageWriteConflict(format(
                    "Two array messages were output to one index, or one outside the array (message row %u, %u occurrences)",
                    err[2], err[3]));
            const char* what = err[0] < sizeof(names) / sizeof(names[0]) ? names[err[0]] : "device error";
            THROW exception::DeviceError(format("Device error: %s (name hash 0x%08x, agent index %u, %u occurrences)", what,
                                                err[1], err[2], err[3]));
        }
    }
};

}  // namespace detail

using detail::SimulationImpl;
using exception::format;

// ------------------------------------------------------------------ HostAPI

void HostAPI::Environment::get(const std::string& name, const std::type_info& t, size_t size, void* out) const {
    for (size_t i = 0; i < sim->model->environment.size(); ++i) {
        const auto& p = sim->model->environment[i];
        if (p.name != name) continue;
        if (p.type != std::type_index(t) || p.type_size != size)
            THROW exception::InvalidEnvPropertyType(format("Environment property '%s' has another type", name.c_str()));
        std::memcpy(out, sim->env_host.data() + sim->env_offset[i], size);
        return;
    }
    THROW exception::InvalidEnvProperty(format("Environment has no property '%s'", name.c_str()));
}

void HostAPI::Environment::set(const std::string& name, const std::type_info& t, size_t size, const void* in) {
    for (size_t i = 0; i < sim->model->environment.size(); ++i) {
        const auto& p = sim->model->environment[i];
        if (p.name != name) continue;
        if (p.type != std::type_index(t) || p.type_size != size)
            THROW exception::InvalidEnvPropertyType(format("Environment property '%s' has another type", name.c_str()));
        if (p.is_const) THROW exception::ReservedName(format("Environment property '%s' is constant", name.c_str()));
        std::memcpy(sim->env_host.data() + sim->env_offset[i], in, size);
        sim->env_dirty = true;
        return;
    }
    THROW exception::InvalidEnvProperty(format("Environment has no property '%s'", name.c_str()));
}

void HostAPI::Environment::element(const std::string& name, const std::type_info& t, size_t size,
                                    flamegpu::size_type n, flamegpu::size_type index, void* out, const void* in) const {
    for (size_t i = 0; i < sim->model->environment.size(); ++i) {
        const auto& p = sim->model->environment[i];
        if (p.name != name) continue;
        if (p.type != std::type_index(t) || p.type_size != size)
            THROW exception::InvalidEnvPropertyType(format("Environment property '%s' has another type", name.c_str()));
        if (n != 0 && n != p.elements)
            THROW exception::OutOfBoundsException(format("Environment property '%s' has %u elements, not %u", name.c_str(),
                                                         p.elements, static_cast<unsigned>(n)));
        if (index >= p.elements)
            THROW exception::OutOfBoundsException(format("Index %u is past the %u elements of environment property '%s'",
                                                         static_cast<unsigned>(index), p.elements, name.c_str()));
        char* at = sim->env_host.data() + sim->env_offset[i] + static_cast<size_t>(index) * size;
        std::memcpy(out, at, size);
        if (in) {
            if (p.is_const) THROW exception::ReservedName(format("Environment property '%s' is constant", name.c_str()));
            std::memcpy(at, in, size);
            sim->env_dirty = true;
        }
        return;
    }
    THROW exception::InvalidEnvProperty(format("Environment has no property '%s'", name.c_str()));
}

size_t HostAPI::Environment::elements(const std::string& name) const {
    for (const auto& p : sim->model->environment)
        if (p.name == name) return p.elements;
    THROW exception::InvalidEnvProperty(format("Environment has no property '%s'", name.c_str()));
}

detail::HostMacroData::~HostMacroData() {
    if (!dirty || !device) return;
    // a destructor does not throw: a failed copy is left to the next checked call
    if (cudaStreamSynchronize(stream) == cudaSuccess)
        cudaMemcpy(device, host.data(), host.size(), cudaMemcpyHostToDevice);
}

std::shared_ptr<detail::HostMacroData> HostAPI::Environment::macro(const std::string& name, const std::type_info& t, size_t size,
                                                           const uint32_t (&dims)[4]) const {
    const auto& props = sim->model->macro_environment;
    for (size_t i = 0; i < props.size(); ++i) {
        const detail::MacroProperty& p = props[i];
        if (p.name != name) continue;
        if (p.type != std::type_index(t) || p.type_size != size)
            THROW exception::InvalidEnvPropertyType(format("Environment macro property '%s' has another type", name.c_str()));
        for (int a = 0; a < 4; ++a)
            if (p.dims[a] != dims[a])
                THROW exception::InvalidEnvPropertyType(format(
                    "Environment macro property '%s' has dimensions %u x %u x %u x %u, not %u x %u x %u x %u", name.c_str(),
                    p.dims[0], p.dims[1], p.dims[2], p.dims[3], dims[0], dims[1], dims[2], dims[3]));
        if (auto live = sim->macro_views[name].lock()) return live;
        auto d = std::make_shared<detail::HostMacroData>();
        d->device = sim->d_env + sim->macro_offset[i];
        d->stream = sim->stream;
        d->host.resize(static_cast<size_t>(p.type_size) * p.elements());
        FG_CUDA(cudaStreamSynchronize(sim->stream));
        FG_CUDA(cudaMemcpy(d->host.data(), d->device, d->host.size(), cudaMemcpyDeviceToHost));
        sim->macro_views[name] = d;
        return d;
    }
    THROW exception::InvalidEnvProperty(format("Environment has no macro property '%s'", name.c_str()));
}

std::mt19937_64& HostAPI::Random::engine() const { return sim->host_rng; }
void HostAPI::Random::setSeed(uint64_t seed) {
    sim->host_rng_seed = seed;
    sim->host_rng.seed(seed);
}
uint64_t HostAPI::Random::getSeed() const { return sim->host_rng_seed; }

void HostAPI::Environment::setRaw(const std::string& name, const void* in, size_t size) {
    for (size_t i = 0; i < sim->model->environment.size(); ++i) {
        const auto& p = sim->model->environment[i];
        if (p.name != name) continue;
        if (p.value.size() != size) THROW exception::InvalidEnvPropertyType(format("Environment property '%s' has another size", name.c_str()));
        std::memcpy(sim->env_host.data() + sim->env_offset[i], in, size);
        sim->env_dirty = true;
        return;
    }
    THROW exception::InvalidEnvProperty(format("Environment has no property '%s'", name.c_str()));
}

unsigned int HostAPI::AgentAPI::count() const {
    detail::AgentList* l = sim->list_of(agent, state);
    sim->sync_host_view(agent, state);
    uint32_t c = 0;
    FG_CUDA(cudaStreamSynchronize(sim->stream));
    FG_CUDA(cudaMemcpy(&c, l->d_count, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    return c;
}

HostNewAgentAPI HostAPI::AgentAPI::newAgent() {
    detail::AgentList* l = sim->list_of(agent, state);
    auto& buf = sim->host_births[{agent, state}];
    if (!buf) buf = std::make_unique<AgentVector>(AgentDescription(sim->model, const_cast<detail::AgentData*>(l->agent)));
    buf->push_back();
    return HostNewAgentAPI(buf.get(), buf->size() - 1);
}

AgentVector& HostAPI::AgentAPI::getPopulationData() {
    detail::AgentList* l = sim->list_of(agent, state);
    auto& v = sim->host_views[{agent, state}];
    if (!v) {
        v = std::make_unique<AgentVector>(AgentDescription(sim->model, const_cast<detail::AgentData*>(l->agent)));
        sim->owner->getPopulationData(*v, state);
    }
    return *v;
}

const void* HostAPI::AgentAPI::device_column(const std::string& variable, const std::type_info& t, const uint32_t** d_n,
                                             cudaStream_t* stream) const {
    // the checks of HostAgentAPI::sum (HostAgentAPI.cuh:536-546)
    const detail::AgentList* l = sim->list_of(agent, state);
    sim->sync_host_view(agent, state);
    const int v = l->var_index(variable);
    if (v < 0)
        THROW exception::InvalidAgentVar(format("Agent '%s' has no variable '%s'", agent.c_str(), variable.c_str()));
    const auto& var = l->agent->variables[v];
    if (var.elements != 1)
        THROW exception::UnsupportedVarType(format("Reductions do not support agent array variables ('%s')", variable.c_str()));
    if (var.type != std::type_index(t))
        THROW exception::InvalidVarType(format("Wrong variable type for the reduction of '%s'", variable.c_str()));
    *d_n = l->d_count;
    *stream = sim->stream;
    return l->cols[v][l->parity];
}

void HostAPI::AgentAPI::sort_by(const std::string& variable, const std::type_info& t, uint32_t kind, uint32_t bytes,
                                bool descending, int begin_bit, int end_bit) {
    const uint32_t* d_n = nullptr;
    cudaStream_t st = nullptr;
    device_column(variable, t, &d_n, &st);  // the checks
    if (begin_bit < 0 || end_bit > static_cast<int>(8 * bytes) || begin_bit >= end_bit)
        THROW exception::InvalidArgument(format("HostAgentAPI::sort: bits [%d, %d) are not within the variable's %u bits",
                                                begin_bit, end_bit, 8 * bytes));
    detail::AgentList* l = sim->list_of(agent, state);
    FG_CUDA(cudaStreamSynchronize(st));
    uint32_t n = 0;
    FG_CUDA(cudaMemcpy(&n, l->d_count, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    if (n < 2) return;
    const uint32_t ntiles = (n + detail::kSortTile - 1) / detail::kSortTile;
    const uint32_t ncount = 256u * ntiles;
    const size_t scan_ws = fg_scan_workspace_size(ncount);
    // scratch: two key and two row buffers, the digit counts and starts, the scan's workspace (256-byte aligned)
    const size_t kb = sizeof(uint64_t) * n, rb = sizeof(uint32_t) * n, cb = sizeof(uint32_t) * (ncount + 4u);
    auto align = [](size_t o) { return (o + 255) & ~size_t(255); };
    size_t at[7];
    const size_t sizes[7] = {kb, kb, rb, rb, cb, cb, scan_ws};
    size_t total = 0;
    for (int r = 0; r < 7; ++r) {
        at[r] = total;
        total = align(total + sizes[r]);
    }
    char* scratch = nullptr;
    FG_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&scratch), total, st));
    uint64_t* keys[2] = {reinterpret_cast<uint64_t*>(scratch + at[0]), reinterpret_cast<uint64_t*>(scratch + at[1])};
    uint32_t* rows[2] = {reinterpret_cast<uint32_t*>(scratch + at[2]), reinterpret_cast<uint32_t*>(scratch + at[3])};
    uint32_t* counts = reinterpret_cast<uint32_t*>(scratch + at[4]);
    uint32_t* starts = reinterpret_cast<uint32_t*>(scratch + at[5]);
    void* ws = scratch + at[6];
    try {
        FG_CUDA(cudaMemsetAsync(ws, 0, scan_ws, st));
        const int v = l->var_index(variable);
        const unsigned int grid = std::min((n + 255u) / 256u, static_cast<unsigned int>(sim->sms) * 8u);
        const uint32_t bits = static_cast<uint32_t>(end_bit - begin_bit);
        FG_CUDA(detail::launch_kernel(false, detail::k_hsort_keys, grid, 256, 0, st,
                              static_cast<const char*>(l->cols[v][l->parity]), kind, bytes, descending ? 1u : 0u,
                              static_cast<uint32_t>(begin_bit), bits, n, keys[0], rows[0]));
        int cur = 0;
        for (uint32_t shift = 0; shift < bits; shift += 8, cur ^= 1) {
            FG_CUDA(detail::launch_kernel(false, detail::k_hsort_counts, ntiles, 256, 0, st, static_cast<const uint64_t*>(keys[cur]),
                                  n, shift, ntiles, counts));
            const int rc = fg_exclusive_scan_u32(counts, starts, ncount, ws, scan_ws, st);
            if (rc != FG_OK)
                THROW exception::CUDAError(format("HostAgentAPI::sort: the digit scan failed (%d, %s)", rc,
                                                  cudaGetErrorString(static_cast<cudaError_t>(fg_last_cuda_error()))));
            FG_CUDA(detail::launch_kernel(false, detail::k_hsort_scatter, ntiles, 256, 0, st, static_cast<const uint64_t*>(keys[cur]),
                                  static_cast<const uint32_t*>(rows[cur]), keys[cur ^ 1], rows[cur ^ 1], n, shift, ntiles,
                                  static_cast<const uint32_t*>(starts)));
        }
        // every column in sorted order into the other buffer of the list
        for (size_t c = 0; c < l->cols.size(); ++c)
            FG_CUDA(detail::launch_kernel(false, detail::k_hsort_gather, grid, 256, 0, st, static_cast<const char*>(l->cols[c][l->parity]),
                                  static_cast<char*>(l->cols[c][l->parity ^ 1]), l->agent->variables[c].bytes(),
                                  static_cast<const uint32_t*>(rows[cur]), n));
        l->parity ^= 1;
        FG_CUDA(cudaFreeAsync(scratch, st));
        FG_CUDA(cudaStreamSynchronize(st));
        sim->refresh_host_view(agent, state);
    } catch (...) {
        cudaFreeAsync(scratch, st);
        throw;
    }
}

LogValue HostAPI::AgentAPI::reduce_log(const std::string& variable, const std::type_info& t,
                                       LoggingConfig::Reduction r) const {
    const uint32_t* d_n = nullptr;
    cudaStream_t st = nullptr;
    device_column(variable, t, &d_n, &st);  // the checks
    return sim->owner->reduceAgentVariable(agent, variable, r, state);
}

unsigned int HostAPI::getStepCounter() const { return sim->step_count; }

// ------------------------------------------------------------ CUDASimulation

CUDASimulation::CUDASimulation(const ModelDescription& model, int, const char**)
    : impl(std::make_unique<SimulationImpl>(model.getData())) {
    impl->owner = this;
    impl->init();
}

CUDASimulation::~CUDASimulation() {
    if (log_scratch) {
        cudaStreamSynchronize(impl->stream);
        cudaFree(log_scratch);
    }
}

const std::shared_ptr<detail::ModelData>& CUDASimulation::getModelData() const { return impl->model; }

void CUDASimulation::getEnvironmentRaw(const std::string& name, void* out, size_t bytes) {
    for (size_t i = 0; i < impl->model->environment.size(); ++i) {
        const auto& p = impl->model->environment[i];
        if (p.name != name) continue;
        if (p.value.size() != bytes) THROW exception::InvalidEnvPropertyType(format("Environment property '%s' has another size", name.c_str()));
        std::memcpy(out, impl->env_host.data() + impl->env_offset[i], bytes);
        return;
    }
    THROW exception::InvalidEnvProperty(format("Environment has no property '%s'", name.c_str()));
}

CUDASimulation::SimConfig& CUDASimulation::SimulationConfig() { return impl->config; }
CUDASimulation::Config& CUDASimulation::CUDAConfig() { return impl->cuda_config; }
void CUDASimulation::applyConfig() {
    impl->invalidate();
    // RandomManager::reseed: the host draws follow the simulation's seed (a
    // reapplied configuration with the same seed keeps the sequence going)
    if (!impl->host_rng_applied || impl->host_rng_applied_seed != impl->config.random_seed) {
        impl->host_rng_applied = true;
        impl->host_rng_applied_seed = impl->config.random_seed;
        impl->host_rng_seed = impl->config.random_seed;
        impl->host_rng.seed(impl->config.random_seed);
    }
    if (!impl->config.input_file.empty()) loadState(impl->config.input_file);
}

// ------------------------------------------------------------ state files

namespace {

// One element of a column, as JSON number text (floats with enough digits to
// read back the same value).
std::string number_text(std::type_index t, const char* p) {
    char buf[64];
    // JSON has no NaN or infinity: they are written as null, as the reference's
    // writer (nlohmann::json) does, and read back as NaN
    if (t == std::type_index(typeid(float)) && !std::isfinite(*reinterpret_cast<const float*>(p))) return "null";
    if (t == std::type_index(typeid(double)) && !std::isfinite(*reinterpret_cast<const double*>(p))) return "null";
    if (t == std::type_index(typeid(float))) std::snprintf(buf, sizeof(buf), "%.9g", static_cast<double>(*reinterpret_cast<const float*>(p)));
    else if (t == std::type_index(typeid(double))) std::snprintf(buf, sizeof(buf), "%.17g", *reinterpret_cast<const double*>(p));
    else if (t == std::type_index(typeid(int64_t))) std::snprintf(buf, sizeof(buf), "%lld", static_cast<long long>(*reinterpret_cast<const int64_t*>(p)));
    else if (t == std::type_index(typeid(uint64_t))) std::snprintf(buf, sizeof(buf), "%llu", static_cast<unsigned long long>(*reinterpret_cast<const uint64_t*>(p)));
    else if (t == std::type_index(typeid(int32_t))) std::snprintf(buf, sizeof(buf), "%d", *reinterpret_cast<const int32_t*>(p));
    else if (t == std::type_index(typeid(uint32_t))) std::snprintf(buf, sizeof(buf), "%u", *reinterpret_cast<const uint32_t*>(p));
    else if (t == std::type_index(typeid(int16_t))) std::snprintf(buf, sizeof(buf), "%d", *reinterpret_cast<const int16_t*>(p));
    else if (t == std::type_index(typeid(uint16_t))) std::snprintf(buf, sizeof(buf), "%u", *reinterpret_cast<const uint16_t*>(p));
    else if (t == std::type_index(typeid(int8_t))) std::snprintf(buf, sizeof(buf), "%d", *reinterpret_cast<const int8_t*>(p));
    else if (t == std::type_index(typeid(uint8_t))) std::snprintf(buf, sizeof(buf), "%u", *reinterpret_cast<const uint8_t*>(p));
    else THROW exception::InvalidArgument("State files: unsupported variable type");
    return buf;
}

void number_value(std::type_index t, const detail::json::Value& v, char* p) {
    if (v.kind == detail::json::Value::Null && t == std::type_index(typeid(float))) {
        *reinterpret_cast<float*>(p) = std::numeric_limits<float>::quiet_NaN();
        return;
    }
    if (v.kind == detail::json::Value::Null && t == std::type_index(typeid(double))) {
        *reinterpret_cast<double*>(p) = std::numeric_limits<double>::quiet_NaN();
        return;
    }
    if (v.kind != detail::json::Value::Number) THROW exception::JSONError("State file: a number was expected");
    if (t == std::type_index(typeid(float))) *reinterpret_cast<float*>(p) = std::strtof(v.text.c_str(), nullptr);
    else if (t == std::type_index(typeid(double))) *reinterpret_cast<double*>(p) = v.number();
    else if (t == std::type_index(typeid(int64_t))) *reinterpret_cast<int64_t*>(p) = v.integer();
    else if (t == std::type_index(typeid(uint64_t))) *reinterpret_cast<uint64_t*>(p) = v.uinteger();
    else if (t == std::type_index(typeid(int32_t))) *reinterpret_cast<int32_t*>(p) = static_cast<int32_t>(v.integer());
    else if (t == std::type_index(typeid(uint32_t))) *reinterpret_cast<uint32_t*>(p) = static_cast<uint32_t>(v.uinteger());
    else if (t == std::type_index(typeid(int16_t))) *reinterpret_cast<int16_t*>(p) = static_cast<int16_t>(v.integer());
    else if (t == std::type_index(typeid(uint16_t))) *reinterpret_cast<uint16_t*>(p) = static_cast<uint16_t>(v.uinteger());
    else if (t == std::type_index(typeid(int8_t))) *reinterpret_cast<int8_t*>(p) = static_cast<int8_t>(v.integer());
    else if (t == std::type_index(typeid(uint8_t))) *reinterpret_cast<uint8_t*>(p) = static_cast<uint8_t>(v.uinteger());
    else THROW exception::JSONError("State files: unsupported variable type");
}

// a scalar, or an array of `elements` values
void write_elements(detail::json::Writer& w, std::type_index t, uint32_t size, uint32_t elements, const char* p) {
    if (elements == 1) {
        w.raw(number_text(t, p));
        return;
    }
    w.begin_array();
    for (uint32_t e = 0; e < elements; ++e) w.raw(number_text(t, p + static_cast<size_t>(e) * size));
    w.end_array();
}

void read_elements(const detail::json::Value& v, std::type_index t, uint32_t size, uint32_t elements, char* p,
                   const std::string& what) {
    if (elements == 1) {
        number_value(t, v, p);
        return;
    }
    if (v.kind != detail::json::Value::Array || v.items.size() != elements)
        THROW exception::JSONError(format("State file: '%s' should be an array of %u values", what.c_str(), elements));
    for (uint32_t e = 0; e < elements; ++e) number_value(t, v.items[e], p + static_cast<size_t>(e) * size);
}

}  // namespace

void CUDASimulation::exportData(const std::string& path) {
    // layout of the reference's JSONStateWriter (src/flamegpu/io/JSONStateWriter.cu:55-330):
    // config, stats.step_count, environment, agents -> state -> [ {variable: value} ]
    synchronize();
    std::FILE* f = std::fopen(path.c_str(), "w");
    if (!f) THROW exception::InvalidArgument(format("Cannot open '%s' for writing", path.c_str()));
    detail::json::Writer w(f);
    const auto& m = *impl->model;
    w.begin_object();
    w.key("config");
    w.begin_object();
    w.key("simulation");  // the keys and order of JSONStateWriter::writeConfig (:55-77)
    w.begin_object();
    const auto& sc = impl->config;
    w.key("input_file");
    w.string(sc.input_file);
    w.key("step_log_file");
    w.string(sc.step_log_file);
    w.key("exit_log_file");
    w.string(sc.exit_log_file);
    w.key("common_log_file");
    w.string(sc.common_log_file);
    w.key("truncate_log_files");
    w.raw(sc.truncate_log_files ? "true" : "false");
    w.key("random_seed");
    w.raw(std::to_string(sc.random_seed));
    w.key("steps");
    w.raw(std::to_string(sc.steps));
    w.key("verbosity");
    w.raw(std::to_string(sc.verbosity));
    w.key("timing");
    w.raw(sc.timing ? "true" : "false");
    w.end_object();
    w.key("cuda");
    w.begin_object();
    w.key("device_id");
    w.raw(std::to_string(impl->cuda_config.device_id));
    w.key("inLayerConcurrency");
    w.raw(impl->cuda_config.inLayerConcurrency ? "true" : "false");
    w.end_object();
    w.end_object();
    w.key("stats");
    w.begin_object();
    w.key("step_count");
    w.raw(std::to_string(impl->step_count));
    // GB300 extension: each agent type's next id ("next_id:<agent>"), so a run
    // resumed from this file gives births the ids the uninterrupted run would
    // have. Plain numbers: the reference's reader skips the values of "stats"
    // it does not know (JSONStateReader.cu:203-205), but not nested objects.
    {
        std::vector<uint32_t> next(m.agents.size(), 1u);
        FG_CUDA(cudaMemcpy(next.data(), impl->d_next_id(0), sizeof(uint32_t) * next.size(), cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < m.agents.size(); ++i) {
            w.key("next_id:" + m.agents[i]->name);
            w.raw(std::to_string(next[i]));
        }
    }
    w.end_object();
    if (!m.environment.empty()) {
        w.key("environment");
        w.begin_object();
        for (size_t i = 0; i < m.environment.size(); ++i) {
            const auto& p = m.environment[i];
            w.key(p.name);
            write_elements(w, p.type, p.type_size, p.elements, impl->env_host.data() + impl->env_offset[i]);
        }
        w.end_object();
    }
    w.key("agents");
    w.begin_object();
    std::vector<const detail::AgentData*> agents;
    for (const auto& a : m.agents) agents.push_back(a.get());
    std::sort(agents.begin(), agents.end(), [](const detail::AgentData* x, const detail::AgentData* y) { return x->name < y->name; });
    for (const auto* a : agents) {
        w.key(a->name);
        w.begin_object();
        std::vector<size_t> order(a->variables.size());
        for (size_t v = 0; v < order.size(); ++v) order[v] = v;
        std::sort(order.begin(), order.end(), [&](size_t x, size_t y) { return a->variables[x].name < a->variables[y].name; });
        for (const auto& st : a->states) {
            AgentVector pop(AgentDescription(impl->model, const_cast<detail::AgentData*>(a)));
            getPopulationData(pop, st);
            if (pop.size() == 0) continue;
            w.key(st);
            w.begin_array();
            for (uint32_t i = 0; i < pop.size(); ++i) {
                w.begin_object();
                for (size_t v : order) {
                    const auto& var = a->variables[v];
                    w.key(var.name);
                    write_elements(w, var.type, var.type_size, var.elements,
                                   pop.columns()[v].data() + static_cast<size_t>(i) * var.bytes());
                }
                w.end_object();
            }
            w.end_array();
        }
        w.end_object();
    }
    w.end_object();
    w.end_object();
    std::fputc('\n', f);
    if (std::fclose(f) != 0) THROW exception::InvalidArgument(format("Writing '%s' failed", path.c_str()));
}

void CUDASimulation::loadState(const std::string& path) {
    // the reference's JSONStateReader (src/flamegpu/io/JSONStateReader.cu): populations
    // replace the lists they name, environment properties and the step counter are set
    std::FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) THROW exception::InvalidArgument(format("Cannot open '%s'", path.c_str()));
    std::string text;
    char buf[1 << 16];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, got);
    std::fclose(f);
    detail::json::Value doc;
    try {
        doc = detail::json::Parser(text).parse();
    } catch (const std::exception& e) {
        THROW exception::InvalidArgument(format("'%s': %s", path.c_str(), e.what()));
    }
    auto& m = *impl->model;
    if (const auto* cfg = doc.find("config")) {
        // JSONStateReader.cu:385-416: the known simulation and CUDA items are
        // applied (input_file is not followed), any other is an error
        if (const auto* sc = cfg->find("simulation")) {
            auto& c = impl->config;
            for (const auto& kv : sc->fields) {
                const std::string& k = kv.first;
                const auto& v = kv.second;
                if (k == "random_seed") c.random_seed = v.uinteger();
                else if (k == "steps") c.steps = static_cast<unsigned int>(v.uinteger());
                else if (k == "timing") c.timing = v.kind == detail::json::Value::Bool ? v.b : v.integer() != 0;
                else if (k == "truncate_log_files") c.truncate_log_files = v.kind == detail::json::Value::Bool ? v.b : v.integer() != 0;
                else if (k == "verbosity") c.verbosity = static_cast<unsigned int>(v.uinteger());
                else if (k == "step_log_file") c.step_log_file = v.text;
                else if (k == "exit_log_file") c.exit_log_file = v.text;
                else if (k == "common_log_file") c.common_log_file = v.text;
                else if (k == "input_file" || k == "console_mode") continue;
                else THROW exception::JSONError(format("Unexpected simulation config item '%s' in input file '%s'", k.c_str(), path.c_str()));
            }
        }
        if (const auto* cc = cfg->find("cuda")) {
            for (const auto& kv : cc->fields) {
                if (kv.first == "device_id" || kv.first == "inLayerConcurrency") continue;  // kept as configured
                THROW exception::JSONError(format("Unexpected CUDA config item '%s' in input file '%s'", kv.first.c_str(), path.c_str()));
            }
        }
    }
    if (const auto* env = doc.find("environment")) {
        for (const auto& kv : env->fields) {
            for (size_t i = 0; i < m.environment.size(); ++i) {
                const auto& p = m.environment[i];
                if (p.name != kv.first) continue;
                read_elements(kv.second, p.type, p.type_size, p.elements, impl->env_host.data() + impl->env_offset[i], p.name);
                impl->env_dirty = true;
            }
        }
    }
    if (const auto* agents = doc.find("agents")) {
        for (const auto& ak : agents->fields) {
            const detail::AgentData* a = nullptr;
            for (const auto& x : m.agents)
                if (x->name == ak.first) a = x.get();
            if (!a) THROW exception::JSONError(format("State file: the model has no agent '%s'", ak.first.c_str()));
            for (const auto& sk : ak.second.fields) {
                const auto& rows = sk.second.items;
                AgentVector pop(AgentDescription(impl->model, const_cast<detail::AgentData*>(a)),
                                static_cast<flamegpu::size_type>(rows.size()));
                for (size_t i = 0; i < rows.size(); ++i)
                    for (const auto& vk : rows[i].fields) {
                        const size_t v = pop.columnIndex(vk.first);
                        const auto& var = a->variables[v];
                        read_elements(vk.second, var.type, var.type_size, var.elements,
                                      pop.columns()[v].data() + i * var.bytes(), vk.first);
                    }
                setPopulationData(pop, sk.first);
            }
        }
    }
    if (const auto* stats = doc.find("stats")) {
        if (const auto* sc = stats->find("step_count")) {
            FG_CUDA(cudaStreamSynchronize(impl->stream));
            impl->step_count = static_cast<unsigned int>(sc->uinteger());
            const uint32_t v = impl->step_count;
            FG_CUDA(cudaMemcpy(impl->d_step(), &v, sizeof(uint32_t), cudaMemcpyHostToDevice));
        }
        for (const auto& kv : stats->fields)
            for (size_t i = 0; i < m.agents.size(); ++i)
                if (kv.first == "next_id:" + m.agents[i]->name) {
                    uint32_t cur = 1;
                    FG_CUDA(cudaMemcpy(&cur, impl->d_next_id(i), sizeof(uint32_t), cudaMemcpyDeviceToHost));
                    const uint32_t want = std::max(cur, static_cast<uint32_t>(kv.second.uinteger()));
                    FG_CUDA(cudaMemcpy(impl->d_next_id(i), &want, sizeof(uint32_t), cudaMemcpyHostToDevice));
                }
    }
    impl->upload_env_if_dirty();
}
cudaStream_t CUDASimulation::getStream() const { return impl->stream; }
unsigned long long CUDASimulation::getGraphLaunches() const { return impl->graph_launches; }
unsigned int CUDASimulation::getKernelsPerStep() const { return impl->kernels_last_step; }

void CUDASimulation::harvestOperationTimes() { impl->harvest_graph_ops(); }

std::vector<std::tuple<std::string, double, unsigned long long>> CUDASimulation::takeOperationProfile() {
    FG_CUDA(cudaStreamSynchronize(impl->stream));
    impl->resolve_profile();
    std::vector<std::tuple<std::string, double, unsigned long long>> r;
    for (const auto& kv : impl->op_totals) r.emplace_back(kv.first, kv.second.first, kv.second.second);
    impl->op_totals.clear();
    return r;
}

void CUDASimulation::setPopulationData(AgentVector& pop, const std::string& state) {
    detail::AgentList* l = impl->list_of(pop.getAgentName(), state);
    if (l->agent != pop.getAgentData())
        THROW exception::InvalidArgument("AgentVector belongs to another agent description");
    FG_CUDA(cudaStreamSynchronize(impl->stream));
    const uint32_t n = pop.size();
    const size_t ai = impl->agent_index(l->agent);
    // ids: keep set ones, assign fresh ones to unset (CUDAFatAgent.cu:311-319)
    uint32_t dev_next = 1;
    FG_CUDA(cudaMemcpy(&dev_next, impl->d_next_id(ai), sizeof(uint32_t), cudaMemcpyDeviceToHost));
    {
        const size_t idc = pop.columnIndex("_id");
        id_t* ids = reinterpret_cast<id_t*>(pop.columns()[idc].data());
        // CUDAAgent::validateIDCollisions (CUDAAgent.cu:196-245): set ids must be unique
        {
            std::vector<id_t> set_ids;
            set_ids.reserve(n);
            for (uint32_t i = 0; i < n; ++i)
                if (ids[i] != ID_NOT_SET) set_ids.push_back(ids[i]);
            std::sort(set_ids.begin(), set_ids.end());
            unsigned int dup = 0;
            for (size_t i = 1; i < set_ids.size(); ++i) dup += set_ids[i] == set_ids[i - 1] ? 1u : 0u;
            if (dup)
                THROW exception::AgentIDCollision(format("%u agents of type '%s' share an ID with another agent of the same type",
                                                         dup, l->agent->name.c_str()));
        }
        id_t mx = 0;
        for (uint32_t i = 0; i < n; ++i) mx = std::max(mx, ids[i]);
        uint32_t next = std::max<uint32_t>(dev_next, mx + 1);
        for (uint32_t i = 0; i < n; ++i)
            if (ids[i] == ID_NOT_SET) ids[i] = next++;
        FG_CUDA(cudaMemcpy(impl->d_next_id(ai), &next, sizeof(uint32_t), cudaMemcpyHostToDevice));
    }
    const uint32_t cap = impl->initial_capacity(l, n);
    if (cap > l->capacity) impl->ensure_capacity(*l, cap, 0);
    for (size_t v = 0; v < l->cols.size(); ++v) {
        const size_t b = l->agent->variables[v].bytes();
        if (n) FG_CUDA(cudaMemcpy(l->cols[v][l->parity], pop.columns()[v].data(), b * n, cudaMemcpyHostToDevice));
    }
    FG_CUDA(cudaMemcpy(l->d_count, &n, sizeof(uint32_t), cudaMemcpyHostToDevice));
    l->bound = n;
    impl->forget_counts();
    impl->ensure_all_allocated();
}

void CUDASimulation::getPopulationData(AgentVector& pop, const std::string& state) {
    detail::AgentList* l = impl->list_of(pop.getAgentName(), state);
    synchronize();
    uint32_t n = 0;
    FG_CUDA(cudaMemcpy(&n, l->d_count, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    l->bound = n;
    pop.setCountRaw(n);
    for (size_t v = 0; v < l->cols.size(); ++v) {
        const size_t b = l->agent->variables[v].bytes();
        if (n) FG_CUDA(cudaMemcpy(pop.columns()[v].data(), l->cols[v][l->parity], b * n, cudaMemcpyDeviceToHost));
    }
}

void CUDASimulation::setPopulationColumns(const std::string& agent, const std::string& state, uint32_t n,
                                          const std::vector<std::pair<std::string, const void*>>& host_cols) {
    detail::AgentList* l = impl->list_of(agent, state);
    std::vector<const void*> src(l->cols.size(), nullptr);
    for (const auto& c : host_cols) {
        size_t v = 0;
        while (v < l->agent->variables.size() && l->agent->variables[v].name != c.first) ++v;
        if (v == l->agent->variables.size())
            THROW exception::InvalidAgentVar(format("Agent '%s' has no variable '%s'", agent.c_str(), c.first.c_str()));
        src[v] = c.second;
    }
    size_t idc = l->cols.size();
    for (size_t v = 0; v < src.size(); ++v) {
        if (!src[v] && n)
            THROW exception::InvalidArgument(format("setPopulationColumns: variable '%s' not given",
                                                    l->agent->variables[v].name.c_str()));
        if (l->agent->variables[v].name == "_id") idc = v;
    }
    // copies are ordered after the stream's earlier work; only growing the
    // buffers needs the stream idle
    const uint32_t cap = impl->initial_capacity(l, n);
    if (cap > l->capacity) {
        FG_CUDA(cudaStreamSynchronize(impl->stream));
        impl->ensure_capacity(*l, cap, 0);
    }
    // page-locked host columns: one launch copies them all, sets the count and
    // the next id; otherwise one copy per column
    detail::HostXfer x;
    std::memset(&x, 0, sizeof(x));
    x.id_col = -1;
    bool mapped = l->cols.size() <= static_cast<size_t>(detail::kHostXferCols);
    for (size_t v = 0; mapped && v < l->cols.size(); ++v) {
        x.src[v] = static_cast<const char*>(n ? detail::host_mapped(src[v]) : l->cols[v][l->parity]);
        x.dst[v] = static_cast<char*>(l->cols[v][l->parity]);
        x.elem_bytes[v] = l->agent->variables[v].bytes();
        mapped = x.src[v] != nullptr;
    }
    // the ids: checked (every one set) and their largest found by the transfer
    // launch when the id column takes its 16-byte path, else here on the host
    const bool dev_ids = mapped && idc < src.size() && n && impl->h_pinned_dev &&
                         ((reinterpret_cast<uintptr_t>(x.src[idc]) | reinterpret_cast<uintptr_t>(x.dst[idc]) |
                           (static_cast<size_t>(n) * sizeof(id_t))) & 15) == 0;
    id_t mx = 0;
    if (idc < src.size() && n && !dev_ids) {
        // one branch-free pass (it vectorises): the largest id, and whether any is unset
        const id_t* ids = static_cast<const id_t*>(src[idc]);
        uint32_t unset = 0;
        for (uint32_t i = 0; i < n; ++i) {
            unset |= ids[i] == ID_NOT_SET ? 1u : 0u;
            mx = std::max(mx, ids[i]);
        }
        if (unset) THROW exception::InvalidArgument("setPopulationColumns: every _id must be set");
    }
    if (mapped) {
        x.ncols = static_cast<uint32_t>(l->cols.size());
        x.rows = n;
        x.rows_out = l->d_count;
        x.max_target = impl->d_next_id(impl->agent_index(l->agent));
        x.max_value = dev_ids ? 0u : mx + 1;
        if (dev_ids) {
            x.id_col = static_cast<int32_t>(idc);
            impl->h_pinned[4] = 0u;
            x.id_unset = impl->h_pinned_dev + 4;
        }
        // the recount of the agents entering the next step, in the same launch
        detail::StepEnd e{};
        impl->count_targets(e);
        for (uint32_t k = 0; k < e.ncounts; ++k) x.counts[k] = e.counts[k];
        x.ncounts = e.ncounts;
        x.acc = e.acc;
        FG_CUDA(detail::launch_kernel(detail::pdl_enabled(), detail::k_host_xfer, detail::host_xfer_grid(x, impl->sms),
                                      256, 0, impl->stream, x));
    } else {
        for (size_t v = 0; v < l->cols.size(); ++v) {
            const size_t b = l->agent->variables[v].bytes();
            if (n) FG_CUDA(cudaMemcpyAsync(l->cols[v][l->parity], src[v], b * n, cudaMemcpyHostToDevice, impl->stream));
        }
        // next id: the larger of the device's and one past the largest given
        detail::launch_kernel(detail::pdl_enabled(), detail::k_max_u32, 1, 1, 0, impl->stream,
                             impl->d_next_id(impl->agent_index(l->agent)), mx + 1);
        impl->h_pinned[2] = n;
        FG_CUDA(cudaMemcpyAsync(l->d_count, impl->h_pinned + 2, sizeof(uint32_t), cudaMemcpyHostToDevice, impl->stream));
    }
    // the recount (done by the transfer launch, else queued behind the
    // copies) before the one wait (the caller's buffers are free again when
    // this returns)
    l->bound = n;
    impl->forget_counts(mapped);
    FG_CUDA(cudaStreamSynchronize(impl->stream));
    if (dev_ids && impl->h_pinned[4] != 0u) {
        // an unset id: the list is left empty
        FG_CUDA(cudaMemsetAsync(l->d_count, 0, sizeof(uint32_t), impl->stream));
        impl->forget_counts();
        FG_CUDA(cudaStreamSynchronize(impl->stream));
        l->bound = 0;
        THROW exception::InvalidArgument("setPopulationColumns: every _id must be set");
    }
    impl->ensure_all_allocated();
}

uint32_t CUDASimulation::getPopulationColumns(const std::string& agent, const std::string& state,
                                              const std::vector<std::pair<std::string, void*>>& host_out,
                                              uint32_t cap) {
    detail::AgentList* l = impl->list_of(agent, state);
    std::vector<size_t> vi;
    for (const auto& o : host_out) {
        size_t v = 0;
        while (v < l->agent->variables.size() && l->agent->variables[v].name != o.first) ++v;
        if (v == l->agent->variables.size())
            THROW exception::InvalidAgentVar(format("Agent '%s' has no variable '%s'", agent.c_str(), o.first.c_str()));
        vi.push_back(v);
    }
    // one batch and one wait: status words, the count, and the rows up to the
    // host's bound on the count (never below it), as many as the caller has room for
    const uint32_t rows = std::min(std::min(cap, l->bound), l->capacity);
    // page-locked host buffers: one launch copies the rows, the count and the
    // status words; otherwise one copy each
    detail::HostXfer x;
    std::memset(&x, 0, sizeof(x));
    bool mapped = host_out.size() <= static_cast<size_t>(detail::kHostXferCols) && impl->h_pinned_dev;
    for (size_t k = 0; mapped && k < host_out.size(); ++k) {
        x.src[k] = static_cast<const char*>(l->cols[vi[k]][l->parity]);
        x.dst[k] = static_cast<char*>(detail::host_mapped(host_out[k].second));
        x.elem_bytes[k] = l->agent->variables[vi[k]].bytes();
        mapped = x.dst[k] != nullptr;
    }
    detail::SimulationImpl::StatusList ws;
    if (mapped) {
        ws = impl->status_sources();
        mapped = ws.size() + 4 <= static_cast<size_t>(detail::kHostXferWords);
    }
    if (mapped) {
        uint32_t* hp_dev = impl->h_pinned_dev + 64;  // the status words' host slots, as enqueue_status_reads uses
        for (uint32_t k = 0; k < 4; ++k) {
            x.word_src[k] = impl->d_error() + k;
            x.word_dst[k] = hp_dev + k;
        }
        for (size_t k = 0; k < ws.size(); ++k) {
            x.word_src[4 + k] = static_cast<const uint32_t*>(ws[k].first);
            x.word_dst[4 + k] = hp_dev + 4 + k;
        }
        x.nwords = static_cast<uint32_t>(4 + ws.size());
        x.ncols = static_cast<uint32_t>(host_out.size());
        x.rows = rows;
        x.d_rows = l->d_count;
        x.rows_out = impl->h_pinned_dev + 3;
        FG_CUDA(detail::launch_kernel(detail::pdl_enabled(), detail::k_host_xfer, detail::host_xfer_grid(x, impl->sms),
                                      256, 0, impl->stream, x));
    } else {
        ws = impl->enqueue_status_reads();
        FG_CUDA(cudaMemcpyAsync(impl->h_pinned + 3, l->d_count, sizeof(uint32_t), cudaMemcpyDeviceToHost, impl->stream));
        for (size_t k = 0; k < host_out.size(); ++k) {
            const size_t b = l->agent->variables[vi[k]].bytes();
            if (rows)
                FG_CUDA(cudaMemcpyAsync(host_out[k].second, l->cols[vi[k]][l->parity], b * rows, cudaMemcpyDeviceToHost,
                                        impl->stream));
        }
    }
    FG_CUDA(cudaStreamSynchronize(impl->stream));
    impl->raise_status(ws);
    impl->resolve_step_timers();
    const uint32_t n = impl->h_pinned[3];
    l->bound = n;
    if (n > cap) THROW exception::InvalidArgument(format("getPopulationColumns: %u agents, room for %u", n, cap));
    return n;
}

bool CUDASimulation::step() {
    if (impl->step_count == 0 && !impl->model->init_functions.empty()) {
        HostAPI api(impl.get());
        for (auto fn : impl->model->init_functions) fn(&api);
        impl->flush_host_births();
    }
    impl->step_once(this);
    return !impl->exit_requested;
}

void CUDASimulation::step(unsigned int n) {
    if (n == 0) return;
    if (impl->step_count == 0 && !impl->model->init_functions.empty()) {
        HostAPI api(impl.get());
        for (auto fn : impl->model->init_functions) fn(&api);
        impl->flush_host_births();
    }
    if (!impl->multi_step_ok(step_log != nullptr)) {
        for (unsigned int s = 0; s < n; ++s) {
            impl->step_once(this);
            if (impl->exit_requested) break;
        }
        return;
    }
    constexpr unsigned int kBlock = 16;
    while (n) n -= impl->step_block(n < kBlock ? n : kBlock);
}

void CUDASimulation::simulate() {
    impl->ensure_all_allocated();
    cudaEvent_t s0, s1;
    FG_CUDA(cudaEventCreate(&s0));
    FG_CUDA(cudaEventCreate(&s1));
    FG_CUDA(cudaEventRecord(s0, impl->stream));
    if (!impl->model->init_functions.empty()) {
        FG_CUDA(cudaStreamSynchronize(impl->stream));
        HostAPI api(impl.get());
        for (auto fn : impl->model->init_functions) fn(&api);
        impl->flush_host_births();
    }
    processStepLog(0.0);  // the frame before the first step (CUDASimulation.cu:1263)
    if (impl->multi_step_ok(step_log != nullptr)) {
        for (unsigned int n = impl->config.steps; n;) n -= impl->step_block(n < 16u ? n : 16u);
    } else if (impl->config.steps == 0 && !impl->model->exit_conditions.empty()) {
        // steps 0: until an exit condition ends the simulation
        do impl->step_once(this);
        while (!impl->exit_requested);
    } else {
        for (unsigned int s = 0; s < impl->config.steps; ++s) {
            impl->step_once(this);
            if (impl->exit_requested) break;
        }
    }
    if (!impl->model->exit_functions.empty()) {
        FG_CUDA(cudaStreamSynchronize(impl->stream));
        HostAPI api(impl.get());
        for (auto fn : impl->model->exit_functions) fn(&api);
        impl->flush_host_births();
    }
    FG_CUDA(cudaEventRecord(s1, impl->stream));
    synchronize();
    float ms = 0;
    cudaEventElapsedTime(&ms, s0, s1);
    impl->sim_ms = ms;
    processExitLog(ms / 1000.0);
    cudaEventDestroy(s0);
    cudaEventDestroy(s1);
}

unsigned int CUDASimulation::getStepCounter() const { return impl->step_count; }

void CUDASimulation::resetStepCounter() {
    FG_CUDA(cudaStreamSynchronize(impl->stream));
    impl->step_count = 0;
    FG_CUDA(cudaMemset(impl->d_step(), 0, sizeof(uint32_t)));
}

void CUDASimulation::synchronize() {
    impl->check_errors();
    impl->resolve_step_timers();
}

void detail::SimulationImpl::resolve_step_timers() {
    for (auto& e : step_events) {
        float ms = 0;
        cudaEventElapsedTime(&ms, e.e0, e.e1);
        // steps replayed as one graph share its time equally
        for (unsigned int k = 0; k < e.steps; ++k) step_ms.push_back(ms / e.steps);
        cudaEventDestroy(e.e0);
        cudaEventDestroy(e.e1);
    }
    step_events.clear();
}

unsigned long long CUDASimulation::getAgentStepCount() {
    if (!impl->counts_on_device()) return impl->host_agent_steps;
    unsigned long long v = 0;
    FG_CUDA(cudaStreamSynchronize(impl->stream));
    FG_CUDA(cudaMemcpy(&v, impl->d_agent_steps, sizeof(v), cudaMemcpyDeviceToHost));
    return v;
}

double CUDASimulation::getElapsedTimeSimulation() const { return impl->sim_ms / 1000.0; }

std::vector<double> CUDASimulation::getElapsedTimeSteps() const {
    std::vector<double> r;
    for (double ms : impl->step_ms) r.push_back(ms / 1000.0);
    return r;
}

double CUDASimulation::getElapsedTimeStep(unsigned int s) const {
    if (s >= impl->step_ms.size()) THROW exception::OutOfBoundsException(format("Step %u has no timing", s));
    return impl->step_ms[s] / 1000.0;
}

unsigned int CUDASimulation::getAgentCount(const std::string& agent, const std::string& state) {
    HostAPI api(impl.get());
    return api.agent(agent, state).count();
}

void* CUDASimulation::getDeviceVariable(const std::string& agent, const std::string& variable, const std::string& state) {
    detail::AgentList* l = impl->list_of(agent, state);
    const int v = l->var_index(variable);
    if (v < 0) THROW exception::InvalidAgentVar(format("Agent '%s' has no variable '%s'", agent.c_str(), variable.c_str()));
    impl->ensure_all_allocated();
    return l->cols[v][l->parity];
}

void CUDASimulation::setPopulationDevice(const std::string& agent, const std::string& state, unsigned int n,
                                         const std::vector<std::pair<std::string, const void*>>& columns,
                                         id_t next_id) {
    detail::AgentList* l = impl->list_of(agent, state);
    if (columns.size() != l->cols.size())
        THROW exception::InvalidArgument(format("setPopulationDevice needs all %zu variables of agent '%s'", l->cols.size(), agent.c_str()));
    FG_CUDA(cudaStreamSynchronize(impl->stream));
    if (n > l->capacity) impl->ensure_capacity(*l, n, 0);
    impl->ensure_all_allocated();
    for (const auto& c : columns) {
        const int v = l->var_index(c.first);
        if (v < 0) THROW exception::InvalidAgentVar(format("Agent '%s' has no variable '%s'", agent.c_str(), c.first.c_str()));
        const size_t b = l->agent->variables[v].bytes();
        if (n) FG_CUDA(cudaMemcpyAsync(l->cols[v][l->parity], c.second, b * n, cudaMemcpyDeviceToDevice, impl->stream));
    }
    impl->h_pinned[0] = n;
    impl->h_pinned[1] = next_id;
    FG_CUDA(cudaMemcpyAsync(l->d_count, impl->h_pinned, sizeof(uint32_t), cudaMemcpyHostToDevice, impl->stream));
    FG_CUDA(cudaMemcpyAsync(impl->d_next_id(impl->agent_index(l->agent)), impl->h_pinned + 1, sizeof(uint32_t),
                            cudaMemcpyHostToDevice, impl->stream));
    FG_CUDA(cudaStreamSynchronize(impl->stream));
    l->bound = n;
    impl->forget_counts();
}

void CUDASimulation::setSpatialMessageBounds(const std::string& message, const std::vector<float>& mn,
                                             const std::vector<float>& mx, float radius) {
    detail::MsgList* m = impl->msg_of(message);
    if (!m || !m->spatial()) THROW exception::InvalidMessageName(format("No spatial message '%s'", message.c_str()));
    const int dims = m->grid.dims;
    if (static_cast<int>(mn.size()) < dims || static_cast<int>(mx.size()) < dims)
        THROW exception::InvalidArgument("Spatial bounds need one value per dimension");
    FG_CUDA(cudaStreamSynchronize(impl->stream));
    fg_spatial_grid g{};
    if (fg_spatial_grid_init(&g, dims, mn.data(), mx.data(), radius) != FG_OK)
        THROW exception::InvalidArgument(format("Invalid bounds/radius for message '%s'", message.c_str()));
    m->grid = g;
    impl->mem.release(m->pbm);
    m->pbm_alloc = (g.binCount + 1u + 3u) & ~3u;
    m->pbm = static_cast<uint32_t*>(impl->mem.alloc(sizeof(uint32_t) * (static_cast<size_t>(m->pbm_alloc) + 4)));
    if (m->capacity) {
        impl->mem.release(m->build_ws);
        m->build_ws_bytes = fg_spatial_build_workspace_size(m->capacity, g.binCount);
        m->build_ws = impl->mem.alloc(m->build_ws_bytes);
    }
    for (auto& l : impl->lists) {
        auto it = l->sort_ws.find(m);
        if (it != l->sort_ws.end()) {
            impl->mem.release(it->second.first);
            l->sort_ws.erase(it);
        }
    }
    impl->invalidate();
}

const unsigned int* CUDASimulation::getDeviceCount(const std::string& agent, const std::string& state) {
    return impl->list_of(agent, state)->d_count;
}

}  // namespace flamegpu
