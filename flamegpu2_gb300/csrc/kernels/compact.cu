// Fused, order-preserving birth/death compaction (one pass over the agents).
//
// Each block owns a tile of 2048 agents, read "striped" (item k of thread t is
// agent tile*2048 + k*256 + t) so that every flag load and column copy is
// coalesced. Survivor and birth ranks inside the tile come from warp ballots;
// the tile's offsets among all tiles come from a decoupled look-back on a
// packed (survivors, births) pair. Survivors land at their rank, births at
// S + birth rank where S = total survivors, so the reference's order —
// survivors in order, then children in parent order — falls out of one kernel.
// Tile statuses live in two arrays used on alternate calls; every call clears
// the array the next call will use, so nothing is reset from the host.
#include <algorithm>

#include "common.cuh"

namespace fgk {

constexpr int kCompItems = 8;
constexpr uint32_t kCompTile = kThreads * kCompItems;  // 2048
constexpr uint64_t kPairMask = (1ull << 62) - 1ull;

struct CompactParams {
    fg_column col[FG_MAX_COLUMNS];
    fg_column bcol[FG_MAX_COLUMNS];
    uint32_t ncols;
    int32_t id_col;
};

__device__ __forceinline__ uint64_t pair_pack(uint32_t flag, uint32_t a, uint32_t b) {
    return (static_cast<uint64_t>(flag) << 62) | (static_cast<uint64_t>(a) << 31) | static_cast<uint64_t>(b);
}

// Look back over predecessor tiles; returns the exclusive packed (a << 31 | b).
// At most `limit` polls per predecessor (a give-up is recorded in the header).
__device__ __forceinline__ uint64_t lookback_pair(const uint64_t* status, uint32_t tile, WsHeader* h,
                                                  uint32_t limit) {
    const uint32_t lane = lane_id();
    uint64_t excl = 0;
    int64_t pred = static_cast<int64_t>(tile) - 1;
    while (pred >= 0) {
        const int64_t t = pred - lane;
        uint32_t flag = 2;
        uint64_t val = 0;
        if (t >= 0) {
            uint32_t spins = 0;
            for (;;) {
                const uint64_t s = ld_acquire_u64(status + t);
                flag = static_cast<uint32_t>(s >> 62);
                val = s & kPairMask;
                if (flag != 0) break;
                if (++spins > limit) {
                    record_status(h, FG_ERR_DEVICE_TIMEOUT);
                    flag = 2;
                    val = 0;
                    break;
                }
                if (spins > 16) __nanosleep(spins > 1024 ? 256 : 32);
            }
        }
        const uint32_t pmask = __ballot_sync(0xFFFFFFFFu, flag == 2);
        uint64_t contrib;
        if (pmask) {
            const uint32_t k = __ffs(pmask) - 1;
            contrib = lane <= k ? val : 0;
        } else {
            contrib = val;
        }
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) contrib += __shfl_xor_sync(0xFFFFFFFFu, contrib, d);
        excl += contrib;
        if (pmask) break;
        pred -= 32;
    }
    return excl;
}

__device__ __forceinline__ void copy_col(const fg_column& c, uint32_t src, uint32_t dst) {
    switch (c.elem_bytes) {
        case 4: reinterpret_cast<uint32_t*>(c.out)[dst] = reinterpret_cast<const uint32_t*>(c.in)[src]; break;
        case 8: reinterpret_cast<uint2*>(c.out)[dst] = reinterpret_cast<const uint2*>(c.in)[src]; break;
        case 16: reinterpret_cast<uint4*>(c.out)[dst] = reinterpret_cast<const uint4*>(c.in)[src]; break;
        case 1: reinterpret_cast<uint8_t*>(c.out)[dst] = reinterpret_cast<const uint8_t*>(c.in)[src]; break;
        case 2: reinterpret_cast<uint16_t*>(c.out)[dst] = reinterpret_cast<const uint16_t*>(c.in)[src]; break;
        default: {
            const uint8_t* a = reinterpret_cast<const uint8_t*>(c.in) + static_cast<size_t>(src) * c.elem_bytes;
            uint8_t* b = reinterpret_cast<uint8_t*>(c.out) + static_cast<size_t>(dst) * c.elem_bytes;
            for (uint32_t k = 0; k < c.elem_bytes; ++k) b[k] = a[k];
        }
    }
}

__global__ void __launch_bounds__(kThreads) k_count_alive(uint32_t max_n, const uint32_t* d_n,
                                                          const uint32_t* __restrict__ alive, WsHeader* h) {
    flamegpu::detail::grid_dependency_enter();
    const uint32_t n = d_n ? min(*d_n, max_n) : max_n;
    uint32_t c = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        c += alive[i] != 0 ? 1u : 0u;
    c = __reduce_add_sync(0xFFFFFFFFu, c);
    if (lane_id() == 0 && c) atomicAdd(&h->alive_total, c);
}

__global__ void k_set_alive_total(uint32_t max_n, const uint32_t* d_n, WsHeader* h) {
    flamegpu::detail::grid_dependency_enter();
    h->alive_total = d_n ? min(*d_n, max_n) : max_n;
}

// Row i of every column written at dst (cols: the survivors' or the births'
// sources). Runs of four 4-byte columns are all loaded before any is stored,
// so their latencies overlap; the id column of births gets next_id + r.
__device__ __forceinline__ void copy_row(const fg_column* cols, uint32_t ncols, uint32_t i, uint32_t dst, int id_col,
                                         uint32_t id) {
    for (uint32_t c0 = 0; c0 < ncols; c0 += 4) {
        const uint32_t nk = min(4u, ncols - c0);
        bool words = true;
        for (uint32_t k = 0; k < nk; ++k) words = words && cols[c0 + k].elem_bytes == 4u;
        if (words) {
            uint32_t v[4];
#pragma unroll
            for (uint32_t k = 0; k < 4; ++k)
                if (k < nk) v[k] = static_cast<int32_t>(c0 + k) == id_col ? id : reinterpret_cast<const uint32_t*>(cols[c0 + k].in)[i];
#pragma unroll
            for (uint32_t k = 0; k < 4; ++k)
                if (k < nk) reinterpret_cast<uint32_t*>(cols[c0 + k].out)[dst] = v[k];
        } else {
            for (uint32_t k = 0; k < nk; ++k) {
                if (static_cast<int32_t>(c0 + k) == id_col)
                    reinterpret_cast<uint32_t*>(cols[c0 + k].out)[dst] = id;
                else
                    copy_col(cols[c0 + k], i, dst);
            }
        }
    }
}

// Persistent tiles: each block takes tiles of kCompTile rows by ticket (in
// launch order) until the rows [0, n) are covered, so the grid can be a few
// blocks per SM whatever the capacity, and a small population costs a few
// tiles rather than one block per tile of capacity. A tile waits only on
// lower tiles, taken earlier by running blocks that publish their aggregate
// before they look back themselves.
__global__ void __launch_bounds__(kThreads) k_compact(const __grid_constant__ CompactParams cp, uint32_t max_n,
                                                      const uint32_t* d_n, const uint32_t* __restrict__ alive,
                                                      const uint32_t* __restrict__ born, uint32_t* d_next_id,
                                                      const uint32_t* d_alive_total, uint32_t* d_n_out,
                                                      uint32_t out_capacity, uint64_t* status0, uint32_t stride_tiles,
                                                      WsHeader* h, int partition, uint32_t* d_s_out) {
    flamegpu::detail::grid_dependency_enter();
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_cnt_a[kCompItems][kThreads / 32];
    __shared__ uint32_t s_cnt_b[kCompItems][kThreads / 32];
    __shared__ uint32_t s_tot[2];
    __shared__ uint64_t s_excl;
    const uint32_t tid = threadIdx.x, lane = lane_id(), warp = tid >> 5;
    const uint32_t limit = spin_limit_of(h);  // before the acquire load (no extra round trip)
    const bool withhold = h->withhold != 0;
    const uint32_t parity = ld_acquire_u32(&h->comp_parity) & 1u;
    const uint32_t n = d_n ? min(*d_n, max_n) : max_n;
    const uint32_t S = d_alive_total ? *d_alive_total : h->alive_total;
    const uint32_t next_id = d_next_id ? *d_next_id : 0u;
    uint64_t* status = status0 + static_cast<size_t>(parity) * stride_tiles;
    // clear the whole status array the next call will use (its grid may differ)
    uint64_t* other = status0 + static_cast<size_t>(parity ^ 1u) * stride_tiles;
    for (uint32_t t = blockIdx.x * blockDim.x + tid; t < stride_tiles; t += gridDim.x * blockDim.x) other[t] = 0;
    for (;;) {
        if (tid == 0) s_tile = atomicAdd(&h->comp_ticket, 1u);
        __syncthreads();
        const uint32_t tile = s_tile;
        const uint32_t base = tile * kCompTile;
        if (base >= n) break;  // the same in every thread: no rows left
        uint32_t ba[kCompItems], bb[kCompItems];
#pragma unroll
        for (int k = 0; k < kCompItems; ++k) {
            const uint32_t i = base + k * kThreads + tid;
            const bool in = i < n;
            // partition 2 (births only): no row is a survivor
            const bool a = in && partition != 2 && (alive == nullptr || alive[i] != 0);
            // partition 1: every row not in the first group goes, in order, to the second
            const bool b = in && (partition == 1 ? !a : (born != nullptr && born[i] != 0));
            ba[k] = __ballot_sync(0xFFFFFFFFu, a);
            bb[k] = __ballot_sync(0xFFFFFFFFu, b);
            if (lane == 0) {
                s_cnt_a[k][warp] = __popc(ba[k]);
                s_cnt_b[k][warp] = __popc(bb[k]);
            }
        }
        __syncthreads();
        if (tid == 0) {
            uint32_t ra = 0, rb = 0;
            for (int k = 0; k < kCompItems; ++k)
                for (int w = 0; w < kThreads / 32; ++w) {
                    const uint32_t a = s_cnt_a[k][w], b = s_cnt_b[k][w];
                    s_cnt_a[k][w] = ra;
                    s_cnt_b[k][w] = rb;
                    ra += a;
                    rb += b;
                }
            s_tot[0] = ra;
            s_tot[1] = rb;
        }
        __syncthreads();
        if (tid < 32) {
            const uint64_t agg = (static_cast<uint64_t>(s_tot[0]) << 31) | s_tot[1];
            uint64_t excl = 0;
            if (tile == 0) {
                if (tid == 0 && !withhold) st_release_u64(status, pair_pack(2, s_tot[0], s_tot[1]));
            } else {
                if (tid == 0) st_release_u64(status + tile, (1ull << 62) | agg);
                excl = lookback_pair(status, tile, h, limit);
                if (tid == 0) st_release_u64(status + tile, (2ull << 62) | ((excl + agg) & kPairMask));
            }
            if (tid == 0) {
                s_excl = excl;
                if (base + kCompTile >= n) {  // last tile with rows: publish the totals
                    const uint64_t inc = excl + agg;
                    h->pad[0] = static_cast<uint32_t>(inc & 0x7FFFFFFFu);          // births
                    h->pad[1] = static_cast<uint32_t>((inc >> 31) & 0x7FFFFFFFu);  // survivors
                }
            }
        }
        __syncthreads();
        const uint32_t ea = static_cast<uint32_t>((s_excl >> 31) & 0x7FFFFFFFu);
        const uint32_t eb = static_cast<uint32_t>(s_excl & 0x7FFFFFFFu);
        const uint32_t lt = lanemask_lt();
#pragma unroll
        for (int k = 0; k < kCompItems; ++k) {
            const uint32_t i = base + k * kThreads + tid;
            if ((ba[k] >> lane) & 1u) {
                const uint32_t dst = ea + s_cnt_a[k][warp] + __popc(ba[k] & lt);
                if (dst < out_capacity) copy_row(cp.col, cp.ncols, i, dst, -1, 0u);
            }
            if ((bb[k] >> lane) & 1u) {
                const uint32_t r = eb + s_cnt_b[k][warp] + __popc(bb[k] & lt);
                const uint32_t dst = S + r;
                // a birth flagged 2 claimed its id during the function: kept
                const bool claimed = partition != 1 && born != nullptr && born[i] == 2u;
                if (dst < out_capacity)
                    copy_row(cp.bcol, cp.ncols, i, dst, claimed ? -1 : cp.id_col, next_id + r);
                else
                    record_status(h, FG_ERR_CAPACITY);
            }
        }
        __syncthreads();  // s_tile, s_cnt_*, s_excl are reused by the next tile
    }
    // the last block to finish publishes the new count and resets the tickets
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        if (atomicAdd(&h->comp_done, 1u) == gridDim.x - 1) {
            const uint32_t births = h->pad[0];
            uint32_t total = S + births;
            if (total > out_capacity) total = out_capacity;
            if (d_n_out) *d_n_out = total;
            if (d_s_out) *d_s_out = S;
            if (d_next_id && cp.id_col >= 0) *d_next_id = next_id + births;
            h->pad[0] = 0;
            h->pad[1] = 0;
            h->alive_total = 0;
            h->comp_ticket = 0;
            h->comp_done = 0;
            atomicExch(&h->comp_parity, parity ^ 1u);
            __threadfence();
        }
    }
}

}  // namespace fgk

using namespace fgk;

namespace {
int launch_err() {
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FG_OK : FG_ERR_CUDA;
}
uint32_t comp_tiles(uint32_t max_n) { return std::max(1u, (max_n + kCompTile - 1) / kCompTile); }
uint32_t device_sms() {
    int dev = 0, sms = 132;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return static_cast<uint32_t>(sms);
}
// persistent compaction blocks: four per SM, or one per tile of capacity if fewer
uint32_t comp_grid(uint32_t max_n) { return std::min(comp_tiles(max_n), 4u * device_sms()); }
// survivor-count blocks (grid-stride over the flags): four per SM at most
uint32_t count_grid(uint32_t max_n) {
    return std::max(1u, std::min((max_n + kThreads - 1) / kThreads, 4u * device_sms()));
}
}  // namespace

uint32_t* fgi_compact_survivor_word(void* workspace) {
    return workspace ? &reinterpret_cast<WsHeader*>(workspace)->alive_total : nullptr;
}

extern "C" size_t fg_compact_workspace_size(uint32_t max_n) {
    return sizeof(WsHeader) + align_up(sizeof(uint64_t) * 2 * comp_tiles(max_n), 256);
}

extern "C" int fg_compact_agents(uint32_t max_n, const uint32_t* d_n, const uint32_t* alive, const uint32_t* born,
                                 const fg_column* cols, const fg_column* birth_cols, uint32_t ncols, int32_t id_col,
                                 uint32_t* d_next_id, const uint32_t* d_alive_total, uint32_t* d_n_out,
                                 uint32_t out_capacity, void* workspace, size_t workspace_bytes, void* stream) {
    if (!workspace || ncols > FG_MAX_COLUMNS || (ncols && !cols)) return FG_ERR_INVALID_ARGUMENT;
    if (born && ncols && !birth_cols) return FG_ERR_INVALID_ARGUMENT;
    if (id_col >= static_cast<int32_t>(ncols)) return FG_ERR_INVALID_ARGUMENT;
    if (id_col >= 0 && cols[id_col].elem_bytes != 4) return FG_ERR_INVALID_ARGUMENT;
    if (max_n >= (1u << 31)) return FG_ERR_UNSUPPORTED;
    if (workspace_bytes < fg_compact_workspace_size(max_n) || (reinterpret_cast<uintptr_t>(workspace) & 255))
        return FG_ERR_WORKSPACE;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    char* ws = static_cast<char*>(workspace);
    WsHeader* h = reinterpret_cast<WsHeader*>(ws);
    uint64_t* status = reinterpret_cast<uint64_t*>(ws + sizeof(WsHeader));
    const uint32_t tiles = comp_grid(max_n);
    // h->alive_total is zero here: the workspace starts zeroed
    // (fg_workspace_init) and each compaction's last block resets it
    if (!d_alive_total && alive) {
        launch(k_count_alive, count_grid(max_n), kThreads, st, max_n, d_n, alive, h);
    } else if (!d_alive_total) {
        // every agent survives: S = n
        launch(k_set_alive_total, 1, 1, st, max_n, d_n, h);
    }
    CompactParams cp{};
    for (uint32_t c = 0; c < ncols; ++c) {
        cp.col[c] = cols[c];
        cp.bcol[c] = birth_cols ? birth_cols[c] : cols[c];
    }
    cp.ncols = ncols;
    cp.id_col = id_col;
    // both status arrays are strided by the workspace's tile capacity, so a
    // workspace keeps working when max_n changes between calls
    const uint32_t stride_tiles = static_cast<uint32_t>((workspace_bytes - sizeof(WsHeader)) / (2 * sizeof(uint64_t)));
    launch(k_compact, tiles, kThreads, st, cp, max_n, d_n, alive, born, d_next_id, d_alive_total, d_n_out, out_capacity,
           status, stride_tiles, h, 0, nullptr);
    return launch_err();
}

extern "C" int fg_partition_agents(uint32_t max_n, const uint32_t* d_n, const uint32_t* first_group,
                                   const fg_column* cols, uint32_t ncols, uint32_t* d_first_count,
                                   void* workspace, size_t workspace_bytes, void* stream) {
    if (!workspace || !first_group || ncols > FG_MAX_COLUMNS || (ncols && !cols)) return FG_ERR_INVALID_ARGUMENT;
    if (max_n >= (1u << 31)) return FG_ERR_UNSUPPORTED;
    if (workspace_bytes < fg_compact_workspace_size(max_n) || (reinterpret_cast<uintptr_t>(workspace) & 255))
        return FG_ERR_WORKSPACE;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    char* ws = static_cast<char*>(workspace);
    WsHeader* h = reinterpret_cast<WsHeader*>(ws);
    uint64_t* status = reinterpret_cast<uint64_t*>(ws + sizeof(WsHeader));
    // the first group is the compaction's "survivors" (counted first, so the
    // second group knows where it starts), the rest its "births" in row order;
    // h->alive_total is zero here (see fg_compact_agents)
    launch(k_count_alive, count_grid(max_n), kThreads, st, max_n, d_n, first_group, h);
    CompactParams cp{};
    for (uint32_t c = 0; c < ncols; ++c) cp.col[c] = cp.bcol[c] = cols[c];
    cp.ncols = ncols;
    cp.id_col = -1;
    const uint32_t stride_tiles = static_cast<uint32_t>((workspace_bytes - sizeof(WsHeader)) / (2 * sizeof(uint64_t)));
    launch(k_compact, comp_grid(max_n), kThreads, st, cp, max_n, d_n, first_group, nullptr, nullptr, nullptr, nullptr,
           max_n, status, stride_tiles, h, 1, d_first_count);
    return launch_err();
}

extern "C" int fg_append_births(uint32_t max_n, const uint32_t* d_n, const uint32_t* born, const fg_column* cols,
                                uint32_t ncols, int32_t id_col, uint32_t* d_next_id, uint32_t* d_dst_count,
                                uint32_t dst_capacity, void* workspace, size_t workspace_bytes, void* stream) {
    if (!workspace || !born || !d_dst_count || ncols > FG_MAX_COLUMNS || (ncols && !cols))
        return FG_ERR_INVALID_ARGUMENT;
    if (id_col >= static_cast<int32_t>(ncols)) return FG_ERR_INVALID_ARGUMENT;
    if (id_col >= 0 && (cols[id_col].elem_bytes != 4 || !d_next_id)) return FG_ERR_INVALID_ARGUMENT;
    if (max_n >= (1u << 31)) return FG_ERR_UNSUPPORTED;
    if (workspace_bytes < fg_compact_workspace_size(max_n) || (reinterpret_cast<uintptr_t>(workspace) & 255))
        return FG_ERR_WORKSPACE;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    char* ws = static_cast<char*>(workspace);
    WsHeader* h = reinterpret_cast<WsHeader*>(ws);
    uint64_t* status = reinterpret_cast<uint64_t*>(ws + sizeof(WsHeader));
    // births-only compaction: no survivors, "S" = the destination's count, so
    // birth r lands at *d_dst_count + r and the count grows by the births
    CompactParams cp{};
    for (uint32_t c = 0; c < ncols; ++c) cp.col[c] = cp.bcol[c] = cols[c];
    cp.ncols = ncols;
    cp.id_col = id_col;
    const uint32_t stride_tiles = static_cast<uint32_t>((workspace_bytes - sizeof(WsHeader)) / (2 * sizeof(uint64_t)));
    launch(k_compact, comp_grid(max_n), kThreads, st, cp, max_n, d_n, nullptr, born, id_col >= 0 ? d_next_id : nullptr,
           static_cast<const uint32_t*>(d_dst_count), d_dst_count, dst_capacity, status, stride_tiles, h, 2,
           nullptr);
    return launch_err();
}

namespace fgk {

// rows [begin, end) of the source columns -> rows [dst0, dst0 + end - begin) of the destination
__global__ void __launch_bounds__(kThreads) k_append_rows(const __grid_constant__ CompactParams cp, uint32_t max_rows,
                                                          const uint32_t* d_begin, const uint32_t* d_end,
                                                          const uint32_t* d_dst_count, uint32_t dst_capacity,
                                                          WsHeader* h) {
    flamegpu::detail::grid_dependency_enter();
    const uint32_t begin = d_begin ? *d_begin : 0u;
    const uint32_t end = min(*d_end, max_rows);
    const uint32_t dst0 = *d_dst_count;
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; begin + r < end; r += gridDim.x * blockDim.x) {
        const uint32_t dst = dst0 + r;
        if (dst >= dst_capacity) {
            record_status(h, FG_ERR_CAPACITY);
            return;
        }
        for (uint32_t c = 0; c < cp.ncols; ++c) copy_col(cp.col[c], begin + r, dst);
    }
}

__global__ void k_append_counts(uint32_t max_rows, const uint32_t* d_begin, uint32_t* d_src_count,
                                uint32_t* d_dst_count, uint32_t dst_capacity) {
    flamegpu::detail::grid_dependency_enter();
    const uint32_t begin = d_begin ? *d_begin : 0u;
    const uint32_t end = min(*d_src_count, max_rows);
    const uint32_t moved = end > begin ? end - begin : 0u;
    const uint32_t total = *d_dst_count + moved;
    *d_dst_count = total < dst_capacity ? total : dst_capacity;
    *d_src_count = begin < end ? begin : end;
}

}  // namespace fgk

extern "C" int fg_append_rows(const fg_column* cols, uint32_t ncols, uint32_t max_rows, const uint32_t* d_begin,
                              uint32_t* d_src_count, uint32_t* d_dst_count, uint32_t dst_capacity, void* workspace,
                              size_t workspace_bytes, void* stream) {
    if (!workspace || workspace_bytes < sizeof(WsHeader) || !d_src_count || !d_dst_count || ncols > FG_MAX_COLUMNS ||
        (ncols && !cols))
        return FG_ERR_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    WsHeader* h = reinterpret_cast<WsHeader*>(workspace);
    CompactParams cp{};
    for (uint32_t c = 0; c < ncols; ++c) cp.col[c] = cols[c];
    cp.ncols = ncols;
    cp.id_col = -1;
    int dev = 0, sms = 132;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint32_t grid = std::max(1u, std::min((max_rows + kThreads - 1) / kThreads, static_cast<uint32_t>(sms * 8)));
    launch(k_append_rows, grid, kThreads, st, cp, max_rows, d_begin, d_src_count, d_dst_count, dst_capacity, h);
    launch(k_append_counts, 1, 1, st, max_rows, d_begin, d_src_count, d_dst_count, dst_capacity);
    return launch_err();
}

// ------------------------------------------------------ segmented (batches)
//
// The same fused compaction over a batch of instances (fg_batch_instance):
// instance k owns rows [row_begin_k, row_begin_k + row_capacity_k) of every
// column and its first counts[k] rows are its agents. Its rows are cut into
// tiles of kCompTile rows that never cross into another instance (tile_begin
// maps instances to their first tile), so one launch compacts every instance
// in place of its own segment: a tile looks back only over the tiles of its
// instance, survivors of instance k land from row_begin_k, its births after
// its S_k survivors (counted first, per instance), with ids from next_ids[k].
// The last block to finish writes every instance's new count.
namespace fgk {

__device__ __forceinline__ uint32_t batch_instance_of_row(const fg_batch_instance* inst, uint32_t ninst, uint32_t row) {
    uint32_t lo = 0, hi = ninst - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (__ldg(&inst[mid].row_begin) <= row)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// survivors per instance: rows below the instance's count with alive != 0
// (alive == NULL: every agent survives)
__global__ void __launch_bounds__(kThreads) k_count_alive_batched(const fg_batch_instance* __restrict__ inst,
                                                                  uint32_t ninst, const uint32_t* __restrict__ counts,
                                                                  uint32_t total_rows, const uint32_t* __restrict__ alive,
                                                                  uint32_t* alive_total) {
    flamegpu::detail::grid_dependency_enter();
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < total_rows; base += stride) {
        const uint32_t i = base + threadIdx.x;
        bool a = false;
        uint32_t k = 0;
        if (i < total_rows) {
            k = batch_instance_of_row(inst, ninst, i);
            const uint32_t local = i - __ldg(&inst[k].row_begin);
            a = local < __ldg(counts + k) && (alive == nullptr || alive[i] != 0);
        }
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, a);
        if (a) {
            const uint32_t peers = __match_any_sync(m, k);
            if (lane_id() == static_cast<uint32_t>(__ffs(peers) - 1)) atomicAdd(alive_total + k, __popc(peers));
        }
    }
}

__global__ void __launch_bounds__(kThreads) k_compact_batched(
    const __grid_constant__ CompactParams cp, const fg_batch_instance* __restrict__ inst,
    const uint32_t* __restrict__ tile_begin, uint32_t ninst, uint32_t ntiles, uint32_t* counts,
    const uint32_t* __restrict__ alive, const uint32_t* __restrict__ born, uint32_t* next_ids, uint32_t* alive_total,
    uint32_t* birth_total, uint64_t* status0, uint32_t stride_tiles, WsHeader* h) {
    flamegpu::detail::grid_dependency_enter();
    __shared__ uint32_t s_tile, s_inst, s_last;
    __shared__ uint32_t s_cnt_a[kCompItems][kThreads / 32];
    __shared__ uint32_t s_cnt_b[kCompItems][kThreads / 32];
    __shared__ uint32_t s_tot[2];
    __shared__ uint64_t s_excl;
    const uint32_t tid = threadIdx.x, lane = lane_id(), warp = tid >> 5;
    const uint32_t limit = spin_limit_of(h);  // before the acquire load (no extra round trip)
    const bool withhold = h->withhold != 0;
    const uint32_t parity = ld_acquire_u32(&h->comp_parity) & 1u;
    uint64_t* status = status0 + static_cast<size_t>(parity) * stride_tiles;
    uint64_t* other = status0 + static_cast<size_t>(parity ^ 1u) * stride_tiles;
    for (uint32_t t = blockIdx.x * blockDim.x + tid; t < stride_tiles; t += gridDim.x * blockDim.x) other[t] = 0;
    for (;;) {
        if (tid == 0) {
            const uint32_t t = atomicAdd(&h->comp_ticket, 1u);
            s_tile = t;
            if (t < ntiles) {  // the instance whose tiles hold t
                uint32_t lo = 0, hi = ninst - 1;
                while (lo < hi) {
                    const uint32_t mid = (lo + hi + 1) >> 1;
                    if (__ldg(tile_begin + mid) <= t)
                        lo = mid;
                    else
                        hi = mid - 1;
                }
                s_inst = lo;
            }
        }
        __syncthreads();
        const uint32_t tile = s_tile;
        if (tile >= ntiles) break;  // the same in every thread
        const uint32_t k = s_inst;
        const uint32_t t0 = __ldg(tile_begin + k);
        const uint32_t local = tile - t0;
        const uint32_t rb = __ldg(&inst[k].row_begin), cap = __ldg(&inst[k].row_capacity);
        const uint32_t n = min(counts[k], cap);
        const uint32_t lbase = local * kCompTile;
        if (lbase >= n) {  // no agents in this tile (nor in the instance's later ones)
            __syncthreads();
            continue;
        }
        const uint32_t S = alive_total[k];
        const uint32_t nid = next_ids ? next_ids[k] : 0u;
        uint32_t ba[kCompItems], bb[kCompItems];
#pragma unroll
        for (int q = 0; q < kCompItems; ++q) {
            const uint32_t li = lbase + q * kThreads + tid;
            const bool in = li < n;
            const bool a = in && (alive == nullptr || alive[rb + li] != 0);
            const bool b = in && born != nullptr && born[rb + li] != 0;
            ba[q] = __ballot_sync(0xFFFFFFFFu, a);
            bb[q] = __ballot_sync(0xFFFFFFFFu, b);
            if (lane == 0) {
                s_cnt_a[q][warp] = __popc(ba[q]);
                s_cnt_b[q][warp] = __popc(bb[q]);
            }
        }
        __syncthreads();
        if (tid == 0) {
            uint32_t ra = 0, rbb = 0;
            for (int q = 0; q < kCompItems; ++q)
                for (int w = 0; w < kThreads / 32; ++w) {
                    const uint32_t a = s_cnt_a[q][w], b = s_cnt_b[q][w];
                    s_cnt_a[q][w] = ra;
                    s_cnt_b[q][w] = rbb;
                    ra += a;
                    rbb += b;
                }
            s_tot[0] = ra;
            s_tot[1] = rbb;
        }
        __syncthreads();
        if (tid < 32) {
            const uint64_t agg = (static_cast<uint64_t>(s_tot[0]) << 31) | s_tot[1];
            uint64_t excl = 0;
            uint64_t* st = status + t0;
            if (local == 0) {
                if (tid == 0 && !(withhold && tile == 0)) st_release_u64(st, pair_pack(2, s_tot[0], s_tot[1]));
            } else {
                if (tid == 0) st_release_u64(st + local, (1ull << 62) | agg);
                excl = lookback_pair(st, local, h, limit);
                if (tid == 0) st_release_u64(st + local, (2ull << 62) | ((excl + agg) & kPairMask));
            }
            if (tid == 0) {
                s_excl = excl;
                if (lbase + kCompTile >= n)  // the instance's last tile with agents: its births
                    birth_total[k] = static_cast<uint32_t>((excl + agg) & 0x7FFFFFFFu);
            }
        }
        __syncthreads();
        const uint32_t ea = static_cast<uint32_t>((s_excl >> 31) & 0x7FFFFFFFu);
        const uint32_t eb = static_cast<uint32_t>(s_excl & 0x7FFFFFFFu);
        const uint32_t lt = lanemask_lt();
#pragma unroll
        for (int q = 0; q < kCompItems; ++q) {
            const uint32_t i = rb + lbase + q * kThreads + tid;
            if ((ba[q] >> lane) & 1u) copy_row(cp.col, cp.ncols, i, rb + ea + s_cnt_a[q][warp] + __popc(ba[q] & lt), -1, 0u);
            if ((bb[q] >> lane) & 1u) {
                const uint32_t r = eb + s_cnt_b[q][warp] + __popc(bb[q] & lt);
                const bool claimed = born[i] == 2u;  // id claimed during the function: kept
                if (S + r < cap)
                    copy_row(cp.bcol, cp.ncols, i, rb + S + r, claimed ? -1 : cp.id_col, nid + r);
                else
                    record_status(h, FG_ERR_CAPACITY);
            }
        }
        __syncthreads();  // shared state is reused by the next tile
    }
    // the last block to finish writes the counts and resets the tickets
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        s_last = atomicAdd(&h->comp_done, 1u) == gridDim.x - 1 ? 1u : 0u;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    for (uint32_t k = tid; k < ninst; k += blockDim.x) {
        const uint32_t births = *reinterpret_cast<volatile uint32_t*>(birth_total + k);
        const uint32_t S = *reinterpret_cast<volatile uint32_t*>(alive_total + k);
        const uint32_t cap = __ldg(&inst[k].row_capacity);
        const uint32_t total = S + births;
        counts[k] = total < cap ? total : cap;
        if (next_ids && cp.id_col >= 0) next_ids[k] += births;
        birth_total[k] = 0;
        alive_total[k] = 0;
    }
    __syncthreads();
    if (tid == 0) {
        h->comp_ticket = 0;
        h->comp_done = 0;
        atomicExch(&h->comp_parity, parity ^ 1u);
        __threadfence();
    }
}

__global__ void k_set_alive_total_batched(const uint32_t* counts, uint32_t ninst, uint32_t* alive_total) {
    flamegpu::detail::grid_dependency_enter();
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < ninst; k += gridDim.x * blockDim.x)
        alive_total[k] = counts[k];
}

struct BatchCompactLayout {
    size_t alive, births, status, total;
};
inline BatchCompactLayout batch_compact_layout(uint32_t ntiles, uint32_t ninst) {
    BatchCompactLayout L;
    L.alive = sizeof(WsHeader);
    L.births = L.alive + align_up(sizeof(uint32_t) * ninst, 256);
    L.status = L.births + align_up(sizeof(uint32_t) * ninst, 256);
    L.total = L.status + align_up(sizeof(uint64_t) * 2 * std::max(ntiles, 1u), 256);
    return L;
}

}  // namespace fgk

extern "C" uint32_t fg_batch_compact_tiles(const fg_batch_instance* instances, uint32_t ninst, uint32_t* tile_begin) {
    uint32_t t = 0;
    for (uint32_t k = 0; k < ninst; ++k) {
        if (tile_begin) tile_begin[k] = t;
        t += std::max(1u, (instances[k].row_capacity + kCompTile - 1) / kCompTile);
    }
    if (tile_begin) tile_begin[ninst] = t;
    return t;
}

extern "C" size_t fg_compact_batched_workspace_size(uint32_t ntiles, uint32_t ninst) {
    return batch_compact_layout(ntiles, ninst).total;
}

extern "C" int fg_compact_agents_batched(const fg_batch_instance* instances, const uint32_t* tile_begin, uint32_t ninst,
                                         uint32_t ntiles, uint32_t total_rows, uint32_t* counts, const uint32_t* alive,
                                         const uint32_t* born, const fg_column* cols, const fg_column* birth_cols,
                                         uint32_t ncols, int32_t id_col, uint32_t* next_ids, void* workspace,
                                         size_t workspace_bytes, void* stream) {
    if (!instances || !tile_begin || !ninst || !counts || !workspace || ncols > FG_MAX_COLUMNS || (ncols && !cols))
        return FG_ERR_INVALID_ARGUMENT;
    if (born && ncols && !birth_cols) return FG_ERR_INVALID_ARGUMENT;
    if (id_col >= static_cast<int32_t>(ncols)) return FG_ERR_INVALID_ARGUMENT;
    if (id_col >= 0 && (cols[id_col].elem_bytes != 4 || !next_ids)) return FG_ERR_INVALID_ARGUMENT;
    if (total_rows >= (1u << 31)) return FG_ERR_UNSUPPORTED;
    const BatchCompactLayout L = batch_compact_layout(ntiles, ninst);
    if (workspace_bytes < L.total || (reinterpret_cast<uintptr_t>(workspace) & 255)) return FG_ERR_WORKSPACE;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    char* ws = static_cast<char*>(workspace);
    WsHeader* h = reinterpret_cast<WsHeader*>(ws);
    uint32_t* alive_total = reinterpret_cast<uint32_t*>(ws + L.alive);
    uint32_t* birth_total = reinterpret_cast<uint32_t*>(ws + L.births);
    uint64_t* status = reinterpret_cast<uint64_t*>(ws + L.status);
    // alive_total / birth_total are zero here: the workspace starts zeroed and
    // every call's last block clears them
    if (alive)
        launch(k_count_alive_batched, count_grid(total_rows), kThreads, st, instances, ninst,
               static_cast<const uint32_t*>(counts), total_rows, alive, alive_total);
    else
        launch(k_set_alive_total_batched, std::max(1u, (ninst + kThreads - 1) / kThreads), kThreads, st,
               static_cast<const uint32_t*>(counts), ninst, alive_total);
    CompactParams cp{};
    for (uint32_t c = 0; c < ncols; ++c) {
        cp.col[c] = cols[c];
        cp.bcol[c] = birth_cols ? birth_cols[c] : cols[c];
    }
    cp.ncols = ncols;
    cp.id_col = id_col;
    const uint32_t stride_tiles =
        static_cast<uint32_t>((workspace_bytes - L.status) / (2 * sizeof(uint64_t)));
    launch(k_compact_batched, std::min(ntiles, 4u * device_sms()), kThreads, st, cp, instances, tile_begin, ninst,
           ntiles, counts, alive, born, next_ids, alive_total, birth_total, status, stride_tiles, h);
    return launch_err();
}
