// Single-pass exclusive scan of u32 values with decoupled look-back
// (Merrill & Garland, "Single-pass Parallel Prefix Scan with Decoupled
// Look-back", 2016). Tiles are handed out by a ticket counter in launch order,
// so every tile a block waits on belongs to a block that is already running;
// every wait is bounded and a give-up is recorded in the workspace header.
//
// Tile statuses are 64-bit words: [63:62] flag (1 aggregate, 2 inclusive
// prefix), [61:32] a 30-bit epoch, [31:0] the value. The epoch changes after
// each scan (the last block to finish advances it and resets the ticket), so
// stale statuses of earlier scans read as "not ready" and the status array
// never needs clearing.
#pragma once

#include "common.cuh"

namespace fgk {

constexpr int kScanItems = 16;                       // u32 per thread
constexpr int kScanTile = kThreads * kScanItems;     // 4096 per tile

__device__ __forceinline__ uint64_t scan_pack(uint32_t flag, uint32_t epoch, uint32_t v) {
    return (static_cast<uint64_t>(flag) << 62) | (static_cast<uint64_t>(epoch & 0x3FFFFFFFu) << 32) | v;
}

// Block-wide exclusive scan of one u32 per thread; returns the exclusive
// prefix of this thread and writes the block total to *total.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total, uint32_t* smem_warp) {
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    uint32_t inc = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, inc, d);
        if (lane >= static_cast<uint32_t>(d)) inc += t;
    }
    if (lane == 31) smem_warp[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const uint32_t nw = blockDim.x >> 5;
        uint32_t w = lane < nw ? smem_warp[lane] : 0;
        uint32_t winc = w;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, winc, d);
            if (lane >= static_cast<uint32_t>(d)) winc += t;
        }
        if (lane < nw) smem_warp[lane] = winc - w;   // exclusive warp offsets
        if (lane == nw - 1) smem_warp[32] = winc;    // block total
    }
    __syncthreads();
    const uint32_t r = smem_warp[warp] + inc - v;
    *total = smem_warp[32];
    return r;
}

// Warp 0 of a block: look back over predecessor tiles of `tile` and return the
// exclusive prefix. `status` must already hold this tile's aggregate.
// At most spin_limit_of(h) polls per predecessor (read once a wait gets
// long, off the fast path); a give-up is recorded in the header and the
// predecessor counts as an inclusive prefix of 0, so the scan finishes (with
// wrong prefixes) instead of hanging.
__device__ __forceinline__ uint32_t lookback_u32(const uint64_t* status, uint32_t tile, uint32_t epoch, WsHeader* h) {
    const uint32_t lane = lane_id();
    uint32_t excl = 0;
    int64_t pred = static_cast<int64_t>(tile) - 1;
    while (pred >= 0) {
        const int64_t t = pred - lane;
        uint32_t flag = 2, val = 0;
        if (t >= 0) {
            uint32_t spins = 0, limit = 0xFFFFFFFFu;
            for (;;) {
                const uint64_t s = ld_acquire_u64(status + t);
                const uint32_t e = static_cast<uint32_t>(s >> 32) & 0x3FFFFFFFu;
                flag = static_cast<uint32_t>(s >> 62);
                val = static_cast<uint32_t>(s);
                if (flag != 0 && e == (epoch & 0x3FFFFFFFu)) break;
                if (spins == 16) limit = spin_limit_of(h);
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
        if (pmask) {
            const uint32_t k = __ffs(pmask) - 1;  // nearest inclusive prefix
            uint32_t contrib = lane <= k ? val : 0;
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) contrib += __shfl_xor_sync(0xFFFFFFFFu, contrib, d);
            excl += contrib;
            break;
        }
        uint32_t contrib = val;
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) contrib += __shfl_xor_sync(0xFFFFFFFFu, contrib, d);
        excl += contrib;
        pred -= 32;
    }
    return excl;
}

// Exclusive scan of in[0..n) into out[0..n). If zero_in, in[] is cleared to 0
// after it has been read (in != out). A tile is R sub-tiles of kScanTile
// values: the block sums them (R block scans), publishes the tile's total and
// looks back once, then reads them again (from L2) to write the prefixes. A
// look-back resolves at most 32 tiles per round of the inclusive-prefix
// frontier, so large scans take R = 4 and need a quarter of the rounds. With
// self_reset the last block to finish resets the ticket and advances the epoch
// for the next scan on this workspace; without it the kernel launched just
// before this one has done so (scan_reset), which spares every block a fence
// and an atomic at its end.
__device__ __forceinline__ void scan_reset(WsHeader* h) {
    h->scan_ticket = 0u;
    h->scan_epoch = (h->scan_epoch + 1u) & 0x3FFFFFFFu;
}

__device__ __forceinline__ void scan_load(const uint32_t* in, uint64_t base, uint32_t n, bool vec,
                                          uint32_t (&v)[kScanItems]) {
    if (vec) {
        const uint4* p = reinterpret_cast<const uint4*>(in + base);
#pragma unroll
        for (int k = 0; k < kScanItems / 4; ++k) {
            const uint4 q = p[k];
            v[4 * k] = q.x; v[4 * k + 1] = q.y; v[4 * k + 2] = q.z; v[4 * k + 3] = q.w;
        }
    } else {
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) v[k] = (base + k < n) ? in[base + k] : 0u;
    }
}

// The row-order check a build's scan finishes for the key launch before it
// (edges null: none). That launch compared each row's key with the row before
// it inside 32-row groups and wrote each group's first and last key (edges[2w],
// edges[2w + 1]); the scan compares the keys of rows 32w - 1 and 32w, and
// raises the workspace's disorder flag at a descent.
struct OrderCheck {
    const uint32_t* edges = nullptr;
    const uint32_t* d_n = nullptr;  // rows (device), at most max_n; null: max_n
    uint32_t max_n = 0;
};

// The blocks share the 32-row group boundaries (block `b` of `nb` taking part);
// unless the key launch already found a descent (`pending` false), each block
// reads its boundaries' keys.
__device__ __forceinline__ void order_check_boundaries(const OrderCheck& oc, bool pending, WsHeader* h, uint32_t b,
                                                       uint32_t nb) {
    uint32_t bad = 0u;
    if (pending) {
        const uint32_t rows = oc.d_n ? min(*oc.d_n, oc.max_n) : oc.max_n;
        const uint2* e = reinterpret_cast<const uint2*>(oc.edges);
#pragma unroll 4
        for (uint32_t w = 1u + b * blockDim.x + threadIdx.x; static_cast<uint64_t>(w) * 32u < rows; w += nb * blockDim.x)
            bad |= e[w - 1u].y > e[w].x ? 1u : 0u;
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0) h->disorder = 1u;
}

// One exclusive scan of a launch: in[0..n) into out[0..n) on the workspace
// header h and its tile statuses; last, last_floor and oc as k_scan_u32's.
struct ScanJob {
    const uint32_t* in;
    uint32_t* out;
    uint32_t n;
    int zero_in;
    uint64_t* status;
    WsHeader* h;
    const uint32_t* last;
    uint32_t last_floor;
    OrderCheck oc;
};

// Tile `tile` (of `ntiles`) of scan j, by the whole block, under the epoch the
// block read; withhold (tile 0: a test hook) and pending (the row-order check
// is still open) as read by thread 0. Returns false for a tile wholly past the
// scan's last value (it only takes part in the order check).
template <int R>
__device__ __forceinline__ bool scan_tile(const ScanJob& j, uint32_t tile, uint32_t ntiles, uint32_t epoch,
                                          bool withhold, bool pending, uint32_t* s_warp, uint32_t* s_excl) {
    uint32_t n = j.n;
    // last (no self reset): the values past index max(*last, last_floor) + 1
    // are zero and their prefixes unused; the tiles wholly past it have nothing to do
    if (j.last) n = min(n, max(*j.last, j.last_floor) + 2u);
    if (static_cast<uint64_t>(tile) * R * kScanTile >= n && tile != 0) {
        if (j.oc.edges) order_check_boundaries(j.oc, pending, j.h, tile, ntiles);
        return false;
    }
    const uint32_t* in = j.in;
    uint32_t* out = j.out;
    const bool in_al = (reinterpret_cast<uintptr_t>(in) & 15) == 0;
    const bool out_al = (reinterpret_cast<uintptr_t>(out) & 15) == 0;
    uint32_t v[kScanItems];
    uint32_t texcl[R];  // this thread's prefix inside the tile, per sub-tile
    uint32_t ttotal = 0;
    const uint64_t base0 = static_cast<uint64_t>(tile) * R * kScanTile + threadIdx.x * kScanItems;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const uint64_t base = base0 + r * kScanTile;
        scan_load(in, base, n, in_al && base + kScanItems <= n, v);
        uint32_t tsum = 0;
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) tsum += v[k];
        uint32_t btotal;
        texcl[r] = ttotal + block_exclusive_scan(tsum, &btotal, s_warp);
        ttotal += btotal;
        if (R > 1) __syncthreads();  // s_warp is reused by the next sub-tile's scan
    }
    // publish this tile and look back
    if (threadIdx.x < 32) {
        uint32_t excl = 0;
        if (tile == 0) {
            if (threadIdx.x == 0 && !withhold) st_release_u64(j.status, scan_pack(2, epoch, ttotal));
        } else {
            if (threadIdx.x == 0) st_release_u64(j.status + tile, scan_pack(1, epoch, ttotal));
            excl = lookback_u32(j.status, tile, epoch, j.h);
            if (threadIdx.x == 0) st_release_u64(j.status + tile, scan_pack(2, epoch, excl + ttotal));
        }
        if (threadIdx.x == 0) *s_excl = excl;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const uint64_t base = base0 + r * kScanTile;
        const bool full = base + kScanItems <= n;
        if (R > 1) scan_load(in, base, n, in_al && full, v);  // the one sub-tile of R = 1 is still held
        uint32_t run = *s_excl + texcl[r];
        uint32_t o[kScanItems];
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            o[k] = run;
            run += v[k];
        }
        if (full && out_al) {
            uint4* p = reinterpret_cast<uint4*>(out + base);
#pragma unroll
            for (int k = 0; k < kScanItems / 4; ++k)
                p[k] = make_uint4(o[4 * k], o[4 * k + 1], o[4 * k + 2], o[4 * k + 3]);
        } else {
#pragma unroll
            for (int k = 0; k < kScanItems; ++k)
                if (base + k < n) out[base + k] = o[k];
        }
        if (j.zero_in) {
            uint32_t* zin = const_cast<uint32_t*>(in);
            if (full && in_al) {
                uint4* p = reinterpret_cast<uint4*>(zin + base);
#pragma unroll
                for (int k = 0; k < kScanItems / 4; ++k) p[k] = make_uint4(0, 0, 0, 0);
            } else {
#pragma unroll
                for (int k = 0; k < kScanItems; ++k)
                    if (base + k < n) zin[base + k] = 0;
            }
        }
    }
    if (j.oc.edges) order_check_boundaries(j.oc, pending, j.h, tile, ntiles);
    return true;
}

// Thread 0: the block's tile (ticket), the scan's epoch, and the test hook
// and order-check state. The key launch's flag is final (it completed before
// this launch): read before the acquire, so the loads overlap.
struct ScanTicket {
    uint32_t tile, epoch, withhold, pending;
};
__device__ __forceinline__ ScanTicket scan_ticket_of(const ScanJob& j, uint32_t ticket) {
    ScanTicket t;
    t.pending = j.oc.edges != nullptr && j.h->disorder == 0u;
    t.tile = ticket;
    t.epoch = ld_acquire_u32(&j.h->scan_epoch);
    t.withhold = ticket == 0 ? j.h->withhold : 0u;
    return t;
}

template <int R>
__global__ void __launch_bounds__(kThreads, 6) k_scan_u32(const __grid_constant__ ScanJob j, int self_reset) {
    flamegpu::detail::grid_dependency_enter();
    __shared__ ScanTicket s_t;
    __shared__ uint32_t s_warp[33];
    __shared__ uint32_t s_excl;
    // a test hook (fg_workspace_set_wait_limit): tile 0 does not publish. Only
    // tile 0's thread 0 reads it, before its data loads, and uses it when it
    // publishes, so the load adds nothing to the look-back chain
    if (threadIdx.x == 0) s_t = scan_ticket_of(j, atomicAdd(&j.h->scan_ticket, 1u));
    __syncthreads();
    const ScanTicket t = s_t;
    if (!scan_tile<R>(j, t.tile, gridDim.x, t.epoch, t.withhold != 0u, t.pending != 0u, s_warp, &s_excl)) return;
    if (!self_reset) return;
    // the last block to finish resets the ticket and advances the epoch
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&j.h->scan_done, 1u) == gridDim.x - 1) {
            j.h->scan_ticket = 0;
            j.h->scan_done = 0;
            atomicExch(&j.h->scan_epoch, (t.epoch + 1) & 0x3FFFFFFFu);
            __threadfence();
        }
    }
}

// Two scans in one launch (an agent sort's and a message build's): tickets
// below `tiles_a` are scan a's tiles, the rest scan b's, so each tile still
// waits only on lower tickets of its own scan. The tickets come from a's
// header (reset by the launch before, as for a single scan); no self reset.
template <int R>
__global__ void __launch_bounds__(kThreads, 6) k_scan_pair(const __grid_constant__ ScanJob a,
                                                           const __grid_constant__ ScanJob b, uint32_t tiles_a) {
    flamegpu::detail::grid_dependency_enter();
    __shared__ ScanTicket s_t;
    __shared__ uint32_t s_in_b;
    __shared__ uint32_t s_warp[33];
    __shared__ uint32_t s_excl;
    if (threadIdx.x == 0) {
        const uint32_t ticket = atomicAdd(&a.h->scan_ticket, 1u);
        s_in_b = ticket >= tiles_a;
        s_t = ticket < tiles_a ? scan_ticket_of(a, ticket) : scan_ticket_of(b, ticket - tiles_a);
    }
    __syncthreads();
    const ScanTicket t = s_t;
    if (s_in_b)
        scan_tile<R>(b, t.tile, gridDim.x - tiles_a, t.epoch, t.withhold != 0u, t.pending != 0u, s_warp, &s_excl);
    else
        scan_tile<R>(a, t.tile, tiles_a, t.epoch, t.withhold != 0u, t.pending != 0u, s_warp, &s_excl);
}

// Tiles of a scan of n values with one sub-tile per tile (an upper bound on
// the tiles of any scan of n values: sizes the status array).
inline uint32_t scan_tiles(uint32_t n) { return (n + kScanTile - 1) / kScanTile; }

// Scans of more than this many values take four sub-tiles per tile.
constexpr uint32_t kScanWideMin = 1u << 22;
// The threshold of the calling thread's scans (fg_set_thread_tuning).
inline thread_local uint32_t t_scan_wide_min = kScanWideMin;

// last, last_floor: optional (device) bound, as in k_scan_u32; only without self_reset.
inline cudaError_t launch_scan(const uint32_t* in, uint32_t* out, uint32_t n, int zero_in, uint64_t* status,
                               WsHeader* h, int self_reset, cudaStream_t st, const uint32_t* last = nullptr,
                               uint32_t last_floor = 0, const OrderCheck& oc = OrderCheck()) {
    const ScanJob j{in, out, n, zero_in, status, h, last, last_floor, oc};
    if (n > t_scan_wide_min)
        return launch(k_scan_u32<4>, (n + 4u * kScanTile - 1) / (4u * kScanTile), kThreads, st, j, self_reset);
    return launch(k_scan_u32<1>, scan_tiles(n), kThreads, st, j, self_reset);
}

// Scans a and b (no self reset) in one launch; both take four sub-tiles per
// tile when either is wide.
inline cudaError_t launch_scan_pair(const ScanJob& a, const ScanJob& b, cudaStream_t st) {
    const uint32_t r = (a.n > t_scan_wide_min || b.n > t_scan_wide_min) ? 4u : 1u;
    const uint32_t ta = (a.n + r * kScanTile - 1) / (r * kScanTile), tb = (b.n + r * kScanTile - 1) / (r * kScanTile);
    if (r == 4u) return launch(k_scan_pair<4>, ta + tb, kThreads, st, a, b, ta);
    return launch(k_scan_pair<1>, ta + tb, kThreads, st, a, b, ta);
}

}  // namespace fgk
