#ifndef INCLUDE_FLAMEGPU_DETAIL_SPATIAL_KEYS_CUH_
#define INCLUDE_FLAMEGPU_DETAIL_SPATIAL_KEYS_CUH_
// Bin keys of spatial messages and agents, shared by the index-build kernels
// and by agent-function launches that compute them for the build or sort that
// follows (so that its first kernel, which only computes them, is not run).
#include <cstdint>

#include "flamegpu_gb300/fg_capi.h"

namespace flamegpu {
namespace detail {

// getGridPosition3D + getHash3D (MessageSpatial3DDevice.cuh:646-672) /
// getGridPosition2D + getHash2D (MessageSpatial2DDevice.cuh:605-627).
__device__ __forceinline__ uint32_t spatial_message_bin(const fg_spatial_grid& g, float x, float y, float z) {
    int gx = static_cast<int>(floorf((x - g.min[0]) / g.radius));
    int gy = static_cast<int>(floorf((y - g.min[1]) / g.radius));
    const int dx = static_cast<int>(g.gridDim[0]), dy = static_cast<int>(g.gridDim[1]);
    gx = gx < 0 ? 0 : (gx >= dx ? dx - 1 : gx);
    gy = gy < 0 ? 0 : (gy >= dy ? dy - 1 : gy);
    if (g.dims == 3) {
        int gz = static_cast<int>(floorf((z - g.min[2]) / g.radius));
        const int dz = static_cast<int>(g.gridDim[2]);
        gz = gz < 0 ? 0 : (gz >= dz ? dz - 1 : gz);
        return static_cast<uint32_t>(gz) * g.gridDim[0] * g.gridDim[1] + static_cast<uint32_t>(gy) * g.gridDim[0] +
               static_cast<uint32_t>(gx);
    }
    return static_cast<uint32_t>(gy) * g.gridDim[0] + static_cast<uint32_t>(gx);
}

/** The automatic spatial sort's grid (CUDASimulation.cu:494-507, :569-571). */
struct SortKeyGrid {
    float min[3];
    float width[3];
    float gd_f[3];
    uint32_t gd[3];
    uint32_t mask;
};

// Cells of the sort grid; keys at or past it come from positions outside the
// environment (the key is not clamped).
__host__ __device__ __forceinline__ uint32_t sort_cells(const SortKeyGrid& s) { return s.gd[0] * s.gd[1] * s.gd[2]; }

// calculateSpatialHash (src/flamegpu/simulation/CUDASimulation.cu:380-408): unclamped,
// width based; masked to the radix sort's bit range (:569-571).
__device__ __forceinline__ uint32_t spatial_sort_key(const SortKeyGrid& s, int dims, float x, float y, float z) {
    const int gx = static_cast<int>(floorf(((x - s.min[0]) / s.width[0]) * s.gd_f[0]));
    const int gy = static_cast<int>(floorf(((y - s.min[1]) / s.width[1]) * s.gd_f[1]));
    uint32_t h;
    if (dims == 3) {
        const int gz = static_cast<int>(floorf(((z - s.min[2]) / s.width[2]) * s.gd_f[2]));
        h = static_cast<uint32_t>(gz * s.gd[0] * s.gd[1] + (gy * s.gd[0]) + gx);
    } else {
        h = static_cast<uint32_t>((gy * s.gd[0]) + gx);
    }
    return h & s.mask;
}

// Words of a build workspace's header that a key-computing launch resets for
// the kernels after it (the layout of the kernels' workspace header).
constexpr int kWsHdrScanEpoch = 1;
constexpr int kWsHdrScanTicket = 2;
constexpr int kWsHdrLongCount = 4;
// raised to the largest sort key past the grid's cells (positions outside the
// environment; 0 if none): the sort's scan stops past max(it, cells - 1)
constexpr int kWsHdrKeyMax = 9;
// raised when a build's keys are not in row order (non-decreasing over rows
// that all carry a key); left 0, the rows are already in the order the build
// would give them and its placement and ranking are skipped
constexpr int kWsHdrDisorder = 12;

/** Where a launch writes the keys of a build or an agent sort (mode 0: none). */
struct KeyTarget {
    uint32_t mode;           // kKeyNone, kKeyMessageBin or kKeySortKey
    uint32_t dims;
    fg_spatial_grid grid;    // message bins
    SortKeyGrid sort;        // sort keys
    const float* x;          // positions: the message's (by message row) or the agent's (by agent row)
    const float* y;
    const float* z;
    uint32_t* keys;          // per row: its key, or 0xFFFFFFFF when it carries no message
    uint32_t* slot;          // per row: its place among the rows of its key (histogram order)
    uint32_t* hist;          // per key: rows counted (zero before the launch)
    uint32_t* header;        // the workspace header
    uint32_t* edges;         // per 32-row group w: keys of rows 32w and 32w + 31 (row-order check)
};
constexpr uint32_t kKeyNone = 0, kKeyMessageBin = 1, kKeySortKey = 2;

// Block 0, thread 0 of the launch: what the key kernel did at its start.
__device__ __forceinline__ void key_target_reset(const KeyTarget& t) {
    t.header[kWsHdrLongCount] = 0u;
    t.header[kWsHdrScanTicket] = 0u;
    t.header[kWsHdrScanEpoch] = (t.header[kWsHdrScanEpoch] + 1u) & 0x3FFFFFFFu;
}

// Key of a row at position (px, py, pz); 0xFFFFFFFF when it carries none.
__device__ __forceinline__ uint32_t key_target_key(const KeyTarget& t, bool valid, float px, float py, float pz) {
    if (!valid) return 0xFFFFFFFFu;
    return t.mode == kKeyMessageBin ? spatial_message_bin(t.grid, px, py, pz)
                                    : spatial_sort_key(t.sort, static_cast<int>(t.dims), px, py, pz);
}

// Histogram counts and slots of the keys k[0], k[1] of rows row[0], row[1]
// for the targets t[0], t[1] (mode kKeyNone: skipped), by the lanes that
// reach it together: lanes with the same key share one atomic, and the two
// targets' atomics are issued before either result is used. Returns bit j set
// where target j's rows here are out of order (the same in every lane); the
// launch raises the targets' disorder flags once per block at its end
// (key_targets_order_flush), so a launch over unsorted rows does not store to
// one word from every warp.
__device__ __forceinline__ uint32_t key_targets_write(const KeyTarget (&t)[2], const uint32_t (&row)[2],
                                                      const uint32_t (&k)[2]) {
    // the lanes here together (rows skipped or finished earlier are not);
    // every one of them executes the ballots, those with a key the matches
    const uint32_t active = __activemask();
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t peers[2] = {0u, 0u}, base[2] = {0u, 0u};
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        if (t[j].mode == kKeyNone) continue;  // the same for every lane
        const uint32_t counted = __ballot_sync(active, k[j] != 0xFFFFFFFFu);
        if (k[j] != 0xFFFFFFFFu) peers[j] = __match_any_sync(counted, k[j]);
    }
#pragma unroll
    for (int j = 0; j < 2; ++j)
        if (peers[j] && lane == static_cast<uint32_t>(__ffs(peers[j]) - 1))
            base[j] = atomicAdd(t[j].hist + k[j], static_cast<uint32_t>(__popc(peers[j])));
    // an agent sort's scan stops past the grid's cells, or past the largest
    // key of a row outside them (rare: one atomic per such row)
    if (t[1].mode == kKeySortKey && k[1] >= sort_cells(t[1].sort)) atomicMax(t[1].header + kWsHdrKeyMax, k[1]);
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        if (t[j].mode == kKeyNone) continue;
        uint32_t s = 0;
        if (peers[j]) s = __shfl_sync(peers[j], base[j], __ffs(peers[j]) - 1) + __popc(peers[j] & ((1u << lane) - 1u));
        t[j].keys[row[j]] = k[j];
        t[j].slot[row[j]] = s;
    }
    // row order: each key against the key of the row before it when that row
    // is the lane below's; a row whose predecessor is elsewhere is compared by
    // the build's scan if it starts a 32-row group (rows 32w - 1, 32w, through
    // the group edge keys written here), else counted as out of order. A row
    // without a key is out of order.
    uint32_t out_of_order = 0u;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        if (t[j].mode == kKeyNone) continue;
        const uint32_t g = row[j] & 31u;
        if (g == 0u || g == 31u) t[j].edges[2u * (row[j] >> 5) + (g ? 1u : 0u)] = k[j];
        const uint32_t pk = __shfl_up_sync(active, k[j], 1);
        const uint32_t pr = __shfl_up_sync(active, row[j], 1);
        const bool has_prev = lane > 0u && ((active >> (lane - 1u)) & 1u) && pr + 1u == row[j];
        const bool bad = k[j] == 0xFFFFFFFFu || (has_prev ? pk > k[j] : (row[j] & 31u) != 0u);
        if (__ballot_sync(active, bad)) out_of_order |= 1u << j;
    }
    return out_of_order;
}

// End of a key-computing launch, reached by every thread of the block:
// raises target j's disorder flag if any of the block's rows were out of
// order for it (bit j of `out_of_order`, as key_targets_write returned).
__device__ __forceinline__ void key_targets_order_flush(const KeyTarget (&t)[2], uint32_t out_of_order) {
    const int any0 = __syncthreads_or(out_of_order & 1u);
    const int any1 = __syncthreads_or(out_of_order & 2u);
    if (threadIdx.x == 0) {
        if (any0 && t[0].mode != kKeyNone) t[0].header[kWsHdrDisorder] = 1u;
        if (any1 && t[1].mode != kKeyNone) t[1].header[kWsHdrDisorder] = 1u;
    }
}

}  // namespace detail
}  // namespace flamegpu

#endif  // INCLUDE_FLAMEGPU_DETAIL_SPATIAL_KEYS_CUH_
