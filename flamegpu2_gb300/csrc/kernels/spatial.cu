// Spatial message index build and automatic spatial agent sort on GB300.
//
// One build = five kernels, no host synchronisation, no allocation:
//   k_bin        bin index per message (clamped floor((p-min)/r), the reference's
//                getGridPosition3D/getHash3D) + warp-aggregated histogram atomics;
//                keeps each message's slot from the atomic (an agent-function
//                launch may do this instead)
//   k_scan_u32   single-pass exclusive scan histogram -> PBM (clears the histogram)
//   k_perm       unstable placement perm[PBM[bin] + slot] = message
//   k_stabilize  per sorted position: restores ascending original index inside
//                short bins (<= kShortBin) and emits the record (or index);
//                long bins are queued as 256-element chunks
//   k_long       orders long bins: a bin whose indices are contiguous is
//                copied in order; otherwise up to 1024 messages one warp each
//                (a bitmap over their indices, or a bitonic sort), up to 8192
//                one block each (a bitmap over the span of their indices, or a
//                bitonic sort in shared memory), longer ones by ranking each
//                256-element chunk against the whole bin
// The automatic agent sort runs the same pipeline on the reference's sort key;
// its k_stabilize / k_long write every agent column at the stable position.
#include <algorithm>
#include <cstring>
#include <mutex>

#include "common.cuh"
#include "scan.cuh"

namespace fgk {

constexpr uint32_t kShortBin = 32;
// Batches mark the keys of padding rows (rows past an instance's count, or
// messages not output) with this bit: they are counted in their instance's
// padding bucket so positions stay inside the instance's segment, but they are
// never ranked or copied as messages.
constexpr uint32_t kPadBit = 0x80000000u;
constexpr uint32_t kChunk = 256;     // elements of a long bin ranked by one block pass
constexpr uint32_t kRankTile = 2048; // bin elements staged in shared memory per pass

enum KeyMode { kMessageBin = 0, kSortKey = 1 };
enum EmitMode { kEmitRecord = 0, kEmitPerm = 1, kEmitPermColumns = 2 };

// The sort grid and both key functions are shared with agent-function
// launches that compute the keys themselves (flamegpu/detail/spatial_keys.cuh).
using SortGrid = flamegpu::detail::SortKeyGrid;

__device__ __forceinline__ uint32_t load_count(const uint32_t* d_n, uint32_t max_n) {
    if (!d_n) return max_n;
    const uint32_t n = *d_n;
    return n < max_n ? n : max_n;
}

__device__ __forceinline__ uint32_t message_bin(const fg_spatial_grid& g, float x, float y, float z) {
    return flamegpu::detail::spatial_message_bin(g, x, y, z);
}

__device__ __forceinline__ uint32_t sort_key(const SortGrid& s, int dims, float x, float y, float z) {
    return flamegpu::detail::spatial_sort_key(s, dims, x, y, z);
}

// pstride: floats between one row's coordinate and the next row's (1 for
// separate x, y, z columns; 2 or 3 for a packed "xy" / "xyz" array variable)
template <int MODE>
__global__ void __launch_bounds__(kThreads) k_bin(fg_spatial_grid g, SortGrid sg, uint32_t max_n, const uint32_t* d_n,
                                                  const float* __restrict__ x, const float* __restrict__ y,
                                                  const float* __restrict__ z, const uint32_t* __restrict__ valid,
                                                  uint32_t* __restrict__ keys, uint32_t* __restrict__ slot,
                                                  uint32_t* hist, WsHeader* h, uint32_t pstride,
                                                  uint32_t* __restrict__ edges) {
    flamegpu::detail::grid_dependency_enter();
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        h->long_count = 0;
        scan_reset(h);  // for the scan launched next
    }
    const uint32_t n = load_count(d_n, max_n);
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t cells = flamegpu::detail::sort_cells(sg);
    bool out_of_order = false;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint32_t i = base + threadIdx.x;
        const bool act = i < n;
        uint32_t key = kInvalid;
        if (act && (valid == nullptr || valid[i] != 0)) {
            const size_t e = static_cast<size_t>(i) * pstride;
            const float px = x[e], py = y[e], pz = (g.dims == 3) ? z[e] : 0.0f;
            key = (MODE == kMessageBin) ? message_bin(g, px, py, pz) : sort_key(sg, g.dims, px, py, pz);
        }
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, key != kInvalid);
        uint32_t s = 0;
        if (key != kInvalid) {
            s = warp_aggregated_inc(hist, key, m);
            // the sort's scan stops past the cells, or past the largest key of
            // a row outside them (rare)
            if (MODE == kSortKey && key >= cells) atomicMax(&h->key_max, key);
        }
        if (act) {
            keys[i] = key;
            slot[i] = s;
        }
        // row order (rows 32w - 1, 32w are compared by the scan, through the
        // first and last key of every 32-row group)
        if (act && (lane_id() == 0u || lane_id() == 31u)) edges[2u * (i >> 5) + (lane_id() ? 1u : 0u)] = key;
        const uint32_t pk = __shfl_up_sync(0xFFFFFFFFu, key, 1);
        out_of_order = out_of_order || (act && (key == kInvalid || (lane_id() > 0u && pk > key)));
    }
    // one store per block at most (a store per warp to one word serialises)
    if (__syncthreads_or(out_of_order) && threadIdx.x == 0) h->disorder = 1u;
}

// The slot came from the histogram atomics, so pbm[k] + slot < n holds as long
// as the histogram started at zero (fg_workspace_init); a workspace that broke
// that invariant is reported instead of written out of bounds.
__device__ __forceinline__ uint32_t find_instance(const fg_batch_instance* inst, uint32_t ninst, uint32_t row) {
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

// Keys of a batch: each row's instance (binary search of the row offsets),
// then the instance's own message bin / sort key shifted into its bucket
// range; padding rows go to the instance's padding bucket with kPadBit set.
template <int MODE>
__global__ void __launch_bounds__(kThreads) k_bin_batched(const fg_batch_instance* __restrict__ inst,
                                                          const uint32_t* __restrict__ counts, uint32_t ninst,
                                                          uint32_t total_rows, int dims, const float* __restrict__ x,
                                                          const float* __restrict__ y, const float* __restrict__ z,
                                                          const uint32_t* __restrict__ valid,
                                                          uint32_t* __restrict__ keys, uint32_t* __restrict__ slot,
                                                          uint32_t* hist, WsHeader* h) {
    flamegpu::detail::grid_dependency_enter();
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        h->long_count = 0;
        h->disorder = 1u;  // batches always take the placement and ranking path
        scan_reset(h);  // for the scan launched next
    }
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < total_rows; base += stride) {
        const uint32_t i = base + threadIdx.x;
        const bool act = i < total_rows;
        uint32_t key = kInvalid;
        // the instance of the warp's first row, searched once; a lane past that
        // instance's rows (a warp across a boundary) searches its own
        const uint32_t wrow = min(base + (threadIdx.x & ~31u), total_rows - 1u);
        const uint32_t k0 = __shfl_sync(0xFFFFFFFFu, lane_id() == 0 ? find_instance(inst, ninst, wrow) : 0u, 0);
        if (act) {
            const bool in_k0 = k0 + 1 >= ninst || i < __ldg(&inst[k0 + 1].row_begin);
            const uint32_t k = in_k0 ? k0 : find_instance(inst, ninst, i);
            const fg_batch_instance& I = inst[k];
            const uint32_t local = i - I.row_begin;
            const uint32_t bb = I.bucket_begin;
            if (local >= __ldg(counts + k) || (valid != nullptr && valid[i] == 0)) {
                key = (bb + I.nbuckets) | kPadBit;
            } else {
                const float px = x[i], py = y[i], pz = dims == 3 ? z[i] : 0.0f;
                if (MODE == kMessageBin) {
                    key = bb + message_bin(I.grid, px, py, pz);
                } else {
                    SortGrid sg;
                    for (int a = 0; a < 3; ++a) {
                        sg.min[a] = a < dims ? I.grid.min[a] : 0.0f;
                        sg.width[a] = I.sort_width[a];
                        sg.gd[a] = I.sort_gd[a];
                        sg.gd_f[a] = static_cast<float>(I.sort_gd[a]);
                    }
                    sg.mask = I.sort_mask;
                    key = bb + sort_key(sg, dims, px, py, pz);
                }
            }
        }
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, key != kInvalid);
        uint32_t sl = 0;
        if (key != kInvalid) sl = warp_aggregated_inc(hist, key & ~kPadBit, m);
        if (act) {
            keys[i] = key;
            slot[i] = sl;
        }
    }
}

// One counting sort's placement: perm[PBM[key] + slot] = row.
struct PermJob {
    uint32_t max_n;
    const uint32_t* d_n;
    const uint32_t* keys;
    const uint32_t* slot;
    const uint32_t* pbm;
    uint32_t* perm;
    WsHeader* h;
};

// By block b of the nb blocks working on job j.
__device__ __forceinline__ void perm_rows(const PermJob& j, uint32_t b, uint32_t nb) {
    if (j.h->disorder == 0u) return;  // keys in row order: every row keeps its place
    const uint32_t n = load_count(j.d_n, j.max_n);
    for (uint32_t i = b * blockDim.x + threadIdx.x; i < n; i += nb * blockDim.x) {
        const uint32_t k = j.keys[i];
        if (k != kInvalid) {
            const uint32_t at = j.pbm[k & ~kPadBit] + j.slot[i];
            if (at < n)
                j.perm[at] = i;
            else
                record_status(j.h, FG_ERR_WORKSPACE);
        }
    }
}

__global__ void __launch_bounds__(kThreads) k_perm(const __grid_constant__ PermJob j) {
    flamegpu::detail::grid_dependency_enter();
    perm_rows(j, blockIdx.x, gridDim.x);
}

// an agent sort's placement (the first ga blocks) and a message build's (the
// rest), in one launch: the two run side by side as two kernels would
__global__ void __launch_bounds__(kThreads) k_perm_pair(const __grid_constant__ PermJob a,
                                                        const __grid_constant__ PermJob b, uint32_t ga) {
    flamegpu::detail::grid_dependency_enter();
    if (blockIdx.x < ga)
        perm_rows(a, blockIdx.x, ga);
    else
        perm_rows(b, blockIdx.x - ga, gridDim.x - ga);
}

struct RecordParams {
    fg_record_desc rec;
    uint32_t* out;
};

// Gathers record i from its source columns and writes it at dst. Sixteen words
// at a time are all loaded before any is stored, so their latencies overlap.
__device__ __forceinline__ void emit_record(const RecordParams& rp, uint32_t i, uint32_t dst) {
    const uint32_t words = rp.rec.words;
    uint4* o = reinterpret_cast<uint4*>(rp.out + static_cast<size_t>(dst) * words);
    for (uint32_t w0 = 0; w0 < words; w0 += 16) {
        uint32_t v[16];
#pragma unroll
        for (uint32_t k = 0; k < 16; ++k) {
            const uint32_t w = w0 + k;
            const uint32_t* src = w < words ? rp.rec.src[w] : nullptr;
            v[k] = src ? ld_nc_u32(src + static_cast<size_t>(i) * rp.rec.src_stride[w] + rp.rec.src_word[w]) : 0u;
        }
#pragma unroll
        for (uint32_t k = 0; k < 16; k += 4)
            if (w0 + k < words) o[(w0 + k) >> 2] = make_uint4(v[k], v[k + 1], v[k + 2], v[k + 3]);
    }
}

struct ColumnParams {
    fg_column col[FG_MAX_COLUMNS];
    uint32_t ncols;
    uint32_t keep_perm;  // also write the stable permutation (the caller asked for it)
};

template <typename T>
__device__ __forceinline__ void copy_elem(const void* in, void* out, uint32_t src, uint32_t dst) {
    reinterpret_cast<T*>(out)[dst] = reinterpret_cast<const T*>(in)[src];
}

__device__ __forceinline__ void copy_column_elem(const fg_column& c, uint32_t src, uint32_t dst) {
    switch (c.elem_bytes) {
        case 4: copy_elem<uint32_t>(c.in, c.out, src, dst); break;
        case 8: copy_elem<uint2>(c.in, c.out, src, dst); break;
        case 16: copy_elem<uint4>(c.in, c.out, src, dst); break;
        case 1: copy_elem<uint8_t>(c.in, c.out, src, dst); break;
        case 2: copy_elem<uint16_t>(c.in, c.out, src, dst); break;
        default: {
            const uint8_t* a = reinterpret_cast<const uint8_t*>(c.in) + static_cast<size_t>(src) * c.elem_bytes;
            uint8_t* b = reinterpret_cast<uint8_t*>(c.out) + static_cast<size_t>(dst) * c.elem_bytes;
            if ((c.elem_bytes & 3) == 0) {
                for (uint32_t k = 0; k < c.elem_bytes; k += 4)
                    *reinterpret_cast<uint32_t*>(b + k) = *reinterpret_cast<const uint32_t*>(a + k);
            } else {
                for (uint32_t k = 0; k < c.elem_bytes; ++k) b[k] = a[k];
            }
        }
    }
}

// What the last build kernels write for message (or agent) i at sorted
// position dst: its record, its index, or its index and every agent column.
struct EmitParams {
    RecordParams rp;
    ColumnParams cp;
};

// Every agent column's element i written at dst. Runs of four 4-byte columns
// (the common float / int variables) are all loaded before any is stored, so
// their latencies overlap; other columns are copied one by one.
__device__ __forceinline__ void emit_columns(const ColumnParams& cp, uint32_t i, uint32_t dst) {
    for (uint32_t c0 = 0; c0 < cp.ncols; c0 += 4) {
        const uint32_t nk = min(4u, cp.ncols - c0);
        bool words = true;
        for (uint32_t k = 0; k < nk; ++k) words = words && cp.col[c0 + k].elem_bytes == 4u;
        if (words) {
            uint32_t v[4];
#pragma unroll
            for (uint32_t k = 0; k < 4; ++k)
                if (k < nk) v[k] = static_cast<const uint32_t*>(cp.col[c0 + k].in)[i];
#pragma unroll
            for (uint32_t k = 0; k < 4; ++k)
                if (k < nk) static_cast<uint32_t*>(cp.col[c0 + k].out)[dst] = v[k];
        } else {
            for (uint32_t k = 0; k < nk; ++k) copy_column_elem(cp.col[c0 + k], i, dst);
        }
    }
}

template <int EMIT>
__device__ __forceinline__ void emit(const EmitParams& ep, uint32_t* sperm, uint32_t i, uint32_t dst) {
    if (EMIT == kEmitRecord) {
        emit_record(ep.rp, i, dst);
    } else {
        if (EMIT == kEmitPerm || ep.cp.keep_perm) sperm[dst] = i;
        if (EMIT == kEmitPermColumns) emit_columns(ep.cp, i, dst);
    }
}

// Messages lo .. lo + len - 1 written at s .. s + len - 1 (a bin whose
// original indices are already in order) by threads t, t + nt, ... of the
// caller. Records of up to 8 words go four messages per thread at a time,
// every load issued before any store, so each thread keeps four messages'
// loads in flight instead of one.
template <int EMIT>
__device__ __forceinline__ void emit_run(const EmitParams& ep, uint32_t* sperm, uint32_t lo, uint32_t s,
                                         uint32_t len, uint32_t t, uint32_t nt) {
    if (EMIT == kEmitRecord && ep.rp.rec.words <= 8) {
        const fg_record_desc& rec = ep.rp.rec;
        const uint32_t words = rec.words;  // 4 or 8: records are 16-byte aligned
        for (uint32_t k0 = t; k0 < len; k0 += 4 * nt) {
            uint32_t v[4][8];
#pragma unroll
            for (uint32_t m = 0; m < 4; ++m) {
                const uint32_t k = k0 + m * nt;
#pragma unroll
                for (uint32_t w = 0; w < 8; ++w) {
                    const uint32_t* src = w < words ? rec.src[w] : nullptr;
                    v[m][w] = (k < len && src)
                                  ? ld_nc_u32(src + static_cast<size_t>(lo + k) * rec.src_stride[w] + rec.src_word[w])
                                  : 0u;
                }
            }
#pragma unroll
            for (uint32_t m = 0; m < 4; ++m) {
                const uint32_t k = k0 + m * nt;
                if (k < len) {
                    uint4* o = reinterpret_cast<uint4*>(ep.rp.out + static_cast<size_t>(s + k) * words);
                    o[0] = make_uint4(v[m][0], v[m][1], v[m][2], v[m][3]);
                    if (words > 4) o[1] = make_uint4(v[m][4], v[m][5], v[m][6], v[m][7]);
                }
            }
        }
        return;
    }
    if constexpr (EMIT == kEmitPermColumns) {
        // every column a straight copy of [lo, lo + len) to [s, s + len); runs of
        // four 4-byte columns go four rows at a time (16 loads before any store)
        const ColumnParams& cp = ep.cp;
        if (cp.keep_perm)
            for (uint32_t k = t; k < len; k += nt) sperm[s + k] = lo + k;
        for (uint32_t c0 = 0; c0 < cp.ncols; c0 += 4) {
            const uint32_t nk = min(4u, cp.ncols - c0);
            bool words = true;
            for (uint32_t c = 0; c < nk; ++c) words = words && cp.col[c0 + c].elem_bytes == 4u;
            if (!words) {
                for (uint32_t c = 0; c < nk; ++c)
                    for (uint32_t k = t; k < len; k += nt) copy_column_elem(cp.col[c0 + c], lo + k, s + k);
                continue;
            }
            for (uint32_t k0 = t; k0 < len; k0 += 4 * nt) {
                uint32_t v[4][4];
#pragma unroll
                for (uint32_t c = 0; c < 4; ++c)
#pragma unroll
                    for (uint32_t m = 0; m < 4; ++m) {
                        const uint32_t k = k0 + m * nt;
                        v[c][m] = (c < nk && k < len) ? static_cast<const uint32_t*>(cp.col[c0 + c].in)[lo + k] : 0u;
                    }
#pragma unroll
                for (uint32_t c = 0; c < 4; ++c)
#pragma unroll
                    for (uint32_t m = 0; m < 4; ++m) {
                        const uint32_t k = k0 + m * nt;
                        if (c < nk && k < len) static_cast<uint32_t*>(cp.col[c0 + c].out)[s + k] = v[c][m];
                    }
            }
        }
    } else {
        for (uint32_t k = t; k < len; k += nt) emit<EMIT>(ep, sperm, lo + k, s + k);
    }
}

// What the stabilising and long-bin kernels of one counting sort read and
// write: the emission, the keys, PBM and unstable placement, the stable
// permutation (agent sorts), the long-bin chunk queue, the workspace header,
// and for agent sorts the recorded largest key (key_max) and its floor.
struct StabJob {
    EmitParams rp;
    uint32_t nbuckets;
    const uint32_t* keys;
    const uint32_t* pbm;
    const uint32_t* perm;
    uint32_t* sperm;
    uint2* chunk_list;
    uint32_t chunk_cap;
    WsHeader* h;
    uint32_t* key_max;
    uint32_t key_floor;
    uint32_t max_n;
};

// Sorted positions p < total = pbm[nbuckets] (for an agent sort, whose scan
// stopped past max(recorded key, cells - 1), the PBM entry after that). Short bins are ranked in place
// (count of smaller original indices in the bin); long bins are queued as
// chunks (bucket, chunk index) for k_long.
template <int EMIT>
__device__ __forceinline__ void stabilize_positions(const StabJob& j, uint32_t blk, uint32_t nblk) {
    // key_max (agent sorts): the PBM ends at max(recorded key, key_floor) + 1
    const uint32_t total = j.pbm[j.key_max ? min(j.nbuckets, max(*j.key_max, j.key_floor) + 1u) : j.nbuckets];
    if (j.h->disorder == 0u) {
        // keys in row order (the key launch and the scan found no descent):
        // the stable order is the row order, so rows are emitted in place, as
        // one run over the grid's threads (four rows in flight per thread)
        emit_run<EMIT>(j.rp, j.sperm, 0u, 0u, min(total, j.max_n), blk * blockDim.x + threadIdx.x, nblk * blockDim.x);
        return;
    }
    for (uint32_t p = blk * blockDim.x + threadIdx.x; p < total; p += nblk * blockDim.x) {
        const uint32_t i = j.perm[p];
        const uint32_t b = j.keys[i];
        if (b & kPadBit) {  // padding row of a batch: keeps its slot, carries no message
            if (EMIT != kEmitRecord) j.sperm[p] = i;
            continue;
        }
        const uint32_t s = j.pbm[b], e = j.pbm[b + 1];
        // a PBM from a scan whose look-back gave up (FG_ERR_DEVICE_TIMEOUT
        // recorded) may run backwards: such a bin is skipped, so no bin is
        // queued or ranked past the messages (entries never exceed their count)
        if (e < s) continue;
        const uint32_t len = e - s;
        if (len > kShortBin) {
            if (p == s) {
                const uint32_t nch = (len + kChunk - 1) / kChunk;
                const uint32_t at = atomicAdd(&j.h->long_count, nch);
                for (uint32_t c = 0; c < nch; ++c)
                    if (at + c < j.chunk_cap) j.chunk_list[at + c] = make_uint2(b, c);
                if (at + nch > j.chunk_cap) record_status(j.h, FG_ERR_CAPACITY);
            }
            continue;
        }
        uint32_t dst = s;
        if (len > 1) {
            for (uint32_t q = s; q < e; ++q) dst += (j.perm[q] < i) ? 1u : 0u;
        }
        emit<EMIT>(j.rp, j.sperm, i, dst);
    }
}

template <int EMIT>
__global__ void __launch_bounds__(kThreads) k_stabilize(const __grid_constant__ StabJob j) {
    flamegpu::detail::grid_dependency_enter();
    stabilize_positions<EMIT>(j, blockIdx.x, gridDim.x);
}

// an agent sort's stable positions (EA, the first ga blocks) and a message
// build's (EB, the rest), in one launch
template <int EA, int EB>
__global__ void __launch_bounds__(kThreads) k_stabilize_pair(const __grid_constant__ StabJob a,
                                                             const __grid_constant__ StabJob b, uint32_t ga) {
    flamegpu::detail::grid_dependency_enter();
    if (blockIdx.x < ga)
        stabilize_positions<EA>(a, blockIdx.x, ga);
    else
        stabilize_positions<EB>(b, blockIdx.x - ga, gridDim.x - ga);
}

// Long bins. A bin of up to kSortCap messages is ordered by one block (the
// bin's chunk 0; its other chunks are skipped). When its original indices are
// distinct values filling [min, max] (messages of agents in bin order), the
// k-th smallest is min + k and they are copied in that order, without ranking.
// Otherwise, when its original indices
// span at most kSpanCap values (messages that arrive nearly in bin order, as
// those of spatially sorted agents do), each index sets one bit of a bitmap
// over that span and its rank is the number of set bits before it: O(length
// + span / 32). Otherwise the indices (distinct) are sorted ascending in
// shared memory with a bitonic network (Batcher 1968), padded to a power of
// two. Longer bins rank every element against the whole bin, chunk by chunk.
constexpr uint32_t kSortCap = 8192;
constexpr uint32_t kSpanWords = kSortCap / 2;   // bitmap words; the other half holds their prefix counts
constexpr uint32_t kSpanCap = kSpanWords * 32;  // 131,072 indices
// Bins of up to kWarpBin messages (most long bins of clustered inputs) are
// ordered first, one warp each and without block barriers: a bitmap over
// their indices when those span at most kWarpSpanWords * 32 values, else a
// bitonic sort of the indices in the warp's slice of shared memory. The block
// pass then takes the longer ones.
constexpr uint32_t kWarpBin = 1024;
constexpr uint32_t kWarpSpanWords = 128;
static_assert((kThreads / 32) * kWarpBin <= kSortCap, "a warp's bitonic slice lies in s_idx");

// Shared memory of the long-bin pass.
struct LongSmem {
    uint32_t idx[kSortCap];
    uint32_t warp[33];
    uint32_t lo, hi;
    uint32_t wbits[kThreads / 32][kWarpSpanWords];
    uint32_t wpre[kThreads / 32][kWarpSpanWords];
};

template <int EMIT>
__device__ __forceinline__ void long_bins(const StabJob& job, LongSmem& sm, uint32_t blk, uint32_t nblk) {
    const EmitParams& rp = job.rp;
    const uint32_t* __restrict__ pbm = job.pbm;
    const uint32_t* __restrict__ perm = job.perm;
    uint32_t* sperm = job.sperm;
    const uint2* __restrict__ chunk_list = job.chunk_list;
    uint32_t* s_idx = sm.idx;
    uint32_t* s_warp = sm.warp;
    uint32_t& s_lo = sm.lo;
    uint32_t& s_hi = sm.hi;
    const uint32_t nchunks = min(job.h->long_count, job.chunk_cap);
    // warp pass: bins of up to kWarpBin messages
    {
        const uint32_t lane = threadIdx.x & 31u, wib = threadIdx.x >> 5;
        uint32_t* bits = sm.wbits[wib];
        uint32_t* pre = sm.wpre[wib];
        for (uint32_t c = blk * (kThreads / 32) + wib; c < nchunks; c += nblk * (kThreads / 32)) {
            const uint2 ch = chunk_list[c];
            const uint32_t s = pbm[ch.x], e = pbm[ch.x + 1];
            const uint32_t len = e - s;
            if (len > kWarpBin || ch.y != 0) continue;  // the same for every lane
            uint32_t lo = 0xFFFFFFFFu, hi = 0u;
            for (uint32_t k = lane; k < len; k += 32u) {
                const uint32_t i = perm[s + k];
                lo = min(lo, i);
                hi = max(hi, i);
            }
            lo = __reduce_min_sync(0xFFFFFFFFu, lo);
            hi = __reduce_max_sync(0xFFFFFFFFu, hi);
            if (hi - lo == len - 1u) {  // distinct indices filling [lo, hi]: already ascending from lo
                emit_run<EMIT>(rp, sperm, lo, s, len, lane, 32u);
            } else if (hi - lo < kWarpSpanWords * 32u) {
                const uint32_t words = (hi - lo) / 32u + 1u;
                for (uint32_t w = lane; w < words; w += 32u) bits[w] = 0u;
                __syncwarp();
                for (uint32_t k = lane; k < len; k += 32u) {
                    const uint32_t d = perm[s + k] - lo;
                    atomicOr(&bits[d >> 5], 1u << (d & 31u));
                }
                __syncwarp();
                // set bits before each word: lane l sums words 4l..4l+3, a warp scan offsets them
                uint32_t cnt[4], sum = 0;
#pragma unroll
                for (uint32_t j = 0; j < 4; ++j) {
                    const uint32_t w = lane * 4u + j;
                    cnt[j] = w < words ? __popc(bits[w]) : 0u;
                    sum += cnt[j];
                }
                uint32_t inc = sum;
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, inc, d);
                    if (lane >= static_cast<uint32_t>(d)) inc += t;
                }
                uint32_t ex = inc - sum;
#pragma unroll
                for (uint32_t j = 0; j < 4; ++j) {
                    const uint32_t w = lane * 4u + j;
                    if (w < words) pre[w] = ex;
                    ex += cnt[j];
                }
                __syncwarp();
                for (uint32_t k = lane; k < len; k += 32u) {
                    const uint32_t i = perm[s + k];
                    const uint32_t d = i - lo;
                    emit<EMIT>(rp, sperm, i, s + pre[d >> 5] + __popc(bits[d >> 5] & ((1u << (d & 31u)) - 1u)));
                }
                __syncwarp();  // bits and pre are reused by the warp's next bin
            } else {
                // indices spread wider: bitonic sort in the warp's slice of s_idx
                // (the block pass below writes s_idx only after a block barrier)
                uint32_t* w = s_idx + wib * kWarpBin;
                uint32_t p2 = 32;
                while (p2 < len) p2 <<= 1;
                for (uint32_t k = lane; k < p2; k += 32u) w[k] = k < len ? perm[s + k] : 0xFFFFFFFFu;
                __syncwarp();
                for (uint32_t k = 2; k <= p2; k <<= 1) {
                    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
                        for (uint32_t t = lane; t < p2; t += 32u) {
                            const uint32_t u = t ^ j;
                            if (u > t) {
                                const uint32_t a = w[t], b = w[u];
                                if (((t & k) == 0) == (a > b)) {
                                    w[t] = b;
                                    w[u] = a;
                                }
                            }
                        }
                        __syncwarp();
                    }
                }
                for (uint32_t k = lane; k < len; k += 32u) emit<EMIT>(rp, sperm, w[k], s + k);
                __syncwarp();  // w is reused by the warp's next bin
            }
        }
    }
    // block pass: longer bins
    for (uint32_t c = blk; c < nchunks; c += nblk) {
        const uint2 ch = chunk_list[c];
        const uint32_t s = pbm[ch.x], e = pbm[ch.x + 1];
        const uint32_t len = e - s;
        if (len <= kWarpBin) continue;  // done by the warp pass
        if (len <= kSortCap) {
            if (ch.y != 0) continue;  // the bin's chunk 0 orders the whole bin
            // span of the bin's original indices
            uint32_t lo = 0xFFFFFFFFu, hi = 0u;
            for (uint32_t k = threadIdx.x; k < len; k += blockDim.x) {
                const uint32_t i = perm[s + k];
                lo = min(lo, i);
                hi = max(hi, i);
            }
            lo = __reduce_min_sync(0xFFFFFFFFu, lo);
            hi = __reduce_max_sync(0xFFFFFFFFu, hi);
            __syncthreads();  // the previous bin is done with shared memory
            if (threadIdx.x == 0) {
                s_lo = 0xFFFFFFFFu;
                s_hi = 0u;
            }
            __syncthreads();
            if ((threadIdx.x & 31u) == 0) {
                atomicMin(&s_lo, lo);
                atomicMax(&s_hi, hi);
            }
            __syncthreads();
            lo = s_lo;
            hi = s_hi;
            if (hi - lo == len - 1u) {  // distinct indices filling [lo, hi]: already ascending from lo
                emit_run<EMIT>(rp, sperm, lo, s, len, threadIdx.x, blockDim.x);
                continue;
            }
            if (hi - lo < kSpanCap) {
                const uint32_t words = (hi - lo) / 32u + 1u;
                uint32_t* bits = s_idx;
                uint32_t* before = s_idx + kSpanWords;
                for (uint32_t w = threadIdx.x; w < words; w += blockDim.x) bits[w] = 0u;
                __syncthreads();
                for (uint32_t k = threadIdx.x; k < len; k += blockDim.x) {
                    const uint32_t d = perm[s + k] - lo;
                    atomicOr(&bits[d >> 5], 1u << (d & 31u));
                }
                __syncthreads();
                // set bits before each word: each thread sums a run of words,
                // a block scan offsets the runs
                const uint32_t per = (words + blockDim.x - 1) / blockDim.x;
                const uint32_t w0 = threadIdx.x * per;
                uint32_t run = 0;
                for (uint32_t w = w0; w < min(w0 + per, words); ++w) run += __popc(bits[w]);
                uint32_t total;
                uint32_t acc = block_exclusive_scan(run, &total, s_warp);
                for (uint32_t w = w0; w < min(w0 + per, words); ++w) {
                    before[w] = acc;
                    acc += __popc(bits[w]);
                }
                __syncthreads();
                for (uint32_t k = threadIdx.x; k < len; k += blockDim.x) {
                    const uint32_t i = perm[s + k];
                    const uint32_t d = i - lo;
                    const uint32_t rank = before[d >> 5] + __popc(bits[d >> 5] & ((1u << (d & 31u)) - 1u));
                    emit<EMIT>(rp, sperm, i, s + rank);
                }
                continue;
            }
            uint32_t p2 = 64;
            while (p2 < len) p2 <<= 1;
            __syncthreads();
            for (uint32_t k = threadIdx.x; k < p2; k += blockDim.x) s_idx[k] = k < len ? perm[s + k] : 0xFFFFFFFFu;
            __syncthreads();
            for (uint32_t k = 2; k <= p2; k <<= 1) {
                for (uint32_t j = k >> 1; j > 0; j >>= 1) {
                    for (uint32_t t = threadIdx.x; t < p2; t += blockDim.x) {
                        const uint32_t u = t ^ j;
                        if (u > t) {
                            const uint32_t a = s_idx[t], b = s_idx[u];
                            if (((t & k) == 0) == (a > b)) {
                                s_idx[t] = b;
                                s_idx[u] = a;
                            }
                        }
                    }
                    __syncthreads();
                }
            }
            for (uint32_t k = threadIdx.x; k < len; k += blockDim.x) emit<EMIT>(rp, sperm, s_idx[k], s + k);
            continue;
        }
        const uint32_t q = s + ch.y * kChunk + threadIdx.x;
        const bool act = q < e;
        const uint32_t i = act ? perm[q] : 0u;
        uint32_t rank = 0;
        for (uint32_t t0 = s; t0 < e; t0 += kRankTile) {
            const uint32_t tn = min(kRankTile, e - t0);
            __syncthreads();
            for (uint32_t k = threadIdx.x; k < tn; k += blockDim.x) s_idx[k] = perm[t0 + k];
            __syncthreads();
            if (act) {
                uint32_t r = 0;
                for (uint32_t k = 0; k < tn; ++k) r += (s_idx[k] < i) ? 1u : 0u;
                rank += r;
            }
        }
        if (act) emit<EMIT>(rp, sperm, i, s + rank);
    }
}

template <int EMIT>
__global__ void __launch_bounds__(kThreads) k_long(const __grid_constant__ StabJob j) {
    flamegpu::detail::grid_dependency_enter();
    // the last kernel of an agent sort: the largest key is no longer read;
    // the last of any build: the order flag is no longer read (the next key
    // launch raises it again where its keys descend)
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (j.key_max) *j.key_max = 0u;
        j.h->disorder = 0u;
    }
    __shared__ LongSmem sm;
    long_bins<EMIT>(j, sm, blockIdx.x, gridDim.x);
}

// an agent sort's long bins (EA) and a message build's (EB), in one launch
template <int EA, int EB>
__global__ void __launch_bounds__(kThreads) k_long_pair(const __grid_constant__ StabJob a,
                                                        const __grid_constant__ StabJob b, uint32_t ga) {
    flamegpu::detail::grid_dependency_enter();
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (a.key_max) *a.key_max = 0u;
        a.h->disorder = 0u;
        if (b.key_max) *b.key_max = 0u;
        b.h->disorder = 0u;
    }
    __shared__ LongSmem sm;
    // the first ga blocks take a's long bins, the rest b's
    if (blockIdx.x < ga)
        long_bins<EA>(a, sm, blockIdx.x, ga);
    else
        long_bins<EB>(b, sm, blockIdx.x - ga, gridDim.x - ga);
}

// ------------------------------------------------------------------- host side

struct BuildLayout {
    size_t hist, scan_status, keys, slot, perm, sperm, chunks, pbm, edges, total;
    uint32_t chunk_cap;
};

static BuildLayout build_layout(uint32_t max_n, uint32_t nbuckets, bool sort_mode) {
    BuildLayout L{};
    size_t off = sizeof(WsHeader);
    auto take = [&](size_t bytes) {
        const size_t at = off;
        off = align_up(off + bytes, 256);
        return at;
    };
    // The scan statuses and the (kept-zero) histogram come first: their
    // offsets depend only on the bucket count, so a workspace stays valid when
    // max_n changes as long as the grid does not.
    const uint32_t scan_n = nbuckets + 1;
    L.scan_status = take(sizeof(uint64_t) * (scan_tiles(scan_n) + 1));
    L.hist = take(sizeof(uint32_t) * (static_cast<size_t>(scan_n) + 4));
    L.keys = take(sizeof(uint32_t) * (static_cast<size_t>(max_n) + 1));
    L.slot = take(sizeof(uint32_t) * (static_cast<size_t>(max_n) + 1));
    L.perm = take(sizeof(uint32_t) * (static_cast<size_t>(max_n) + 1));
    L.chunk_cap = max_n / (kShortBin + 1) + max_n / kChunk + 16;
    L.chunks = take(sizeof(uint2) * L.chunk_cap);
    L.edges = take(sizeof(uint32_t) * 2 * (static_cast<size_t>(max_n) / 32 + 1));
    if (sort_mode) {
        L.sperm = take(sizeof(uint32_t) * (static_cast<size_t>(max_n) + 1));
        L.pbm = take(sizeof(uint32_t) * (static_cast<size_t>(scan_n) + 4));
    }
    L.total = off;
    return L;
}

}  // namespace fgk

using namespace fgk;

namespace {

thread_local int g_last_cuda_error = 0;

int sm_count() {
    static int cached[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) dev = 0;
    if (!cached[dev]) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        cached[dev] = v > 0 ? v : 132;
    }
    return cached[dev];
}

uint32_t grid_for(uint32_t max_n, int per_sm = 8) {
    const uint32_t need = (max_n + kThreads - 1) / kThreads;
    const uint32_t cap = static_cast<uint32_t>(sm_count() * per_sm);
    return std::max(1u, std::min(need, cap));
}

// a long bin has more than 32 rows and a chunk 256: one block per 128 rows
// covers every chunk of a small list at once; large lists get 4 per SM
uint32_t long_grid_for(uint32_t max_n) {
    return std::max(1u, std::min((max_n + 127u) / 128u, static_cast<uint32_t>(sm_count() * 4)));
}

int check_launch() {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        g_last_cuda_error = static_cast<int>(e);
        return FG_ERR_CUDA;
    }
    return FG_OK;
}

bool sort_grid_from(const fg_spatial_grid* g, SortGrid* s, uint32_t* nbuckets) {
    // CUDASimulation.cu:494-507 and :569-571
    uint64_t prod = 1;
    for (int a = 0; a < 3; ++a) {
        const float w = a < g->dims ? (g->max[a] - g->min[a]) : 0.0f;
        s->min[a] = a < g->dims ? g->min[a] : 0.0f;
        s->width[a] = w;
        s->gd[a] = w != 0.0f ? static_cast<uint32_t>(ceilf(w / g->radius)) : 1u;
        s->gd_f[a] = static_cast<float>(s->gd[a]);
        prod *= s->gd[a];
    }
    const int bits = static_cast<int>(std::floor(std::log2(static_cast<double>(static_cast<uint32_t>(prod))))) + 1;
    if (bits > 30 || prod == 0) return false;
    s->mask = (1u << bits) - 1u;
    *nbuckets = 1u << bits;
    return true;
}

}  // namespace

extern "C" int fg_last_cuda_error(void) { return g_last_cuda_error; }



extern "C" int fg_spatial_grid_init(fg_spatial_grid* g, int32_t dims, const float* mn, const float* mx, float radius) {
    // MessageSpatial3D::CUDAModelHandler::CUDAModelHandler (MessageSpatial3D.cu:31-52)
    if (!g || !mn || !mx || (dims != 2 && dims != 3) || !(radius > 0.0f)) return FG_ERR_INVALID_ARGUMENT;
    *g = fg_spatial_grid{};
    g->dims = dims;
    g->radius = radius;
    g->binCount = 1;
    g->wrapCompatible = 1;
    uint64_t prod = 1;
    for (int a = 0; a < 3; ++a) {
        if (a < dims) {
            if (!(mx[a] > mn[a])) return FG_ERR_INVALID_ARGUMENT;
            g->min[a] = mn[a];
            g->max[a] = mx[a];
            g->width[a] = g->max[a] - g->min[a];
            g->gridDim[a] = static_cast<uint32_t>(std::ceil(g->width[a] / g->radius));
            prod *= g->gridDim[a];
            // numeric::approxExactlyDivisible<float> (include/flamegpu/detail/numeric.h:24-31)
            const float x = g->width[a], y = g->radius;
            const float eps = std::max(std::fabs(x), std::fabs(y)) * 1.1920929e-07f;
            const float v = std::fmod(x, y);
            g->wrapCompatible = g->wrapCompatible && (v <= eps || v > y - eps);
        } else {
            g->gridDim[a] = 1;
        }
    }
    if (prod >= 0xFFFFFFF0ull) return FG_ERR_INVALID_ARGUMENT;
    g->binCount = static_cast<uint32_t>(prod);
    return FG_OK;
}

extern "C" size_t fg_spatial_build_workspace_size(uint32_t max_n, uint32_t bin_count) {
    return build_layout(max_n, bin_count, false).total;
}

extern "C" size_t fg_spatial_sort_workspace_size(uint32_t max_n, const fg_spatial_grid* g) {
    SortGrid sg{};
    uint32_t nb = 0;
    if (!g || !sort_grid_from(g, &sg, &nb)) return 0;
    return build_layout(max_n, nb, true).total;
}

namespace {

struct BatchKeys {
    const fg_batch_instance* inst = nullptr;  // null: single list
    const uint32_t* counts = nullptr;
    uint32_t ninst = 0;
    int dims = 3;
};

template <int MODE, int EMIT>
int run_pipeline(const fg_spatial_grid* g, const SortGrid& sg, uint32_t nbuckets, uint32_t max_n, const uint32_t* d_n,
                 const float* x, const float* y, const float* z, const uint32_t* valid, const EmitParams& rp,
                 uint32_t* pbm_out, const BuildLayout& L, char* ws, cudaStream_t st, const BatchKeys& batch = BatchKeys(),
                 bool keys_ready = false, uint32_t pos_stride = 1) {
    WsHeader* h = reinterpret_cast<WsHeader*>(ws);
    uint32_t* hist = reinterpret_cast<uint32_t*>(ws + L.hist);
    uint64_t* sstat = reinterpret_cast<uint64_t*>(ws + L.scan_status);
    uint32_t* keys = reinterpret_cast<uint32_t*>(ws + L.keys);
    uint32_t* slot = reinterpret_cast<uint32_t*>(ws + L.slot);
    uint32_t* perm = reinterpret_cast<uint32_t*>(ws + L.perm);
    uint32_t* sperm = EMIT != kEmitRecord ? reinterpret_cast<uint32_t*>(ws + L.sperm) : nullptr;
    uint2* chunks = reinterpret_cast<uint2*>(ws + L.chunks);
    uint32_t* edges = reinterpret_cast<uint32_t*>(ws + L.edges);
    const uint32_t grid = grid_for(max_n);
    if (keys_ready) {
        // the launch before wrote keys, slots and the histogram (key_targets_write)
    } else if (batch.inst) {
        launch(k_bin_batched<MODE>, grid, kThreads, st, batch.inst, batch.counts, batch.ninst, max_n, batch.dims, x, y, z,
               valid, keys, slot, hist, h);
    } else {
        launch(k_bin<MODE>, grid, kThreads, st, *g, sg, max_n, d_n, x, y, z, valid, keys, slot, hist, h, pos_stride,
               edges);
    }
    const uint32_t scan_n = nbuckets + 1;
    // an agent sort's buckets (2^bits) run past the grid's cells: its scan stops
    // past the cells, or past the largest key beyond them that the key kernel
    // (or launch) recorded
    uint32_t* key_max = (MODE == kSortKey && !batch.inst) ? &h->key_max : nullptr;
    const uint32_t key_floor = flamegpu::detail::sort_cells(sg) - 1u;
    // the scan also compares the keys of rows 32w - 1 and 32w (row order; a batch's keys are never in it)
    const OrderCheck oc{batch.inst ? nullptr : edges, d_n, max_n};
    launch_scan(hist, pbm_out, scan_n, 1, sstat, h, 0, st, key_max, key_floor, oc);
    launch(k_perm, grid, kThreads, st, PermJob{max_n, d_n, keys, slot, pbm_out, perm, h});
    const StabJob sj{rp, nbuckets, keys, pbm_out, perm, sperm, chunks, L.chunk_cap, h, key_max, key_floor, max_n};
    launch(k_stabilize<EMIT>, grid, kThreads, st, sj);
    launch(k_long<EMIT>, long_grid_for(max_n), kThreads, st, sj);
    return check_launch();
}

}  // namespace

int fgi_spatial_build(const fg_spatial_grid* g, uint32_t max_n, const uint32_t* d_n, const float* x, const float* y,
                      const float* z, const uint32_t* valid, const fg_record_desc* rec, uint32_t* sorted, uint32_t* pbm,
                      void* workspace, size_t workspace_bytes, void* stream, bool keys_ready) {
    if (!g || !rec || !pbm || !workspace || (g->dims != 2 && g->dims != 3)) return FG_ERR_INVALID_ARGUMENT;
    if (rec->words == 0 || (rec->words & 3) || rec->words > FG_MAX_RECORD_WORDS) return FG_ERR_INVALID_ARGUMENT;
    if (max_n && (!x || !y || (g->dims == 3 && !z) || !sorted)) return FG_ERR_INVALID_ARGUMENT;
    if (reinterpret_cast<uintptr_t>(sorted) & 15) return FG_ERR_INVALID_ARGUMENT;
    const BuildLayout L = build_layout(max_n, g->binCount, false);
    if (workspace_bytes < L.total || (reinterpret_cast<uintptr_t>(workspace) & 255)) return FG_ERR_WORKSPACE;
    EmitParams rp{};
    rp.rp.rec = *rec;
    rp.rp.out = sorted;
    SortGrid sg{};
    return run_pipeline<kMessageBin, kEmitRecord>(g, sg, g->binCount, max_n, d_n, x, y, z, valid, rp, pbm, L,
                                                  static_cast<char*>(workspace), static_cast<cudaStream_t>(stream),
                                                  BatchKeys(), keys_ready);
}

extern "C" int fg_spatial_build(const fg_spatial_grid* g, uint32_t max_n, const uint32_t* d_n, const float* x,
                                const float* y, const float* z, const uint32_t* valid, const fg_record_desc* rec,
                                uint32_t* sorted, uint32_t* pbm, void* workspace, size_t workspace_bytes,
                                void* stream) {
    return fgi_spatial_build(g, max_n, d_n, x, y, z, valid, rec, sorted, pbm, workspace, workspace_bytes, stream, false);
}

int fgi_spatial_sort_agents(const fg_spatial_grid* g, uint32_t max_n, const uint32_t* d_n, const float* x,
                            const float* y, const float* z, const fg_column* cols, uint32_t ncols, uint32_t* perm_out,
                            void* workspace, size_t workspace_bytes, void* stream, bool keys_ready,
                            uint32_t pos_stride) {
    if (pos_stride < 1 || pos_stride > 3 || (keys_ready && pos_stride != 1)) return FG_ERR_INVALID_ARGUMENT;
    if (!g || !workspace || (g->dims != 2 && g->dims != 3) || ncols > FG_MAX_COLUMNS) return FG_ERR_INVALID_ARGUMENT;
    if (max_n && (!x || !y || (g->dims == 3 && !z))) return FG_ERR_INVALID_ARGUMENT;
    if (ncols && !cols) return FG_ERR_INVALID_ARGUMENT;
    SortGrid sg{};
    uint32_t nb = 0;
    if (!sort_grid_from(g, &sg, &nb)) return FG_ERR_UNSUPPORTED;
    const BuildLayout L = build_layout(max_n, nb, true);
    if (workspace_bytes < L.total || (reinterpret_cast<uintptr_t>(workspace) & 255)) return FG_ERR_WORKSPACE;
    char* ws = static_cast<char*>(workspace);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // the stable positions' kernels write every column directly (no gather pass)
    EmitParams rp{};
    for (uint32_t c = 0; c < ncols; ++c) rp.cp.col[c] = cols[c];
    rp.cp.ncols = ncols;
    rp.cp.keep_perm = perm_out != nullptr;
    int rc = ncols ? run_pipeline<kSortKey, kEmitPermColumns>(g, sg, nb, max_n, d_n, x, y, z, nullptr, rp,
                                                              reinterpret_cast<uint32_t*>(ws + L.pbm), L, ws, st,
                                                              BatchKeys(), keys_ready, pos_stride)
                   : run_pipeline<kSortKey, kEmitPerm>(g, sg, nb, max_n, d_n, x, y, z, nullptr, rp,
                                                       reinterpret_cast<uint32_t*>(ws + L.pbm), L, ws, st,
                                                       BatchKeys(), keys_ready, pos_stride);
    if (rc != FG_OK) return rc;
    const uint32_t* sperm = reinterpret_cast<const uint32_t*>(ws + L.sperm);
    if (perm_out && max_n) {
        cudaMemcpyAsync(perm_out, sperm, sizeof(uint32_t) * max_n, cudaMemcpyDeviceToDevice, st);
    }
    return check_launch();
}

// The automatic agent sort of a list and the index build of the spatial
// messages it output, both on the message list's grid, as one pipeline of
// paired launches (scan, placement, stable positions, long bins, each doing
// both sorts): one chain of four kernels instead of two concurrent chains
// joined before the function that reads the messages. The launch before
// wrote both key sets (keys_ready for both). Results are those of
// fgi_spatial_sort_agents and fgi_spatial_build run one after the other.
int fgi_spatial_sort_and_build(const fg_spatial_grid* g, uint32_t sort_max_n, const uint32_t* sort_d_n,
                               const fg_column* cols, uint32_t ncols, void* sort_ws, size_t sort_ws_bytes,
                               uint32_t msg_max_n, const uint32_t* msg_d_n, const fg_record_desc* rec,
                               uint32_t* sorted, uint32_t* pbm, void* build_ws, size_t build_ws_bytes, void* stream) {
    if (!g || (g->dims != 2 && g->dims != 3) || !cols || ncols == 0 || ncols > FG_MAX_COLUMNS) return FG_ERR_INVALID_ARGUMENT;
    if (!rec || !pbm || !sort_ws || !build_ws) return FG_ERR_INVALID_ARGUMENT;
    if (rec->words == 0 || (rec->words & 3) || rec->words > FG_MAX_RECORD_WORDS) return FG_ERR_INVALID_ARGUMENT;
    if ((msg_max_n && !sorted) || (reinterpret_cast<uintptr_t>(sorted) & 15)) return FG_ERR_INVALID_ARGUMENT;
    SortGrid sg{};
    uint32_t nb = 0;
    if (!sort_grid_from(g, &sg, &nb)) return FG_ERR_UNSUPPORTED;
    const BuildLayout La = build_layout(sort_max_n, nb, true);
    const BuildLayout Lb = build_layout(msg_max_n, g->binCount, false);
    if (sort_ws_bytes < La.total || (reinterpret_cast<uintptr_t>(sort_ws) & 255)) return FG_ERR_WORKSPACE;
    if (build_ws_bytes < Lb.total || (reinterpret_cast<uintptr_t>(build_ws) & 255)) return FG_ERR_WORKSPACE;
    char* wa = static_cast<char*>(sort_ws);
    char* wb = static_cast<char*>(build_ws);
    WsHeader* ha = reinterpret_cast<WsHeader*>(wa);
    WsHeader* hb = reinterpret_cast<WsHeader*>(wb);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    auto at = [](char* w, size_t off) { return reinterpret_cast<uint32_t*>(w + off); };
    EmitParams ea{};
    for (uint32_t c = 0; c < ncols; ++c) ea.cp.col[c] = cols[c];
    ea.cp.ncols = ncols;
    ea.cp.keep_perm = 0;
    EmitParams eb{};
    eb.rp.rec = *rec;
    eb.rp.out = sorted;
    uint32_t* pbm_a = at(wa, La.pbm);
    const uint32_t key_floor = flamegpu::detail::sort_cells(sg) - 1u;
    const ScanJob sa{at(wa, La.hist), pbm_a, nb + 1, 1, reinterpret_cast<uint64_t*>(wa + La.scan_status), ha,
                     &ha->key_max, key_floor, OrderCheck{at(wa, La.edges), sort_d_n, sort_max_n}};
    const ScanJob sb{at(wb, Lb.hist), pbm, g->binCount + 1, 1, reinterpret_cast<uint64_t*>(wb + Lb.scan_status), hb,
                     nullptr, 0, OrderCheck{at(wb, Lb.edges), msg_d_n, msg_max_n}};
    launch_scan_pair(sa, sb, st);
    // each launch gives each sort the blocks its own kernel would have
    const uint32_t ga = grid_for(sort_max_n), gb = grid_for(msg_max_n);
    launch(k_perm_pair, ga + gb, kThreads, st, PermJob{sort_max_n, sort_d_n, at(wa, La.keys), at(wa, La.slot), pbm_a,
                                                       at(wa, La.perm), ha},
           PermJob{msg_max_n, msg_d_n, at(wb, Lb.keys), at(wb, Lb.slot), pbm, at(wb, Lb.perm), hb}, ga);
    const StabJob ja{ea, nb, at(wa, La.keys), pbm_a, at(wa, La.perm), at(wa, La.sperm),
                     reinterpret_cast<uint2*>(wa + La.chunks), La.chunk_cap, ha, &ha->key_max, key_floor, sort_max_n};
    const StabJob jb{eb, g->binCount, at(wb, Lb.keys), pbm, at(wb, Lb.perm), nullptr,
                     reinterpret_cast<uint2*>(wb + Lb.chunks), Lb.chunk_cap, hb, nullptr, 0, msg_max_n};
    launch(k_stabilize_pair<kEmitPermColumns, kEmitRecord>, ga + gb, kThreads, st, ja, jb, ga);
    const uint32_t la = long_grid_for(sort_max_n), lb = long_grid_for(msg_max_n);
    launch(k_long_pair<kEmitPermColumns, kEmitRecord>, la + lb, kThreads, st, ja, jb, la);
    return check_launch();
}

extern "C" int fg_spatial_sort_agents(const fg_spatial_grid* g, uint32_t max_n, const uint32_t* d_n, const float* x,
                                      const float* y, const float* z, const fg_column* cols, uint32_t ncols,
                                      uint32_t* perm_out, void* workspace, size_t workspace_bytes, void* stream) {
    return fgi_spatial_sort_agents(g, max_n, d_n, x, y, z, cols, ncols, perm_out, workspace, workspace_bytes, stream,
                                   false, 1);
}

// Where a launch computing the keys of a build (sort_mode false) or an agent
// sort (true) on this workspace writes them; the sort's grid for its keys.
int fgi_key_target(const fg_spatial_grid* g, uint32_t max_n, bool sort_mode, void* workspace, size_t workspace_bytes,
                   flamegpu::detail::KeyTarget* t) {
    if (!g || !workspace || !t || (g->dims != 2 && g->dims != 3)) return FG_ERR_INVALID_ARGUMENT;
    std::memset(t, 0, sizeof(*t));
    uint32_t nb = g->binCount;
    if (sort_mode && !sort_grid_from(g, &t->sort, &nb)) return FG_ERR_UNSUPPORTED;
    const BuildLayout L = build_layout(max_n, nb, sort_mode);
    if (workspace_bytes < L.total || (reinterpret_cast<uintptr_t>(workspace) & 255)) return FG_ERR_WORKSPACE;
    char* ws = static_cast<char*>(workspace);
    t->mode = sort_mode ? flamegpu::detail::kKeySortKey : flamegpu::detail::kKeyMessageBin;
    t->dims = static_cast<uint32_t>(g->dims);
    t->grid = *g;
    t->keys = reinterpret_cast<uint32_t*>(ws + L.keys);
    t->slot = reinterpret_cast<uint32_t*>(ws + L.slot);
    t->hist = reinterpret_cast<uint32_t*>(ws + L.hist);
    t->header = reinterpret_cast<uint32_t*>(ws);
    t->edges = reinterpret_cast<uint32_t*>(ws + L.edges);
    return FG_OK;
}

extern "C" size_t fg_scan_workspace_size(uint32_t n) {
    return sizeof(WsHeader) + align_up(sizeof(uint64_t) * (scan_tiles(n) + 1), 256);
}

extern "C" int fg_exclusive_scan_u32(const uint32_t* in, uint32_t* out, uint32_t n, void* workspace,
                                     size_t workspace_bytes, void* stream) {
    if (!workspace || (n && (!in || !out))) return FG_ERR_INVALID_ARGUMENT;
    if (workspace_bytes < fg_scan_workspace_size(n) || (reinterpret_cast<uintptr_t>(workspace) & 255))
        return FG_ERR_WORKSPACE;
    if (!n) return FG_OK;
    char* ws = static_cast<char*>(workspace);
    launch_scan(in, out, n, 0, reinterpret_cast<uint64_t*>(ws + sizeof(WsHeader)), reinterpret_cast<WsHeader*>(ws), 1,
                static_cast<cudaStream_t>(stream));
    return check_launch();
}

// ------------------------------------------------- allocation-free scan

namespace {

// Header plus one 8-byte status per 4096-value tile (and one spare), rounded to
// 256 bytes: the layout fg_scan_workspace_size() describes, at the largest n.
constexpr size_t kNoAllocScanBytes =
    sizeof(WsHeader) +
    (sizeof(uint64_t) * ((FG_NOALLOC_SCAN_MAX_N + kScanTile - 1) / kScanTile + 1) + 255) / 256 * 256;
static_assert(kNoAllocScanBytes == 66048, "scratch size quoted in fg_capi.h");

}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scan_scratch[kNoAllocScanBytes];

namespace {

// Set-up state of one device's scratch. Only a successful set-up is kept: a
// failed one (e.g. while another thread holds a global-mode stream capture)
// is tried again by the next call. The cached address assumes the device's
// context lives as long as the process (cudaDeviceReset is not supported).
struct NoAllocScratch {
    std::mutex mu;
    void* ptr = nullptr;
};
NoAllocScratch g_noalloc_scratch[64];

// The scratch of the current device; set up by the first call on that device.
int noalloc_scratch(char** out) {
    int dev = 0;
    const cudaError_t de = cudaGetDevice(&dev);
    if (de != cudaSuccess) {
        g_last_cuda_error = static_cast<int>(de);
        return FG_ERR_CUDA;
    }
    if (dev < 0 || dev >= 64) return FG_ERR_UNSUPPORTED;
    NoAllocScratch& s = g_noalloc_scratch[dev];
    std::lock_guard<std::mutex> lock(s.mu);
    if (!s.ptr) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scan_scratch);
        if (e == cudaSuccess) e = cudaMemset(p, 0, kNoAllocScanBytes);
        if (e == cudaSuccess) e = cudaStreamSynchronize(cudaStreamLegacy);
        if (e != cudaSuccess) {
            g_last_cuda_error = static_cast<int>(e);
            return FG_ERR_CUDA;
        }
        s.ptr = p;
    }
    *out = static_cast<char*>(s.ptr);
    return FG_OK;
}

}  // namespace

extern "C" int fg_exclusive_scan_u32_noalloc(const uint32_t* in, uint32_t* out, uint32_t n, void* stream) {
    if (n && (!in || !out)) return FG_ERR_INVALID_ARGUMENT;
    if (n > FG_NOALLOC_SCAN_MAX_N) return FG_ERR_WORKSPACE;
    char* ws = nullptr;
    const int rc = noalloc_scratch(&ws);
    if (rc != FG_OK) return rc;
    if (!n) return FG_OK;
    launch_scan(in, out, n, 0, reinterpret_cast<uint64_t*>(ws + sizeof(WsHeader)), reinterpret_cast<WsHeader*>(ws), 1,
                static_cast<cudaStream_t>(stream));
    return check_launch();
}

extern "C" int fg_noalloc_scan_status(void* stream, int32_t clear) {
    char* ws = nullptr;
    const int rc = noalloc_scratch(&ws);
    if (rc != FG_OK) return rc;
    return fg_workspace_status(ws, sizeof(WsHeader), stream, clear);
}

namespace fgk {
__global__ void k_set_wait_limit(WsHeader* h, uint32_t spin_limit, uint32_t withhold) {
    flamegpu::detail::grid_dependency_enter();
    h->spin_limit = spin_limit;
    h->withhold = withhold;
}
}  // namespace fgk

extern "C" int fg_workspace_set_wait_limit(void* workspace, size_t workspace_bytes, uint32_t spin_limit,
                                           int32_t withhold_first_tile, void* stream) {
    if (!workspace || workspace_bytes < sizeof(WsHeader) || (reinterpret_cast<uintptr_t>(workspace) & 255))
        return FG_ERR_INVALID_ARGUMENT;
    launch(k_set_wait_limit, 1, 1, static_cast<cudaStream_t>(stream), reinterpret_cast<WsHeader*>(workspace),
           spin_limit, withhold_first_tile ? 1u : 0u);
    return check_launch();
}

extern "C" int fg_workspace_init(void* workspace, size_t workspace_bytes, void* stream) {
    if (!workspace) return FG_ERR_INVALID_ARGUMENT;
    if (cudaMemsetAsync(workspace, 0, workspace_bytes, static_cast<cudaStream_t>(stream)) != cudaSuccess)
        return check_launch();
    return FG_OK;
}

extern "C" int fg_workspace_status(void* workspace, size_t workspace_bytes, void* stream, int32_t clear) {
    if (!workspace || workspace_bytes < sizeof(WsHeader)) return FG_ERR_INVALID_ARGUMENT;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    uint32_t v = 0;
    if (cudaMemcpyAsync(&v, workspace, sizeof(v), cudaMemcpyDeviceToHost, st) != cudaSuccess) return check_launch();
    if (cudaStreamSynchronize(st) != cudaSuccess) return check_launch();
    if (clear && v) {
        if (cudaMemsetAsync(workspace, 0, sizeof(uint32_t), st) != cudaSuccess) return check_launch();
    }
    return static_cast<int>(static_cast<int32_t>(v));
}

extern "C" int fg_set_thread_tuning(const fg_tuning* t) {
    if (t && t->scan_wide_min > 0 && t->scan_wide_min < kScanTile) return FG_ERR_INVALID_ARGUMENT;
    t_scan_wide_min = (t && t->scan_wide_min) ? t->scan_wide_min : kScanWideMin;
    return FG_OK;
}

extern "C" const char* fg_version(void) { return "flamegpu2_gb300 0.1 (sm_103a)"; }

// ------------------------------------------------------------------ batches

extern "C" int fg_batch_instance_init(fg_batch_instance* inst, const fg_spatial_grid* g, uint32_t row_begin,
                                      uint32_t row_capacity, uint32_t bucket_begin, int32_t mode,
                                      uint32_t* nbuckets_total) {
    if (!inst || !g || (mode != 0 && mode != 1)) return FG_ERR_INVALID_ARGUMENT;
    *inst = fg_batch_instance{};
    inst->grid = *g;
    inst->row_begin = row_begin;
    inst->row_capacity = row_capacity;
    inst->bucket_begin = bucket_begin;
    SortGrid sg{};
    uint32_t nb = 0;
    if (!sort_grid_from(g, &sg, &nb)) return FG_ERR_UNSUPPORTED;
    for (int a = 0; a < 3; ++a) {
        inst->sort_width[a] = sg.width[a];
        inst->sort_gd[a] = sg.gd[a];
    }
    inst->sort_mask = sg.mask;
    inst->nbuckets = mode == 0 ? g->binCount : nb;
    if (nbuckets_total) *nbuckets_total = inst->nbuckets + 1;
    if (static_cast<uint64_t>(bucket_begin) + inst->nbuckets + 1 >= kPadBit) return FG_ERR_UNSUPPORTED;
    return FG_OK;
}

extern "C" size_t fg_batched_workspace_size(uint32_t total_rows, uint32_t total_buckets) {
    // the single-list layout over (bucket count - 1) bins holds total_buckets + 1 scan entries
    return build_layout(total_rows, total_buckets, true).total;
}

extern "C" int fg_spatial_build_batched(const fg_batch_instance* instances, const uint32_t* counts, uint32_t ninst,
                                        uint32_t total_rows, uint32_t total_buckets, const float* x, const float* y,
                                        const float* z, int32_t dims, const uint32_t* valid, const fg_record_desc* rec,
                                        uint32_t* sorted, uint32_t* pbm, void* workspace, size_t workspace_bytes,
                                        void* stream) {
    if (!instances || !counts || !ninst || !rec || !pbm || !workspace || (dims != 2 && dims != 3))
        return FG_ERR_INVALID_ARGUMENT;
    if (rec->words == 0 || (rec->words & 3) || rec->words > FG_MAX_RECORD_WORDS) return FG_ERR_INVALID_ARGUMENT;
    if (total_rows && (!x || !y || (dims == 3 && !z) || !sorted)) return FG_ERR_INVALID_ARGUMENT;
    if ((reinterpret_cast<uintptr_t>(sorted) & 15) || total_buckets >= kPadBit) return FG_ERR_INVALID_ARGUMENT;
    const BuildLayout L = build_layout(total_rows, total_buckets, true);
    if (workspace_bytes < L.total || (reinterpret_cast<uintptr_t>(workspace) & 255)) return FG_ERR_WORKSPACE;
    EmitParams rp{};
    rp.rp.rec = *rec;
    rp.rp.out = sorted;
    SortGrid sg{};
    BatchKeys bk;
    bk.inst = instances;
    bk.counts = counts;
    bk.ninst = ninst;
    bk.dims = dims;
    fg_spatial_grid dummy{};
    return run_pipeline<kMessageBin, kEmitRecord>(&dummy, sg, total_buckets, total_rows, nullptr, x, y, z, valid, rp, pbm,
                                                  L, static_cast<char*>(workspace), static_cast<cudaStream_t>(stream), bk);
}

extern "C" int fg_spatial_sort_agents_batched(const fg_batch_instance* instances, const uint32_t* counts,
                                              uint32_t ninst, uint32_t total_rows, uint32_t total_buckets,
                                              const float* x, const float* y, const float* z, int32_t dims,
                                              const fg_column* cols, uint32_t ncols, void* workspace,
                                              size_t workspace_bytes, void* stream) {
    if (!instances || !counts || !ninst || !workspace || (dims != 2 && dims != 3) || ncols > FG_MAX_COLUMNS)
        return FG_ERR_INVALID_ARGUMENT;
    if (total_rows && (!x || !y || (dims == 3 && !z))) return FG_ERR_INVALID_ARGUMENT;
    if (ncols && !cols) return FG_ERR_INVALID_ARGUMENT;
    if (total_buckets >= kPadBit) return FG_ERR_INVALID_ARGUMENT;
    const BuildLayout L = build_layout(total_rows, total_buckets, true);
    if (workspace_bytes < L.total || (reinterpret_cast<uintptr_t>(workspace) & 255)) return FG_ERR_WORKSPACE;
    char* ws = static_cast<char*>(workspace);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    EmitParams rp{};
    for (uint32_t c = 0; c < ncols; ++c) rp.cp.col[c] = cols[c];
    rp.cp.ncols = ncols;
    rp.cp.keep_perm = 0;  // the batched sort returns columns only
    SortGrid sg{};
    BatchKeys bk;
    bk.inst = instances;
    bk.counts = counts;
    bk.ninst = ninst;
    bk.dims = dims;
    fg_spatial_grid dummy{};
    // padding rows (past an instance's count) keep their slot and carry no agent:
    // their columns are left as they are
    int rc = ncols ? run_pipeline<kSortKey, kEmitPermColumns>(&dummy, sg, total_buckets, total_rows, nullptr, x, y, z,
                                                              nullptr, rp, reinterpret_cast<uint32_t*>(ws + L.pbm), L,
                                                              ws, st, bk)
                   : run_pipeline<kSortKey, kEmitPerm>(&dummy, sg, total_buckets, total_rows, nullptr, x, y, z, nullptr,
                                                       rp, reinterpret_cast<uint32_t*>(ws + L.pbm), L, ws, st, bk);
    if (rc != FG_OK) return rc;
    return check_launch();
}
