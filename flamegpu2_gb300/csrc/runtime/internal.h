// Helpers shared by the simulation and ensemble runtimes (not installed).
#pragma once

#include <algorithm>
#include <cstdint>
#include <vector>

#include "flamegpu/detail/device_types.cuh"

namespace flamegpu {
namespace detail {

struct TableEntry {
    uint32_t hash;
    char* ptr;
    uint32_t stride;
    uint32_t elem_bytes;
    uint32_t elements;
};

/** Collision-free multiplicative lookup table over the given variables:
 * slot = (hash * mult) >> shift; throws if no multiplier up to 64 slots works. */
VarTable make_table(const std::vector<TableEntry>& e, const char* what);

/** Layout of a spatial message record: the location (x, y[, z], 4 bytes
 *  each) at words 0..dims-1, then every other variable at word
 *  dims + slot * stride/4, slot being its perfect-hash slot among those
 *  variables (pay_mult, pay_shift: the device computes the same slot from the
 *  name). A field's offset is then arithmetic on launch constants, which the
 *  compiler hoists out of the neighbour loop, instead of a table load in it. */
struct SpatialRecordLayout {
    std::vector<uint32_t> field_word;  // per message variable
    uint32_t record_words = 0;         // multiple of 4
    uint32_t pay_mult = 0, pay_shift = 0, pay_stride = 0;  // stride: bytes per slot
};
/** vars: (name hash, bytes rounded up to 4) of every message variable, the
 *  location first; throws InvalidMessage if the location is not first. */
SpatialRecordLayout spatial_record_layout(const std::vector<std::pair<uint32_t, uint32_t>>& vars, int dims,
                                          const char* what);

// Whether a block's neighbourhood window (the sorted records from one z/y slab
// below its lowest bin to one above its highest) is expected to fit a staging
// buffer of stage_bytes, with per_bin messages in every bin of grid g. Staging
// reserves the buffer's shared memory for every block, which caps occupancy,
// so it is only worth it when the window usually fits.
inline bool stage_window_fits(const fg_spatial_grid& g, double per_bin, uint32_t record_words, uint32_t block,
                              unsigned int stage_bytes) {
    const double span = g.dims == 3 ? static_cast<double>(g.gridDim[0]) * g.gridDim[1] + g.gridDim[0] + 1.0
                                    : static_cast<double>(g.gridDim[0]) + 1.0;
    const double block_bins = std::max(1.0, block / std::max(per_bin, 1e-3));
    const double bins = 2.0 * span + block_bins;
    const double bytes = bins * per_bin * record_words * 4.0 + (bins + 8.0) * 4.0;
    return bytes <= 0.9 * stage_bytes;
}

}  // namespace detail
}  // namespace flamegpu

// The message build and agent sort with the option of keys computed by the
// launch before them (keys_ready: no key kernel), and where such a launch
// writes them (kernels/spatial.cu). Used by the simulation runtime only.
int fgi_spatial_build(const fg_spatial_grid* g, uint32_t max_n, const uint32_t* d_n, const float* x, const float* y,
                      const float* z, const uint32_t* valid, const fg_record_desc* rec, uint32_t* sorted, uint32_t* pbm,
                      void* workspace, size_t workspace_bytes, void* stream, bool keys_ready);
// pos_stride: floats from one row's coordinate to the next (1: x, y, z
// columns; 2 or 3: a packed "xy" / "xyz" array variable, never with keys_ready)
int fgi_spatial_sort_agents(const fg_spatial_grid* g, uint32_t max_n, const uint32_t* d_n, const float* x,
                            const float* y, const float* z, const fg_column* cols, uint32_t ncols, uint32_t* perm_out,
                            void* workspace, size_t workspace_bytes, void* stream, bool keys_ready,
                            uint32_t pos_stride = 1);
// The word of a compaction workspace's header that fg_compact_agents counts
// the survivors into (zero between compactions): a launch that writes the
// death flags may add its survivors there itself and pass it as d_alive_total.
uint32_t* fgi_compact_survivor_word(void* workspace);
// The agent sort of a list and the build of the spatial messages it output
// on the same grid, as one chain of paired launches (both key sets written by
// the launch before).
int fgi_spatial_sort_and_build(const fg_spatial_grid* g, uint32_t sort_max_n, const uint32_t* sort_d_n,
                               const fg_column* cols, uint32_t ncols, void* sort_ws, size_t sort_ws_bytes,
                               uint32_t msg_max_n, const uint32_t* msg_d_n, const fg_record_desc* rec,
                               uint32_t* sorted, uint32_t* pbm, void* build_ws, size_t build_ws_bytes, void* stream);
int fgi_key_target(const fg_spatial_grid* g, uint32_t max_n, bool sort_mode, void* workspace, size_t workspace_bytes,
                   flamegpu::detail::KeyTarget* t);
