/*
 * fg_capi.h — the C ABI of the GB300 kernel library (libflamegpu2_gb300.so).
 *
 * These entry points replace the device work behind FLAME GPU 2's
 * MessageSpecialisationHandler::buildIndex, CUDAScatter and
 * CUDAScanCompaction (see each declaration for the reference interface it
 * stands in for). Plain C: device pointers, sizes, a cudaStream_t passed as
 * void*. No entry point allocates device memory: callers own every buffer and
 * size the scratch ("workspace") with the *_workspace_size() query, then clear
 * it once with fg_workspace_init().
 *
 * Counts may live on the device so that a whole simulation step can be
 * captured into a CUDA graph: wherever a `const uint32_t* d_n` is taken, a
 * non-NULL pointer is read on the device (the host-side `max_n` is then only
 * an upper bound used to size grids); a NULL pointer means "exactly max_n".
 *
 * Every function returns FG_OK (0) or a negative fg_status. Launch errors are
 * reported as FG_ERR_CUDA with cudaGetLastError() left readable by
 * fg_last_cuda_error(). Device-side failures (a bounded wait that gave up)
 * are recorded in the workspace and read back with fg_workspace_status().
 */
#ifndef FLAMEGPU_GB300_FG_CAPI_H_
#define FLAMEGPU_GB300_FG_CAPI_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum fg_status {
    FG_OK = 0,
    FG_ERR_INVALID_ARGUMENT = -1,   /* exception::InvalidArgument */
    FG_ERR_WORKSPACE = -2,          /* workspace too small / misaligned */
    FG_ERR_CUDA = -3,               /* a CUDA runtime call failed */
    FG_ERR_DEVICE_TIMEOUT = -4,     /* a bounded device-side wait gave up (recorded on the device) */
    FG_ERR_CAPACITY = -5,           /* an output would exceed the caller's capacity */
    FG_ERR_UNSUPPORTED = -6
} fg_status;

/* Spatial partitioning grid. Mirrors MessageSpatial3D::MetaData /
 * MessageSpatial2D::MetaData (include/flamegpu/runtime/messaging/MessageSpatial3D.h:38-68,
 * MessageSpatial2D.h:39-69); built on the host as
 * MessageSpatial3D::CUDAModelHandler's constructor does
 * (src/flamegpu/runtime/messaging/MessageSpatial3D.cu:31-52). */
typedef struct fg_spatial_grid {
    int32_t dims;            /* 2 or 3 */
    float min[3];
    float max[3];
    float radius;
    float width[3];          /* max - min */
    uint32_t gridDim[3];     /* ceil(width / radius); 1 on unused axes */
    uint32_t binCount;       /* product of gridDim */
    int32_t wrapCompatible;  /* radius divides every width (numeric.h:24-31) */
} fg_spatial_grid;

/* Largest sorted-message record, in 4-byte words. */
#define FG_MAX_RECORD_WORDS 64
/* Largest number of agent variable columns moved by one sort / compaction. */
#define FG_MAX_COLUMNS 48

/* How the build assembles one sorted message record (an array-of-structs row
 * of `words` 4-byte words, `words` a multiple of 4 so rows are 16-byte aligned)
 * from the unsorted struct-of-arrays message columns. Word w of the record is
 * word `src_word[w]` of element i of column `src[w]`, whose elements are
 * `src_stride[w]` words long; src[w] == NULL writes 0 (padding). */
typedef struct fg_record_desc {
    uint32_t words;
    const uint32_t* src[FG_MAX_RECORD_WORDS];
    uint32_t src_stride[FG_MAX_RECORD_WORDS];
    uint32_t src_word[FG_MAX_RECORD_WORDS];
} fg_record_desc;

/* One agent variable column moved by a sort or compaction: `in` and `out` are
 * distinct device arrays of elements of `elem_bytes` bytes (any size; 4-, 8-
 * and 16-byte multiples take vector paths). */
typedef struct fg_column {
    const void* in;
    void* out;
    uint32_t elem_bytes;
} fg_column;

/* Host-side grid set-up: MessageSpatial3D.cu:31-52 / MessageSpatial2D.cu:36-54.
 * Fails with FG_ERR_INVALID_ARGUMENT for radius <= 0, max <= min, dims not 2/3. */
int fg_spatial_grid_init(fg_spatial_grid* g, int32_t dims, const float* min, const float* max, float radius);

/* Scratch bytes needed by fg_spatial_build / fg_spatial_sort_agents for up to
 * max_n elements over bin_count bins. */
size_t fg_spatial_build_workspace_size(uint32_t max_n, uint32_t bin_count);
size_t fg_spatial_sort_workspace_size(uint32_t max_n, const fg_spatial_grid* msg_grid);
/* Scratch bytes needed by fg_compact_agents for up to max_n agents. */
size_t fg_compact_workspace_size(uint32_t max_n);
/* Zero a freshly allocated workspace once (an async memset on `stream`). The
 * kernels leave it ready for the next call afterwards. */
int fg_workspace_init(void* workspace, size_t workspace_bytes, void* stream);
/* Device-side status recorded in a workspace (FG_OK or FG_ERR_DEVICE_TIMEOUT);
 * synchronises `stream`. clear != 0 resets it. */
int fg_workspace_status(void* workspace, size_t workspace_bytes, void* stream, int32_t clear);
/* Bounded-wait controls kept in a workspace's header, applied by the scans and
 * compactions launched on it after this call (stream-ordered). spin_limit is
 * the number of polls of one predecessor tile's status after which a
 * decoupled look-back gives up, records FG_ERR_DEVICE_TIMEOUT and finishes
 * (0 = the default, 2^22 polls with back-off, about a second).
 * withhold_first_tile != 0 makes tile 0 of those kernels skip publishing its
 * status, so that every look-back that reaches it runs out its limit: a
 * host-side fault injection for testing the give-up path with a short limit.
 * fg_workspace_init() restores both defaults. No counterpart in the reference
 * (CUB's look-back has no bound). */
int fg_workspace_set_wait_limit(void* workspace, size_t workspace_bytes, uint32_t spin_limit,
                                int32_t withhold_first_tile, void* stream);

/* Spatial message index build. Replaces MessageSpatial3D::CUDAModelHandler::buildIndex
 * (src/flamegpu/runtime/messaging/MessageSpatial3D.cu:113-146; 2D: MessageSpatial2D.cu:114-141)
 * together with CUDAScatter::pbm_reorder (src/flamegpu/simulation/detail/CUDAScatter.cu:276-337)
 * and the optional-output compaction of CUDAMessage::swap (CUDAMessage.cu:171-208).
 *
 *   x, y, z      message positions (z ignored/NULL for 2D), device, length >= count
 *   valid        optional per-message output flags (non-zero = message exists), or NULL
 *   rec          record layout of the sorted messages (host struct)
 *   sorted       out: count * rec->words words, device
 *   pbm          out: binCount + 1 entries: pbm[b] = first sorted message of bin b,
 *                pbm[binCount] = number of messages (exclusive scan of the bin histogram)
 *
 * Within a bin, messages are ordered by ascending original index (stable); the
 * reference leaves that order unspecified (atomicInc, MessageSpatial3D.cu:70). */
int fg_spatial_build(const fg_spatial_grid* grid, uint32_t max_n, const uint32_t* d_n,
                     const float* x, const float* y, const float* z, const uint32_t* valid,
                     const fg_record_desc* rec, uint32_t* sorted, uint32_t* pbm,
                     void* workspace, size_t workspace_bytes, void* stream);

/* Automatic spatial agent sort: stable sort of the agents by the reference's
 * unclamped, width-based bin key masked to floor(log2(bins))+1 bits, applied to
 * every column. Replaces CUDASimulation::spatialSortAgent_async + HostAgentAPI::sort_async
 * (src/flamegpu/simulation/CUDASimulation.cu:335-573,
 * include/flamegpu/runtime/agent/HostAgentAPI.cuh:858-915). msg_grid is the
 * grid of the message list the sorting function reads. If perm_out is non-NULL
 * it receives perm[sorted_pos] = original index. */
int fg_spatial_sort_agents(const fg_spatial_grid* msg_grid, uint32_t max_n, const uint32_t* d_n,
                           const float* x, const float* y, const float* z,
                           const fg_column* cols, uint32_t ncols, uint32_t* perm_out,
                           void* workspace, size_t workspace_bytes, void* stream);

/* Fused, order-preserving birth/death compaction. Replaces the death scan +
 * scatter (src/flamegpu/simulation/detail/CUDAFatAgent.cu:105-137,
 * CUDAFatAgentStateList.cu:155-178, CUDAScatter.cu:67-88) and the birth
 * append (CUDAAgentStateList.cu:189-250, CUDAFatAgent.cu:311-346) in one pass:
 *
 *   out[0 .. S)          = rows i with alive[i] != 0, in order
 *   out[S .. S + births) = birth rows i with born[i] != 0, in parent order
 *
 * alive / born may be NULL (all alive / no births). cols move survivors,
 * birth_cols (same count and order as cols, `in` = per-parent staging rows)
 * move births; both write into the same `out` arrays. If id_col >= 0, births'
 * word id_col of cols[] receives *d_next_id + birth rank and *d_next_id is
 * advanced by the number of births (deterministic: the reference draws child
 * ids with atomicInc, DeviceAPI.cuh:546-557); a birth row whose born flag is 2
 * keeps the id its staging row holds (claimed on the device before the call,
 * from *d_next_id, which is then read after those claims). d_alive_total (device) may carry
 * S if the caller already has it (else it is computed here). The new
 * population S + births is written to *d_n_out (device). out_capacity bounds
 * the output; births beyond it are dropped and the status word records
 * FG_ERR_CAPACITY. */
int fg_compact_agents(uint32_t max_n, const uint32_t* d_n, const uint32_t* alive, const uint32_t* born,
                      const fg_column* cols, const fg_column* birth_cols, uint32_t ncols,
                      int32_t id_col, uint32_t* d_next_id, const uint32_t* d_alive_total,
                      uint32_t* d_n_out, uint32_t out_capacity,
                      void* workspace, size_t workspace_bytes, void* stream);

/* Agent birth into another list (another agent type, or another state of the
 * same agent). Replaces CUDAAgent::scatterNew / CUDAAgentStateList::scatterNew
 * (src/flamegpu/simulation/detail/CUDAAgent.cu:427-450,
 * src/flamegpu/simulation/detail/CUDAAgentStateList.cu:189-250), which append
 * the new agents after the destination list's agents in parent order:
 *
 *   out[D + r] = birth row i (the r-th row i < n with born[i] != 0),
 *   D = *d_dst_count before the call; *d_dst_count grows by the births.
 *
 * cols[c].in are the per-parent staging rows, cols[c].out the destination
 * columns (distinct arrays). If id_col >= 0, word id_col of each birth receives
 * *d_next_id + r and *d_next_id advances by the births. Births past
 * dst_capacity are dropped and the workspace records FG_ERR_CAPACITY.
 * Workspace: fg_compact_workspace_size(max_n), shared with fg_compact_agents
 * (calls on one workspace must be ordered). */
int fg_append_births(uint32_t max_n, const uint32_t* d_n, const uint32_t* born, const fg_column* cols,
                     uint32_t ncols, int32_t id_col, uint32_t* d_next_id, uint32_t* d_dst_count,
                     uint32_t dst_capacity, void* workspace, size_t workspace_bytes, void* stream);

/* Stable two-way partition of an agent list. Replaces the agent function
 * condition scatter of CUDAFatAgent::processFunctionCondition
 * (src/flamegpu/simulation/detail/CUDAFatAgent.cu:186-236), which moves the
 * agents whose condition failed to the front of the list and the others after
 * them, each group in its original order. Rows i < n with first_group[i] != 0
 * go first, the rest follow; every column is written from cols[c].in to
 * cols[c].out (distinct arrays). *d_first_count receives the size of the first
 * group (device). Workspace: fg_compact_workspace_size(max_n), shared with
 * fg_compact_agents (calls on one workspace must be ordered). */
int fg_partition_agents(uint32_t max_n, const uint32_t* d_n, const uint32_t* first_group,
                        const fg_column* cols, uint32_t ncols, uint32_t* d_first_count,
                        void* workspace, size_t workspace_bytes, void* stream);

/* Agent state transition. Replaces CUDAFatAgent::transitionState
 * (src/flamegpu/simulation/detail/CUDAFatAgent.cu:139-184): rows
 * [*d_begin (0 if NULL), *d_src_count) of the source columns (cols[c].in) are
 * appended, in order, after the *d_dst_count rows of the destination columns
 * (cols[c].out); then *d_dst_count grows by their number and *d_src_count
 * becomes *d_begin. max_rows bounds the source rows (grid sizing); rows past
 * dst_capacity are not written and the workspace records FG_ERR_CAPACITY
 * (any workspace of at least 256 bytes initialised by fg_workspace_init). */
int fg_append_rows(const fg_column* cols, uint32_t ncols, uint32_t max_rows, const uint32_t* d_begin,
                   uint32_t* d_src_count, uint32_t* d_dst_count, uint32_t dst_capacity, void* workspace,
                   size_t workspace_bytes, void* stream);

/* Exclusive scan of n u32 values (single pass, decoupled look-back); out may
 * alias in. Used for PBMs built elsewhere; replaces cub::DeviceScan::ExclusiveSum
 * on this path. */
size_t fg_scan_workspace_size(uint32_t n);
int fg_exclusive_scan_u32(const uint32_t* in, uint32_t* out, uint32_t n,
                          void* workspace, size_t workspace_bytes, void* stream);

/* Largest n fg_exclusive_scan_u32_noalloc accepts (2^25 values, 128 MiB of input). */
#define FG_NOALLOC_SCAN_MAX_N (1u << 25)

/* The same exclusive scan for a caller that has no scratch to give: one whose
 * device memory all belongs to another allocator, or that is handed only the
 * input and output pointers across a language boundary and has no allocator of
 * its own there. No counterpart in the reference (cub::DeviceScan::ExclusiveSum,
 * which it uses, always takes caller scratch).
 *
 * The scratch is a fixed 66,048-byte array in this library's static device
 * memory, one per device; nothing is allocated, now or later. Its limit:
 * n > FG_NOALLOC_SCAN_MAX_N returns FG_ERR_WORKSPACE and launches nothing.
 * The first call on a device, with that device current, does the set-up: it
 * looks up the array's address and clears it (the scan's tile ticket, epoch
 * and tile statuses must start at zero), waiting for that clear to finish.
 * Make that first call before any stream capture. Every later call only
 * launches the scan on `stream` and leaves the scratch ready for the next.
 * All calls on one device share the one scratch: calls that overlap on the
 * GPU (issued on different streams without ordering, or from several host
 * threads at once) race and give wrong results. Order them, e.g. on one stream.
 * out may alias in. */
int fg_exclusive_scan_u32_noalloc(const uint32_t* in, uint32_t* out, uint32_t n, void* stream);
/* Device-side status of the allocation-free scan's scratch on the current
 * device: FG_OK, or FG_ERR_DEVICE_TIMEOUT if a call's bounded look-back gave up
 * (its output is then wrong). Synchronises `stream`; clear != 0 resets it (the
 * status is sticky until cleared). The counterpart of fg_workspace_status for
 * fg_exclusive_scan_u32_noalloc; does the same first-call set-up. */
int fg_noalloc_scan_status(void* stream, int32_t clear);

/* ------------------------------------------------------------- batches */

/* One instance of a batch: many simulations of one model, concatenated.
 * Rows [row_begin, row_begin + row_capacity) of every column belong to the
 * instance; rows at or past its count (fg_*_batched `counts`) are padding.
 * Its buckets are [bucket_begin, bucket_begin + nbuckets + 1): its own bins
 * (or sort buckets) plus one bucket that collects its padding rows, so a
 * single counting sort over the batch leaves every instance in its segment
 * and instance i's PBM is pbm[bucket_begin .. bucket_begin + binCount]. */
typedef struct fg_batch_instance {
    fg_spatial_grid grid;    /* the instance's message grid */
    uint32_t row_begin;
    uint32_t row_capacity;
    uint32_t bucket_begin;
    uint32_t nbuckets;       /* bins (build) or 2^bits sort buckets (sort); set by fg_batch_instance_init */
    /* sort key data derived from the grid (CUDASimulation.cu:494-507,569-571) */
    float sort_width[3];
    uint32_t sort_gd[3];
    uint32_t sort_mask;
    uint32_t pad;
} fg_batch_instance;

/* Fill an instance record (host). mode 0: message build buckets (binCount),
 * mode 1: automatic-sort buckets (2^bits). Returns the bucket count the
 * instance needs including its padding bucket in *nbuckets_total. */
int fg_batch_instance_init(fg_batch_instance* inst, const fg_spatial_grid* grid, uint32_t row_begin,
                           uint32_t row_capacity, uint32_t bucket_begin, int32_t mode, uint32_t* nbuckets_total);
size_t fg_batched_workspace_size(uint32_t total_rows, uint32_t total_buckets);

/* fg_spatial_build over a batch: `instances` (device, ninst records, ordered
 * by row_begin) and `counts` (device, messages per instance); valid flags are
 * optional as in fg_spatial_build. Rows are the concatenated message columns. */
int fg_spatial_build_batched(const fg_batch_instance* instances, const uint32_t* counts, uint32_t ninst,
                             uint32_t total_rows, uint32_t total_buckets, const float* x, const float* y,
                             const float* z, int32_t dims, const uint32_t* valid, const fg_record_desc* rec,
                             uint32_t* sorted, uint32_t* pbm, void* workspace, size_t workspace_bytes, void* stream);
/* fg_spatial_sort_agents over a batch (sort buckets, mode 1 instances). */
int fg_spatial_sort_agents_batched(const fg_batch_instance* instances, const uint32_t* counts, uint32_t ninst,
                                   uint32_t total_rows, uint32_t total_buckets, const float* x, const float* y,
                                   const float* z, int32_t dims, const fg_column* cols, uint32_t ncols,
                                   void* workspace, size_t workspace_bytes, void* stream);

/* fg_compact_agents over a batch: every instance's agents compacted in place of
 * its own row segment in one launch (the reference compacts each run on its
 * own: CUDAFatAgent.cu:105-137, CUDAAgentStateList.cu:189-250). Instance k's
 * first counts[k] rows (device, in/out) are its agents: survivors (alive, or
 * all if NULL) go first from row_begin_k, in order, then births (born != 0, in
 * parent order; birth_cols as in fg_compact_agents) with ids next_ids[k] + rank
 * (a born flag of 2 keeps the staging row's id); counts[k] and next_ids[k]
 * (device, per instance) are updated. Births past an instance's row_capacity
 * are dropped and FG_ERR_CAPACITY recorded. `instances` (device) as for the
 * batched builds; `tile_begin` (device, ninst + 1 entries) and `ntiles` from
 * fg_batch_compact_tiles over the same instances (host copy). cols[c].in /
 * .out are the whole concatenated columns (distinct arrays). */
uint32_t fg_batch_compact_tiles(const fg_batch_instance* instances, uint32_t ninst, uint32_t* tile_begin);
size_t fg_compact_batched_workspace_size(uint32_t ntiles, uint32_t ninst);
int fg_compact_agents_batched(const fg_batch_instance* instances, const uint32_t* tile_begin, uint32_t ninst,
                              uint32_t ntiles, uint32_t total_rows, uint32_t* counts, const uint32_t* alive,
                              const uint32_t* born, const fg_column* cols, const fg_column* birth_cols,
                              uint32_t ncols, int32_t id_col, uint32_t* next_ids, void* workspace,
                              size_t workspace_bytes, void* stream);

/* Launch-shape settings of the calling thread's later scan, build and sort
 * calls: a tuner's knobs (fg_set_thread_tuning(NULL) restores the defaults).
 * scan_wide_min: scans of more values than this take tiles of four 4,096-value
 * sub-tiles, which need a quarter of the look-back rounds (0: the default,
 * 4,194,304; otherwise at least 4,096). No counterpart in the reference (CUB
 * picks its tile shapes at compile time). */
typedef struct fg_tuning {
    uint32_t scan_wide_min;
    uint32_t reserved[3];
} fg_tuning;
int fg_set_thread_tuning(const fg_tuning* t);

/* Last CUDA error seen by this library on the calling thread (cudaError_t). */
int fg_last_cuda_error(void);
/* Library version string. */
const char* fg_version(void);

#ifdef __cplusplus
}
#endif

#endif /* FLAMEGPU_GB300_FG_CAPI_H_ */
