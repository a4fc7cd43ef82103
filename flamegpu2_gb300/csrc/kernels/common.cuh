// Device helpers shared by the GB300 kernels: acquire/release accesses for the
// single-pass scans, bounded waits, the workspace header and launch sizing.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <utility>

#include "flamegpu/detail/launch.cuh"
#include "flamegpu/detail/spatial_keys.cuh"
#include "flamegpu_gb300/fg_capi.h"

namespace fgk {

// A launch of one of these kernels with no dynamic shared memory, programmatic
// dependency included (flamegpu/detail/launch.cuh).
template <typename... KernelArgs, typename... Args>
inline cudaError_t launch(void (*kernel)(KernelArgs...), dim3 grid, dim3 block, cudaStream_t st, Args&&... args) {
    return flamegpu::detail::launch_kernel(flamegpu::detail::pdl_enabled(), kernel, grid, block, 0, st,
                                           std::forward<Args>(args)...);
}

constexpr uint32_t kInvalid = 0xFFFFFFFFu;
constexpr int kThreads = 256;

// Default upper bound on polls of one predecessor's status in a decoupled
// look-back. A predecessor tile always belongs to a block that is already
// running (tiles are handed out in launch order by a ticket counter), so the
// wait ends in practice within microseconds; the bound only turns a broken
// invariant into a recorded error instead of a hung GPU (~2^22 polls with
// backoff ≈ 1-2 s). A workspace header may carry a smaller bound
// (WsHeader::spin_limit, set by fg_workspace_set_wait_limit).
constexpr uint32_t kSpinLimit = 1u << 22;

// Workspace header: the first 256 bytes of every workspace.
struct WsHeader {
    uint32_t status;        // fg_status recorded on the device (0 = OK)
    uint32_t scan_epoch;    // generation tag of the scan tile statuses
    uint32_t scan_ticket;   // tile ticket counter of the scan
    uint32_t scan_done;     // finished scan blocks (last one resets)
    uint32_t long_count;    // long bins queued for the segment stabiliser
    uint32_t comp_ticket;   // compaction tile tickets
    uint32_t comp_done;     // finished compaction blocks
    uint32_t comp_parity;   // which compaction status array is live
    uint32_t alive_total;   // survivors, when computed here
    uint32_t key_max;       // largest sort key of an agent sort (0 between sorts)
    uint32_t spin_limit;    // look-back poll bound (0 = kSpinLimit)
    uint32_t withhold;      // non-zero: tile 0 of scans and compactions does not publish (wait test)
    uint32_t disorder;      // non-zero: a build's keys are not in row order (0 between builds)
    uint32_t pad[51];
};
static_assert(sizeof(WsHeader) == 256, "header is 256 bytes");
// words an agent-function launch resets when it computes a build's keys
static_assert(offsetof(WsHeader, scan_epoch) == 4 * flamegpu::detail::kWsHdrScanEpoch, "header layout");
static_assert(offsetof(WsHeader, scan_ticket) == 4 * flamegpu::detail::kWsHdrScanTicket, "header layout");
static_assert(offsetof(WsHeader, long_count) == 4 * flamegpu::detail::kWsHdrLongCount, "header layout");
static_assert(offsetof(WsHeader, key_max) == 4 * flamegpu::detail::kWsHdrKeyMax, "header layout");
static_assert(offsetof(WsHeader, disorder) == 4 * flamegpu::detail::kWsHdrDisorder, "header layout");

__device__ __forceinline__ uint64_t ld_acquire_u64(const uint64_t* p) {
    uint64_t v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u64(uint64_t* p, uint64_t v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
// Read-only load (data not written while the kernel runs); not volatile, so
// the compiler may schedule several before their first use.
__device__ __forceinline__ uint32_t ld_nc_u32(const uint32_t* p) {
    uint32_t v;
    asm("ld.global.nc.u32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}

// The look-back poll bound of a workspace.
__device__ __forceinline__ uint32_t spin_limit_of(const WsHeader* h) {
    const uint32_t v = h->spin_limit;
    return v ? v : kSpinLimit;
}

__device__ __forceinline__ void record_status(WsHeader* h, int32_t code) {
    atomicCAS(&h->status, 0u, static_cast<uint32_t>(code));
}

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Warp-aggregated atomicAdd(&hist[key], 1): lanes with equal keys share one
// atomic; each gets old + its rank among lower lanes with the same key.
__device__ __forceinline__ uint32_t warp_aggregated_inc(uint32_t* hist, uint32_t key, uint32_t active) {
    const uint32_t peers = __match_any_sync(active, key);
    const uint32_t leader = __ffs(peers) - 1;
    uint32_t base = 0;
    if (lane_id() == leader) base = atomicAdd(hist + key, static_cast<uint32_t>(__popc(peers)));
    base = __shfl_sync(peers, base, leader);
    return base + __popc(peers & lanemask_lt());
}

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

}  // namespace fgk
