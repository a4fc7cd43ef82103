#ifndef INCLUDE_FLAMEGPU_RUNTIME_AGENTFUNCTION_CUH_
#define INCLUDE_FLAMEGPU_RUNTIME_AGENTFUNCTION_CUH_
// FLAMEGPU_AGENT_FUNCTION and the kernel that runs it
// (include/flamegpu/runtime/AgentFunction_shim.cuh:32-40,
// include/flamegpu/runtime/AgentFunction.cuh:60-120).
//
// The macro keeps the reference's shape: it defines funcName_impl with a
// device operator()(DeviceAPI<In, Out>*) and a global instance funcName. The
// kernel is instantiated in the translation unit that defines the function,
// so the user's code inlines into it. One thread per agent in a grid-stride
// loop over the device-resident population (grid sized once per capacity, so
// the launch can live in a CUDA graph while the population changes). After
// the call the kernel records the death flag (ALIVE/DEAD), the birth flag and
// the optional-message flag of the row.
#include <cuda_runtime.h>

#include <type_traits>
#include <typeindex>
#include <typeinfo>

#include "flamegpu/detail/launch.cuh"
#include "flamegpu/runtime/DeviceAPI.cuh"

namespace flamegpu {
namespace detail {

/** Launches the agent function kernel of one FLAMEGPU_AGENT_FUNCTION. */
typedef cudaError_t (*AgentFunctionLauncher)(const LaunchParams& p, unsigned int grid, unsigned int block,
                                             unsigned int smem, cudaStream_t stream, bool pdl);

constexpr unsigned int kAgentBlock = 128;

#ifdef __CUDACC__
// Instance of row `row` in a batched launch (instances ordered by row_begin).
__device__ __forceinline__ uint32_t batch_find(const BatchInstanceRT* b, uint32_t n, uint32_t row) {
    uint32_t lo = 0, hi = n - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (__ldg(&b[mid].row_begin) <= row)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// Fill the block's instance context for rows starting at `base`. Single
// simulations take it from the launch; batched launches from the instance
// owning `base` (instance segments start at multiples of kAgentBlock, so a
// block never straddles two instances).
__device__ __forceinline__ void fill_ctx(const LaunchParams& P, uint32_t base, uint32_t n_single) {
    if (threadIdx.x != 0) return;
    InstanceCtx& c = ctx();
    if (!P.batch) {
        c.grid = P.in_grid;
        c.pbm = P.in_pbm;
        c.pbm_alloc = P.in_pbm_alloc;
        c.step = P.d_step ? *P.d_step : 0u;
        c.env = P.env;
        c.seed = P.seed;
        c.row_begin = P.d_first ? *P.d_first : 0u;  // rows before it failed the function's condition
        c.count = n_single;
        c.inst = 0;
        return;
    }
    const uint32_t k = batch_find(P.batch, P.batch_n, base);
    const BatchInstanceRT& I = P.batch[k];
    c.grid = I.in_grid;
    c.pbm = P.in_pbm ? P.in_pbm + I.in_bucket_begin : nullptr;
    // each instance's PBM slice reserves binCount + 1 entries rounded up to 4
    c.pbm_alloc = (I.in_grid.binCount + 1u + 3u) & ~3u;
    c.step = (P.d_step ? *P.d_step : 0u) - I.step_offset;
    c.env = I.env;
    c.seed = I.seed;
    c.row_begin = I.row_begin;
    c.count = __ldg(P.batch_counts + k);
    c.inst = k;
}

// Resident blocks per SM the agent-function kernels are compiled for (the
// register budget: 65,536 / (128 x this)). 8 (at most 64 registers) unless a
// model source defines it before including flamegpu.h, for a model whose
// functions fit fewer registers without spilling (more warps to hide latency).
// Each function also has a variant compiled for one block per SM (no register
// cap below 255), launched when the grid is at most one block per SM: there
// occupancy is one block anyway, and spills only lengthen each agent's chain.
#ifndef FLAMEGPU_AGENT_MIN_BLOCKS
#define FLAMEGPU_AGENT_MIN_BLOCKS 8
#endif

template <typename F, int MINB>
__global__ void __launch_bounds__(kAgentBlock, MINB) agent_function_kernel(const __grid_constant__ LaunchParams P) {
    grid_dependency_enter();
    using MsgIn = typename F::MessageIn;
    using MsgOut = typename F::MessageOut;
    // rows to visit: the population (single) or every row of the batch
    const uint32_t n = P.batch ? P.max_n : (P.d_n ? min(*P.d_n, P.max_n) : P.max_n);
    const uint32_t first_row = (!P.batch && P.d_first) ? min(*P.d_first, n) : 0u;
    // message rows: after those already output to the list this step (append), else from 0
    const uint32_t msg_base = (!P.batch && P.msg_out_base) ? *P.msg_out_base : 0u;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        // a launch over no agents leaves the list as it was (the reference skips
        // such a function, CUDASimulation.cu:1050-1059): a persistent list keeps
        // its messages
        if (P.msg_out_count && n > first_row) {
            *P.msg_out_count = msg_base + n - first_row;
            if (P.msg_out_filled) *P.msg_out_filled = 1u;
        }
        if (P.keyed[0].mode) key_target_reset(P.keyed[0]);
        if (P.keyed[1].mode) key_target_reset(P.keyed[1]);
    }
    constexpr int kDims = std::is_same<MsgIn, MessageSpatial3D>::value ? 3 : (std::is_same<MsgIn, MessageSpatial2D>::value ? 2 : 0);
    bool first = true;
    uint32_t out_of_order = 0u;  // keyed targets whose rows were not in key order
    uint32_t alive_rows = 0u;    // rows this thread left ALIVE (survivor count for the compaction)
    if (!P.batch) {
        fill_ctx(P, 0, n);
        __syncthreads();
    }
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        if (P.batch) {
            __syncthreads();  // the previous round is done with the context
            fill_ctx(P, base, 0);
            __syncthreads();
        }
        const uint32_t idx = base + threadIdx.x;
        // rows past the instance's count are padding (batched) / past the population (single)
        const uint32_t limit = P.batch ? ctx().row_begin + ctx().count : n;
        const uint32_t live = idx < limit ? idx : 0xFFFFFFFFu;
        if constexpr (kDims != 0) {
            if (P.stage_bytes) stage_window<kDims>(P, idx, live != 0xFFFFFFFFu, first);
        }
        first = false;
        if (live == 0xFFFFFFFFu) continue;
        if (idx < first_row) {  // failed the condition: kept as it is
            if (P.death_flags) P.death_flags[idx] = static_cast<uint32_t>(ALIVE);
            ++alive_rows;
            if (P.birth_flags) P.birth_flags[idx] = 0u;
            continue;
        }
        const uint32_t msg_row = msg_base + idx - first_row;
        // the agent's sort key at its position before the function, computed
        // alongside the function's own work (again after it if it moved)
        float pre[3] = {0.0f, 0.0f, 0.0f};
        uint32_t pre_key = 0xFFFFFFFFu;
        if (P.keyed[1].mode == kKeySortKey) {
            pre[0] = P.keyed[1].x[idx];
            pre[1] = P.keyed[1].y[idx];
            if (P.keyed[1].dims == 3) pre[2] = P.keyed[1].z[idx];
            pre_key = key_target_key(P.keyed[1], true, pre[0], pre[1], pre[2]);
        }
        DeviceAPI<MsgIn, MsgOut> api(P, idx, msg_row);
        const AGENT_STATUS st = F()(&api);
        alive_rows += st == ALIVE ? 1u : 0u;
        if (P.death_flags) {
            P.death_flags[idx] = static_cast<uint32_t>(st);
        } else if (st == DEAD) {
            device_error(P, kDevDeathNotEnabled, 0, idx);
        }
        if (P.birth_flags) P.birth_flags[idx] = api.agent_out.born();
        const bool wrote = P.msg_out_always || api.message_out.written();
        if (P.msg_out_valid) P.msg_out_valid[msg_row] = wrote ? 1u : 0u;
        // keys for the message build (by message row, if a message was output,
        // at the location it was given) and for the agents' spatial sort (by
        // agent row, at the position the function left) that follow
        if (P.keyed[0].mode != kKeyNone || P.keyed[1].mode != kKeyNone) {
            uint32_t k[2] = {0xFFFFFFFFu, 0xFFFFFFFFu};
            if constexpr (!std::is_same<MsgOut, MessageNone>::value) {
                if (P.keyed[0].mode == kKeyMessageBin)
                    k[0] = key_target_key(P.keyed[0], wrote, api.message_out.location(0), api.message_out.location(1),
                                          api.message_out.location(2));
            }
            if (P.keyed[1].mode == kKeySortKey)
                k[1] = api.pos_set == 0u
                           ? pre_key
                           : key_target_key(P.keyed[1], true, (api.pos_set & 1u) ? api.pos[0] : pre[0],
                                            (api.pos_set & 2u) ? api.pos[1] : pre[1],
                                            (api.pos_set & 4u) ? api.pos[2] : pre[2]);
            const uint32_t rows[2] = {msg_row, idx};
            out_of_order |= key_targets_write(P.keyed, rows, k);
        }
    }
    if (P.keyed[0].mode != kKeyNone || P.keyed[1].mode != kKeyNone) key_targets_order_flush(P.keyed, out_of_order);
    if (P.alive_count) {
        // the block's survivors, one atomic per block (a warp's or a row's
        // atomics on one word would serialise over a large population)
        __shared__ uint32_t s_alive;
        if (threadIdx.x == 0) s_alive = 0u;
        __syncthreads();
        const uint32_t c = __reduce_add_sync(0xFFFFFFFFu, alive_rows);
        if ((threadIdx.x & 31u) == 0 && c) atomicAdd(&s_alive, c);
        __syncthreads();
        if (threadIdx.x == 0 && s_alive) atomicAdd(P.alive_count, s_alive);
    }
}

// FLAMEGPU_AGENT_FUNCTION_CONDITION kernel (AgentFunctionCondition.cuh:44-100):
// cond_fail[i] = 1 for each agent whose condition is false, 0 for those that
// pass and for rows past the population up to max_n (an exclusive scan of the
// max_n + 1 flags then counts and places the failing agents).
template <typename C>
__global__ void __launch_bounds__(kAgentBlock) agent_condition_kernel(const __grid_constant__ LaunchParams P) {
    grid_dependency_enter();
    const uint32_t n = P.d_n ? min(*P.d_n, P.max_n) : P.max_n;
    fill_ctx(P, 0, n);
    __syncthreads();
    for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx <= P.max_n; idx += gridDim.x * blockDim.x) {
        uint32_t fail = 0u;
        if (idx < n) {
            ReadOnlyDeviceAPI api(P, idx);
            fail = C()(&api) ? 0u : 1u;
        }
        P.cond_fail[idx] = fail;
    }
}

template <typename C>
cudaError_t launch_agent_condition(const LaunchParams& p, unsigned int grid, unsigned int block, unsigned int,
                                   cudaStream_t stream, bool pdl) {
    return launch_kernel(pdl, agent_condition_kernel<C>, grid, block, 0, stream, p);
}

template <typename F, int MINB>
cudaError_t launch_agent_variant(const LaunchParams& p, unsigned int grid, unsigned int block, unsigned int smem,
                                 cudaStream_t stream, bool pdl) {
    static unsigned int configured = 48u * 1024u;
    if (smem > configured) {
        const cudaError_t e = cudaFuncSetAttribute(agent_function_kernel<F, MINB>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (e != cudaSuccess) return e;
        configured = smem;
    }
    return launch_kernel(pdl, agent_function_kernel<F, MINB>, grid, block, smem, stream, p);
}

inline unsigned int device_sm_count() {
    static const unsigned int n = [] {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        return static_cast<unsigned int>(sms > 0 ? sms : 1);
    }();
    return n;
}

// block: 32, 64 or 128 threads (kAgentBlock divides into whole blocks). A
// launch of at most one 128-thread block's worth of threads per SM takes the
// variant compiled without a register cap: its blocks fit the SMs anyway.
template <typename F>
cudaError_t launch_agent_function(const LaunchParams& p, unsigned int grid, unsigned int block, unsigned int smem,
                                  cudaStream_t stream, bool pdl) {
    if (static_cast<uint64_t>(grid) * block <= static_cast<uint64_t>(device_sm_count()) * kAgentBlock)
        return launch_agent_variant<F, 1>(p, grid, block, smem, stream, pdl);
    return launch_agent_variant<F, FLAMEGPU_AGENT_MIN_BLOCKS>(p, grid, block, smem, stream, pdl);
}
#endif

}  // namespace detail
}  // namespace flamegpu

#define FLAMEGPU_AGENT_FUNCTION(funcName, message_in, message_out)                                               \
    struct funcName##_impl {                                                                                     \
        using MessageIn = message_in;                                                                            \
        using MessageOut = message_out;                                                                          \
        __device__ __forceinline__ flamegpu::AGENT_STATUS operator()(                                            \
            flamegpu::DeviceAPI<message_in, message_out>* FLAMEGPU) const;                                       \
        static flamegpu::detail::AgentFunctionLauncher launcher() {                                              \
            return &flamegpu::detail::launch_agent_function<funcName##_impl>;                                    \
        }                                                                                                        \
        static std::type_index inType() { return std::type_index(typeid(message_in)); }                          \
        static std::type_index outType() { return std::type_index(typeid(message_out)); }                        \
    };                                                                                                           \
    funcName##_impl funcName;                                                                                    \
    __device__ __forceinline__ flamegpu::AGENT_STATUS funcName##_impl::operator()(                               \
        flamegpu::DeviceAPI<message_in, message_out>* FLAMEGPU) const

/** FLAMEGPU_AGENT_FUNCTION_CONDITION (include/flamegpu/runtime/AgentFunctionCondition_shim.cuh):
 *  a device predicate over the read-only device API; agents for which it is
 *  false skip the function they are attached to (setFunctionCondition). */
#define FLAMEGPU_AGENT_FUNCTION_CONDITION(funcName)                                                              \
    struct funcName##_cdn_impl {                                                                                 \
        __device__ __forceinline__ bool operator()(flamegpu::ReadOnlyDeviceAPI* FLAMEGPU) const;                 \
        static flamegpu::detail::AgentFunctionLauncher launcher() {                                              \
            return &flamegpu::detail::launch_agent_condition<funcName##_cdn_impl>;                               \
        }                                                                                                        \
    };                                                                                                           \
    funcName##_cdn_impl funcName;                                                                                \
    __device__ __forceinline__ bool funcName##_cdn_impl::operator()(flamegpu::ReadOnlyDeviceAPI* FLAMEGPU) const

#endif  // INCLUDE_FLAMEGPU_RUNTIME_AGENTFUNCTION_CUH_
