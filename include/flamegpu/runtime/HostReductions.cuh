#ifndef INCLUDE_FLAMEGPU_RUNTIME_HOSTREDUCTIONS_CUH_
#define INCLUDE_FLAMEGPU_RUNTIME_HOSTREDUCTIONS_CUH_
// Host-function reductions that run user code on the device or count into a
// histogram (HostAgentAPI::count / histogramEven / reduce / transformReduce,
// include/flamegpu/runtime/agent/HostAgentAPI.cuh:226-268): templates over the
// variable type and the user's operators, so their kernels are compiled in the
// model's own translation unit.
//
// A reduction is two launches with a fixed shape, so its result does not
// depend on scheduling: 256 blocks each fold a strided slice of the column in
// index order and then in a fixed tree, one block folds the 256 partials the
// same way. A slot that has seen no value carries a flag instead of an
// identity (a custom operator has none), and init is combined with the total
// once, at the end. Each call waits for its result, as the reference's do.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <string>
#include <type_traits>
#include <vector>

#include "flamegpu/detail/launch.cuh"
#include "flamegpu/exception/FLAMEGPUException.h"
#include "flamegpu/simulation/CUDASimulation.h"

/**
 * A binary reduction operator for HostAgentAPI::reduce / transformReduce
 * (HostAgentAPI.cuh:69-78): FLAMEGPU_CUSTOM_REDUCTION(name, a, b) { return ...; }
 * defines `name`, callable on two values of the reduced type.
 */
#define FLAMEGPU_CUSTOM_REDUCTION(funcName, a, b)                              \
    struct funcName##_impl {                                                   \
        template <typename T>                                                  \
        __host__ __device__ T operator()(const T& a, const T& b) const;        \
    };                                                                         \
    static funcName##_impl funcName;                                           \
    template <typename T>                                                      \
    __host__ __device__ T funcName##_impl::operator()(const T& a, const T& b) const

/**
 * A unary transform for HostAgentAPI::transformReduce (HostAgentAPI.cuh:104-112):
 * FLAMEGPU_CUSTOM_TRANSFORM(name, a) { return ...; } defines `name`, mapping a
 * value of the variable's type to the reduced type.
 */
#define FLAMEGPU_CUSTOM_TRANSFORM(funcName, a)                                 \
    struct funcName##_impl {                                                   \
        template <typename InT, typename OutT>                                 \
        __host__ __device__ OutT apply(const InT& a) const;                    \
    };                                                                         \
    static funcName##_impl funcName;                                           \
    template <typename InT, typename OutT>                                     \
    __host__ __device__ OutT funcName##_impl::apply(const InT& a) const

namespace flamegpu {
namespace detail {

constexpr int kHostRedBlocks = 256;
constexpr int kHostRedThreads = 256;

struct HostReduceIdentity {
    template <typename InT, typename OutT>
    __host__ __device__ OutT apply(const InT& a) const { return static_cast<OutT>(a); }
};

template <typename T, typename Op>
__device__ __forceinline__ void host_fold(T& acc, bool& has, const T& v, const Op& op) {
    acc = has ? op(acc, v) : v;
    has = true;
}

// The block's (value, present) pairs folded in a fixed tree; thread 0 returns the total.
template <typename T, typename Op>
__device__ __forceinline__ bool host_block_fold(T& acc, bool has, const Op& op) {
    __shared__ alignas(16) unsigned char s_raw[sizeof(T) * kHostRedThreads];
    __shared__ unsigned char s_has[kHostRedThreads];
    T* s_v = reinterpret_cast<T*>(s_raw);
    s_v[threadIdx.x] = acc;
    s_has[threadIdx.x] = has ? 1 : 0;
    __syncthreads();
    for (int w = kHostRedThreads / 2; w > 0; w >>= 1) {
        const int t = static_cast<int>(threadIdx.x);
        if (t < w && s_has[t + w]) {
            s_v[t] = s_has[t] ? op(s_v[t], s_v[t + w]) : s_v[t + w];
            s_has[t] = 1;
        }
        __syncthreads();
    }
    acc = s_v[0];
    return s_has[0] != 0;
}

template <typename InT, typename OutT, typename Tr, typename Op>
__global__ void __launch_bounds__(kHostRedThreads) k_host_reduce_parts(const InT* __restrict__ col, const uint32_t* d_n,
                                                                      Tr tr, Op op, OutT* part_v,
                                                                      unsigned char* part_has) {
    grid_dependency_enter();
    const uint32_t n = *d_n;
    OutT acc{};
    bool has = false;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        host_fold(acc, has, tr.template apply<InT, OutT>(col[i]), op);
    has = host_block_fold(acc, has, op);
    if (threadIdx.x == 0) {
        part_v[blockIdx.x] = acc;
        part_has[blockIdx.x] = has ? 1 : 0;
    }
}

template <typename T, typename Op>
__global__ void __launch_bounds__(kHostRedThreads) k_host_reduce_final(const T* part_v, const unsigned char* part_has,
                                                                      Op op, T init, T* out) {
    grid_dependency_enter();
    T acc{};
    bool has = false;
    for (int b = threadIdx.x; b < kHostRedBlocks; b += blockDim.x)
        if (part_has[b]) host_fold(acc, has, part_v[b], op);
    has = host_block_fold(acc, has, op);
    if (threadIdx.x == 0) *out = has ? op(init, acc) : init;
}

template <typename InT>
__global__ void __launch_bounds__(kHostRedThreads) k_host_count(const InT* __restrict__ col, const uint32_t* d_n,
                                                               InT value, unsigned int* out) {
    grid_dependency_enter();
    const uint32_t n = *d_n;
    unsigned int c = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        c += col[i] == value ? 1u : 0u;
    c = __reduce_add_sync(0xFFFFFFFFu, c);
    if ((threadIdx.x & 31u) == 0 && c) atomicAdd(out, c);
}

// Bin of v: floor((v - lower) * bins / (upper - lower)) in double, for the
// values in [lower, upper); counted in shared memory when the bins fit.
template <typename InT>
__global__ void __launch_bounds__(kHostRedThreads) k_host_histogram(const InT* __restrict__ col, const uint32_t* d_n,
                                                                   unsigned int bins, InT lower, InT upper,
                                                                   double scale, unsigned int* hist) {
    grid_dependency_enter();
    constexpr unsigned int kSmemBins = 2048;
    __shared__ unsigned int s_hist[kSmemBins];
    const bool local = bins <= kSmemBins;
    if (local)
        for (unsigned int b = threadIdx.x; b < bins; b += blockDim.x) s_hist[b] = 0u;
    __syncthreads();
    const uint32_t n = *d_n;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const InT v = col[i];
        if (!(v >= lower && v < upper)) continue;
        double f = (static_cast<double>(v) - static_cast<double>(lower)) * scale;
        unsigned int b = f > 0.0 ? static_cast<unsigned int>(f) : 0u;
        if (b >= bins) b = bins - 1;
        atomicAdd(local ? &s_hist[b] : &hist[b], 1u);
    }
    if (local) {
        __syncthreads();
        for (unsigned int b = threadIdx.x; b < bins; b += blockDim.x)
            if (s_hist[b]) atomicAdd(&hist[b], s_hist[b]);
    }
}

// Device scratch of one host reduction, on the simulation's stream.
class HostScratch {
 public:
    HostScratch(size_t bytes, cudaStream_t st) : st_(st) {
        if (cudaMallocAsync(&p_, bytes, st) != cudaSuccess)
            THROW exception::CUDAError("Cannot allocate the scratch of a host reduction");
    }
    ~HostScratch() {
        if (p_) cudaFreeAsync(p_, st_);
    }
    HostScratch(const HostScratch&) = delete;
    HostScratch& operator=(const HostScratch&) = delete;
    char* get() const { return static_cast<char*>(p_); }

 private:
    void* p_ = nullptr;
    cudaStream_t st_;
};

inline void host_reduction_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess)
        THROW exception::CUDAError(exception::format("%s failed: %s", what, cudaGetErrorString(e)));
}

}  // namespace detail

template <typename InT>
unsigned int HostAPI::AgentAPI::count(const std::string& variable, InT value) const {
    const uint32_t* d_n = nullptr;
    cudaStream_t st = nullptr;
    const InT* col = static_cast<const InT*>(device_column(variable, typeid(InT), &d_n, &st));
    detail::HostScratch scratch(sizeof(unsigned int), st);
    unsigned int* d_out = reinterpret_cast<unsigned int*>(scratch.get());
    unsigned int out = 0;
    detail::host_reduction_check(cudaMemsetAsync(d_out, 0, sizeof(unsigned int), st), "count");
    detail::host_reduction_check(detail::launch_kernel(detail::pdl_enabled(), detail::k_host_count<InT>,
                                                       detail::kHostRedBlocks, detail::kHostRedThreads, 0, st, col,
                                                       d_n, value, d_out),
                                 "count");
    detail::host_reduction_check(cudaMemcpyAsync(&out, d_out, sizeof(out), cudaMemcpyDeviceToHost, st), "count");
    detail::host_reduction_check(cudaStreamSynchronize(st), "count");
    return out;
}

template <typename InT>
std::vector<unsigned int> HostAPI::AgentAPI::histogramEven(const std::string& variable, unsigned int histogramBins,
                                                           InT lowerBound, InT upperBound) const {
    return histogramEven<InT, unsigned int>(variable, histogramBins, lowerBound, upperBound);
}

template <typename InT, typename OutT>
std::vector<OutT> HostAPI::AgentAPI::histogramEven(const std::string& variable, unsigned int histogramBins,
                                                   InT lowerBound, InT upperBound) const {
    // HostAgentAPI::histogramEven's argument checks (HostAgentAPI.cuh:567-575)
    if (lowerBound >= upperBound)
        THROW exception::InvalidArgument("histogramEven: lowerBound must be below upperBound");
    if (histogramBins == 0) THROW exception::InvalidArgument("histogramEven: histogramBins must be at least 1");
    const uint32_t* d_n = nullptr;
    cudaStream_t st = nullptr;
    const InT* col = static_cast<const InT*>(device_column(variable, typeid(InT), &d_n, &st));
    detail::HostScratch scratch(sizeof(unsigned int) * histogramBins, st);
    unsigned int* d_hist = reinterpret_cast<unsigned int*>(scratch.get());
    detail::host_reduction_check(cudaMemsetAsync(d_hist, 0, sizeof(unsigned int) * histogramBins, st),
                                 "histogramEven");
    const double scale =
        static_cast<double>(histogramBins) / (static_cast<double>(upperBound) - static_cast<double>(lowerBound));
    detail::host_reduction_check(
        detail::launch_kernel(detail::pdl_enabled(), detail::k_host_histogram<InT>, detail::kHostRedBlocks,
                              detail::kHostRedThreads, 0, st, col, d_n, histogramBins, lowerBound, upperBound, scale,
                              d_hist),
        "histogramEven");
    std::vector<unsigned int> counts(histogramBins);
    detail::host_reduction_check(cudaMemcpyAsync(counts.data(), d_hist, sizeof(unsigned int) * histogramBins,
                                                 cudaMemcpyDeviceToHost, st),
                                 "histogramEven");
    detail::host_reduction_check(cudaStreamSynchronize(st), "histogramEven");
    return std::vector<OutT>(counts.begin(), counts.end());
}

template <typename InT, typename OutT, typename TransformT, typename ReductionT>
OutT HostAPI::AgentAPI::transformReduce(const std::string& variable, TransformT transformOperator,
                                        ReductionT reductionOperator, OutT init) const {
    const uint32_t* d_n = nullptr;
    cudaStream_t st = nullptr;
    const InT* col = static_cast<const InT*>(device_column(variable, typeid(InT), &d_n, &st));
    const size_t vbytes = (sizeof(OutT) * detail::kHostRedBlocks + 15) & ~static_cast<size_t>(15);
    detail::HostScratch scratch(vbytes + sizeof(OutT) + 16 + detail::kHostRedBlocks, st);
    OutT* part_v = reinterpret_cast<OutT*>(scratch.get());
    OutT* d_out = reinterpret_cast<OutT*>(scratch.get() + vbytes);
    unsigned char* part_has = reinterpret_cast<unsigned char*>(scratch.get() + vbytes + sizeof(OutT) + 16);
    detail::host_reduction_check(
        detail::launch_kernel(detail::pdl_enabled(), detail::k_host_reduce_parts<InT, OutT, TransformT, ReductionT>,
                              detail::kHostRedBlocks, detail::kHostRedThreads, 0, st, col, d_n, transformOperator,
                              reductionOperator, part_v, part_has),
        "transformReduce");
    detail::host_reduction_check(
        detail::launch_kernel(detail::pdl_enabled(), detail::k_host_reduce_final<OutT, ReductionT>, 1,
                              detail::kHostRedThreads, 0, st, static_cast<const OutT*>(part_v),
                              static_cast<const unsigned char*>(part_has), reductionOperator, init, d_out),
        "transformReduce");
    OutT out;
    detail::host_reduction_check(cudaMemcpyAsync(&out, d_out, sizeof(OutT), cudaMemcpyDeviceToHost, st),
                                 "transformReduce");
    detail::host_reduction_check(cudaStreamSynchronize(st), "transformReduce");
    return out;
}

template <typename InT, typename ReductionT>
InT HostAPI::AgentAPI::reduce(const std::string& variable, ReductionT reductionOperator, InT init) const {
    return transformReduce<InT, InT>(variable, detail::HostReduceIdentity(), reductionOperator, init);
}

}  // namespace flamegpu

#endif  // INCLUDE_FLAMEGPU_RUNTIME_HOSTREDUCTIONS_CUH_
