// Step and exit logs of CUDASimulation: environment properties, agent counts
// and reductions of agent variables, computed on the device.
//
// A reduction is two kernels so that its result does not depend on scheduling:
// a fixed grid of blocks each reduces a strided slice in a fixed tree order to a
// partial, then one block reduces the partials in order. The standard deviation
// takes a second pass over the squared deviations from the mean (population
// standard deviation, as HostAgentAPI::meanStandardDeviation,
// include/flamegpu/runtime/agent/HostAgentAPI.cuh:259-300).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <type_traits>

#include "flamegpu/detail/launch.cuh"
#include "flamegpu/simulation/CUDASimulation.h"
#include "flamegpu_gb300/fg_capi.h"
#include "flamegpu/simulation/LoggingConfig.h"

namespace flamegpu {
namespace detail {

namespace {

constexpr int kLogBlocks = 256;
constexpr int kLogThreads = 256;

// accumulator of a sum: double for floating point, 64-bit integers otherwise
template <typename T>
using acc_t = typename sum_input_t<T>::result_t;

struct Partial {
    double dsum;        // floating point sum, or squared deviations
    long long isum;     // signed sum
    unsigned long long usum;
    double dmin, dmax;  // min / max as double (floating point types)
    long long imin, imax;
    unsigned long long umin, umax;
};

template <typename T>
__device__ __forceinline__ void fold(Partial& p, T v) {
    if (std::is_floating_point<T>::value) {
        p.dsum += static_cast<double>(v);
        p.dmin = fmin(p.dmin, static_cast<double>(v));
        p.dmax = fmax(p.dmax, static_cast<double>(v));
    } else if (std::is_signed<T>::value) {
        p.isum += static_cast<long long>(v);
        p.imin = min(p.imin, static_cast<long long>(v));
        p.imax = max(p.imax, static_cast<long long>(v));
    } else {
        p.usum += static_cast<unsigned long long>(v);
        p.umin = min(p.umin, static_cast<unsigned long long>(v));
        p.umax = max(p.umax, static_cast<unsigned long long>(v));
    }
}

__device__ __forceinline__ void combine(Partial& a, const Partial& b) {
    a.dsum += b.dsum;
    a.isum += b.isum;
    a.usum += b.usum;
    a.dmin = fmin(a.dmin, b.dmin);
    a.dmax = fmax(a.dmax, b.dmax);
    a.imin = min(a.imin, b.imin);
    a.imax = max(a.imax, b.imax);
    a.umin = min(a.umin, b.umin);
    a.umax = max(a.umax, b.umax);
}

__device__ __forceinline__ Partial identity() {
    Partial p;
    p.dsum = 0.0;
    p.isum = 0;
    p.usum = 0;
    p.dmin = INFINITY;
    p.dmax = -INFINITY;
    p.imin = 0x7FFFFFFFFFFFFFFFll;
    p.imax = -0x7FFFFFFFFFFFFFFFll - 1;
    p.umin = ~0ull;
    p.umax = 0;
    return p;
}

// block tree reduction in shared memory, fixed order
__device__ Partial block_combine(Partial p) {
    __shared__ Partial s[kLogThreads];
    s[threadIdx.x] = p;
    __syncthreads();
    for (int w = kLogThreads / 2; w > 0; w >>= 1) {
        if (static_cast<int>(threadIdx.x) < w) combine(s[threadIdx.x], s[threadIdx.x + w]);
        __syncthreads();
    }
    return s[0];
}

// pass 0: sum / min / max; pass 1: sum of (v - mean)^2 into dsum
template <typename T>
__global__ void __launch_bounds__(kLogThreads) k_log_partials(const T* __restrict__ col, const uint32_t* d_n,
                                                              const double* mean, int pass, Partial* out) {
    grid_dependency_enter();
    const uint32_t n = *d_n;
    Partial p = identity();
    const double m = pass ? *mean : 0.0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (pass) {
            const double d = static_cast<double>(col[i]) - m;
            p.dsum += d * d;
        } else {
            fold<T>(p, col[i]);
        }
    }
    p = block_combine(p);
    if (threadIdx.x == 0) out[blockIdx.x] = p;
}

// one block: the partials in order; result[0] = combined, and for pass 0 the
// mean (as double) in *mean
template <typename T>
__global__ void __launch_bounds__(kLogThreads) k_log_final(const Partial* __restrict__ parts, const uint32_t* d_n,
                                                           int pass, Partial* result, double* mean) {
    grid_dependency_enter();
    Partial p = identity();
    for (int b = threadIdx.x; b < kLogBlocks; b += blockDim.x) combine(p, parts[b]);
    p = block_combine(p);
    if (threadIdx.x == 0) {
        result[pass] = p;
        if (!pass) {
            const uint32_t n = *d_n;
            double s = std::is_floating_point<T>::value ? p.dsum
                       : (std::is_signed<T>::value ? static_cast<double>(p.isum) : static_cast<double>(p.usum));
            *mean = n ? s / n : 0.0;
        }
    }
}

template <typename T>
LogValue make_value(T v) {
    LogValue out;
    out.type = std::type_index(typeid(T));
    out.bytes.resize(sizeof(T));
    std::memcpy(out.bytes.data(), &v, sizeof(T));
    return out;
}

template <typename T>
void reduce_typed(const void* col, const uint32_t* d_n, const std::vector<LoggingConfig::Reduction>& want,
                  cudaStream_t st, char* scratch, std::map<LoggingConfig::NameReduction, LogValue>& out,
                  const std::string& var) {
    Partial* parts = reinterpret_cast<Partial*>(scratch);
    Partial* result = parts + kLogBlocks;   // [0] pass 0, [1] pass 1
    double* mean = reinterpret_cast<double*>(result + 2);
    bool need_sd = false;
    for (auto r : want) need_sd = need_sd || r == LoggingConfig::StandardDev;
    launch_kernel(pdl_enabled(), k_log_partials<T>, kLogBlocks, kLogThreads, 0, st, static_cast<const T*>(col), d_n,
                  mean, 0, parts);
    launch_kernel(pdl_enabled(), k_log_final<T>, 1, kLogThreads, 0, st, parts, d_n, 0, result, mean);
    if (need_sd) {
        launch_kernel(pdl_enabled(), k_log_partials<T>, kLogBlocks, kLogThreads, 0, st, static_cast<const T*>(col),
                      d_n, mean, 1, parts);
        launch_kernel(pdl_enabled(), k_log_final<T>, 1, kLogThreads, 0, st, parts, d_n, 1, result, mean);
    }
    Partial res[2];
    double m = 0.0;
    uint32_t n = 0;
    if (cudaMemcpyAsync(res, result, sizeof(res), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(&m, mean, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(&n, d_n, sizeof(uint32_t), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        THROW exception::CUDAError("Log reduction failed");
    for (auto r : want) {
        switch (r) {
            case LoggingConfig::Mean: out[{var, r}] = make_value<double>(m); break;
            case LoggingConfig::StandardDev: out[{var, r}] = make_value<double>(n ? std::sqrt(res[1].dsum / n) : 0.0); break;
            case LoggingConfig::Sum:
                if (std::is_floating_point<T>::value) out[{var, r}] = make_value<double>(res[0].dsum);
                else if (std::is_signed<T>::value) out[{var, r}] = make_value<int64_t>(res[0].isum);
                else out[{var, r}] = make_value<uint64_t>(res[0].usum);
                break;
            case LoggingConfig::Min:
            case LoggingConfig::Max: {
                const bool mn = r == LoggingConfig::Min;
                T v;
                if (std::is_floating_point<T>::value) v = static_cast<T>(mn ? res[0].dmin : res[0].dmax);
                else if (std::is_signed<T>::value) v = static_cast<T>(mn ? res[0].imin : res[0].imax);
                else v = static_cast<T>(mn ? res[0].umin : res[0].umax);
                if (n == 0) v = T(0);
                out[{var, r}] = make_value<T>(v);
                break;
            }
        }
    }
}

void reduce_column(std::type_index t, const void* col, const uint32_t* d_n, const std::vector<LoggingConfig::Reduction>& want,
                   cudaStream_t st, char* scratch, std::map<LoggingConfig::NameReduction, LogValue>& out,
                   const std::string& var) {
    if (t == std::type_index(typeid(float))) reduce_typed<float>(col, d_n, want, st, scratch, out, var);
    else if (t == std::type_index(typeid(double))) reduce_typed<double>(col, d_n, want, st, scratch, out, var);
    else if (t == std::type_index(typeid(int32_t))) reduce_typed<int32_t>(col, d_n, want, st, scratch, out, var);
    else if (t == std::type_index(typeid(uint32_t))) reduce_typed<uint32_t>(col, d_n, want, st, scratch, out, var);
    else if (t == std::type_index(typeid(int64_t))) reduce_typed<int64_t>(col, d_n, want, st, scratch, out, var);
    else if (t == std::type_index(typeid(uint64_t))) reduce_typed<uint64_t>(col, d_n, want, st, scratch, out, var);
    else if (t == std::type_index(typeid(int16_t))) reduce_typed<int16_t>(col, d_n, want, st, scratch, out, var);
    else if (t == std::type_index(typeid(uint16_t))) reduce_typed<uint16_t>(col, d_n, want, st, scratch, out, var);
    else if (t == std::type_index(typeid(int8_t))) reduce_typed<int8_t>(col, d_n, want, st, scratch, out, var);
    else if (t == std::type_index(typeid(uint8_t))) reduce_typed<uint8_t>(col, d_n, want, st, scratch, out, var);
    else THROW exception::InvalidVarType(exception::format("Variable '%s' has a type logs cannot reduce", var.c_str()));
}

}  // namespace

size_t log_scratch_bytes();
size_t log_scratch_bytes() { return sizeof(Partial) * (kLogBlocks + 2) + sizeof(double) * 2; }

// One reduction of a column (HostAgentAPI reductions through CUDASimulation::reduceAgentVariable).
void reduce_column_of(std::type_index t, const void* col, const uint32_t* d_n, LoggingConfig::Reduction r,
                      cudaStream_t st, char* scratch, std::map<LoggingConfig::NameReduction, LogValue>& out,
                      const std::string& var);
void reduce_column_of(std::type_index t, const void* col, const uint32_t* d_n, LoggingConfig::Reduction r,
                      cudaStream_t st, char* scratch, std::map<LoggingConfig::NameReduction, LogValue>& out,
                      const std::string& var) {
    reduce_column(t, col, d_n, {r}, st, scratch, out, var);
}

void fill_log_frame(const LoggingConfig& cfg, CUDASimulation& sim, char* scratch, LogFrame& frame) {
    const auto& model = *cfg.model();
    for (const auto& name : cfg.environment()) {
        for (const auto& p : model.environment) {
            if (p.name != name) continue;
            LogValue v;
            v.type = p.type;
            v.elements = p.elements;
            v.bytes.resize(p.value.size());
            sim.getEnvironmentRaw(name, v.bytes.data(), v.bytes.size());
            frame.environment[name] = std::move(v);
        }
    }
    for (const auto& kv : cfg.agents()) {
        auto& slot = frame.agents[kv.first];
        slot.second = kv.second.count ? sim.getAgentCount(kv.first.first, kv.first.second) : ~0u;
        // group the requested reductions by variable
        std::map<std::string, std::vector<LoggingConfig::Reduction>> by_var;
        for (const auto& nr : kv.second.reductions) by_var[nr.name].push_back(nr.reduction);
        for (const auto& bv : by_var) {
            const AgentData* a = nullptr;
            for (const auto& x : model.agents)
                if (x->name == kv.first.first) a = x.get();
            const Variable* var = a->find(bv.first);
            reduce_column(var->type, sim.getDeviceVariable(kv.first.first, bv.first, kv.first.second),
                          sim.getDeviceCount(kv.first.first, kv.first.second), bv.second, sim.getStream(), scratch,
                          slot.first, bv.first);
        }
    }
}

}  // namespace detail

namespace {

std::string log_number(const LogValue& v, size_t k = 0) {
    char buf[64];
    const char* p = v.bytes.data() + k * (v.bytes.size() / std::max<uint32_t>(v.elements, 1));
    const auto t = v.type;
    if (t == std::type_index(typeid(double))) std::snprintf(buf, sizeof(buf), "%.17g", *reinterpret_cast<const double*>(p));
    else if (t == std::type_index(typeid(float))) std::snprintf(buf, sizeof(buf), "%.9g", static_cast<double>(*reinterpret_cast<const float*>(p)));
    else if (t == std::type_index(typeid(int64_t))) std::snprintf(buf, sizeof(buf), "%lld", static_cast<long long>(*reinterpret_cast<const int64_t*>(p)));
    else if (t == std::type_index(typeid(uint64_t))) std::snprintf(buf, sizeof(buf), "%llu", static_cast<unsigned long long>(*reinterpret_cast<const uint64_t*>(p)));
    else if (t == std::type_index(typeid(int32_t))) std::snprintf(buf, sizeof(buf), "%d", *reinterpret_cast<const int32_t*>(p));
    else if (t == std::type_index(typeid(uint32_t))) std::snprintf(buf, sizeof(buf), "%u", *reinterpret_cast<const uint32_t*>(p));
    else if (t == std::type_index(typeid(int16_t))) std::snprintf(buf, sizeof(buf), "%d", *reinterpret_cast<const int16_t*>(p));
    else if (t == std::type_index(typeid(uint16_t))) std::snprintf(buf, sizeof(buf), "%u", *reinterpret_cast<const uint16_t*>(p));
    else if (t == std::type_index(typeid(int8_t))) std::snprintf(buf, sizeof(buf), "%d", *reinterpret_cast<const int8_t*>(p));
    else if (t == std::type_index(typeid(uint8_t))) std::snprintf(buf, sizeof(buf), "%u", *reinterpret_cast<const uint8_t*>(p));
    else std::snprintf(buf, sizeof(buf), "null");
    return buf;
}

// a frame as the reference's JSONLogger writes it (src/flamegpu/io/JSONLogger.cu:80-140)
// One frame in JSONLogger::writeLogFrame's layout (src/flamegpu/io/JSONLogger.cu:80-140):
// its times first (a step frame's step_time; an exit frame's rtc_time,
// init_time, exit_time and total_time), then step_index, env, agents.
void write_frame(std::string& o, const LogFrame& f, const std::vector<std::pair<const char*, double>>& times) {
    o += "{";
    for (const auto& t : times) {
        char buf[64];
        std::snprintf(buf, sizeof(buf), "%.17g", t.second);
        o += std::string("\"") + t.first + "\": " + buf + ", ";
    }
    o += "\"step_index\": " + std::to_string(f.getStepCount());
    if (!f.environment.empty()) {
        o += ", \"env\": {";
        bool first = true;
        for (const auto& e : f.environment) {
            o += (first ? "" : ", ") + ("\"" + e.first + "\": ");
            first = false;
            if (e.second.elements == 1) {
                o += log_number(e.second);
            } else {
                o += "[";
                for (uint32_t k = 0; k < e.second.elements; ++k) o += (k ? ", " : "") + log_number(e.second, k);
                o += "]";
            }
        }
        o += "}";
    }
    if (!f.agents.empty()) {
        o += ", \"agents\": {";
        std::map<std::string, std::vector<const std::pair<const std::pair<std::string, std::string>,
                                                             std::pair<std::map<LoggingConfig::NameReduction, LogValue>, unsigned int>>*>>
            by_agent;
        for (const auto& a : f.agents) by_agent[a.first.first].push_back(&a);
        bool fa = true;
        for (const auto& ba : by_agent) {
            o += (fa ? "" : ", ") + ("\"" + ba.first + "\": {");
            fa = false;
            bool fs = true;
            for (const auto* a : ba.second) {
                o += (fs ? "" : ", ") + ("\"" + a->first.second + "\": [{");
                fs = false;
                bool fk = true;
                if (a->second.second != ~0u) {
                    o += "\"count\": " + std::to_string(a->second.second);
                    fk = false;
                }
                if (!a->second.first.empty()) {
                    o += (fk ? "" : ", ") + std::string("\"variables\": {");
                    std::string cur;
                    bool fv = true;
                    for (const auto& r : a->second.first) {
                        if (r.first.name != cur) {
                            if (!cur.empty()) o += "}";
                            o += (fv ? "" : ", ") + ("\"" + r.first.name + "\": {");
                            fv = false;
                            cur = r.first.name;
                        } else {
                            o += ", ";
                        }
                        o += std::string("\"") + LoggingConfig::toString(r.first.reduction) + "\": " + log_number(r.second);
                    }
                    if (!cur.empty()) o += "}";
                    o += "}";
                }
                o += "}]";
            }
            o += "}";
        }
        o += "}";
    }
    o += "}";
}

}  // namespace

std::string CUDASimulation::runLogJSON(bool with_times) const {
    // JSONLogger::logCommon (src/flamegpu/io/JSONLogger.cu:179-197): config,
    // performance_specs (only with the times), steps, exit
    std::string o = "{\"config\": {\"random_seed\": " + std::to_string(run_log.getRandomSeed()) + "}";
    if (with_times) {
        cudaDeviceProp prop{};
        int rt = 0;
        int dev = 0;
        cudaGetDevice(&dev);
        cudaGetDeviceProperties(&prop, dev);
        cudaRuntimeGetVersion(&rt);
        o += ", \"performance_specs\": {\"device_name\": \"" + std::string(prop.name) +
             "\", \"device_cc_major\": " + std::to_string(prop.major) + ", \"device_cc_minor\": " +
             std::to_string(prop.minor) + ", \"cuda_version\": " + std::to_string(rt) +
             // device checks are compiled per model source here; on unless a source turns them off
             ", \"seatbelts\": true, \"flamegpu_version\": \"" + fg_version() + "\"}";
    }
    o += ", \"steps\": [";
    bool first = true;
    for (const auto& f : run_log.getStepLog()) {
        if (!first) o += ", ";
        first = false;
        write_frame(o, f, with_times ? std::vector<std::pair<const char*, double>>{{"step_time", f.getStepTime()}}
                                     : std::vector<std::pair<const char*, double>>{});
    }
    o += "]";
    if (exit_log) {
        const ExitLogFrame& e = run_log.getExitLog();
        o += ", \"exit\": ";
        write_frame(o, e, with_times ? std::vector<std::pair<const char*, double>>{{"rtc_time", e.getRTCTime()},
                                                                                    {"init_time", e.getInitTime()},
                                                                                    {"exit_time", e.getExitTime()},
                                                                                    {"total_time", e.getTotalTime()}}
                                     : std::vector<std::pair<const char*, double>>{});
    }
    o += "}";
    return o;
}

void CUDASimulation::setStepLog(const StepLoggingConfig& cfg) {
    if (cfg.model() != getModelData()) THROW exception::InvalidArgument("The logging configuration belongs to another model");
    step_log = std::make_unique<StepLoggingConfig>(cfg);
    run_log.step_log_frequency = step_log->frequency();
}

void CUDASimulation::setExitLog(const LoggingConfig& cfg) {
    if (cfg.model() != getModelData()) THROW exception::InvalidArgument("The logging configuration belongs to another model");
    exit_log = std::make_unique<LoggingConfig>(cfg);
}

void CUDASimulation::processStepLog(double step_seconds) {
    // CUDASimulation::processStepLog (CUDASimulation.cu:1949-1983)
    if (!step_log) return;
    const unsigned int step = getStepCounter();
    if (step % step_log->frequency() != 0) return;
    if (!log_scratch && cudaMalloc(&log_scratch, detail::log_scratch_bytes()) != cudaSuccess)
        THROW exception::CUDAError("Cannot allocate the log reduction buffer");
    synchronize();
    StepLogFrame frame;
    frame.step_count = step;
    if (step_seconds < 0.0) {
        const std::vector<double> t = getElapsedTimeSteps();
        step_seconds = t.empty() ? 0.0 : t.back();
    }
    frame.step_time = step_seconds;
    detail::fill_log_frame(*step_log, *this, log_scratch, frame);
    run_log.random_seed = SimulationConfig().random_seed;
    run_log.step.push_back(std::move(frame));
}

LogValue CUDASimulation::reduceAgentVariable(const std::string& agent, const std::string& variable,
                                             LoggingConfig::Reduction r, const std::string& state) {
    if (!log_scratch && cudaMalloc(&log_scratch, detail::log_scratch_bytes()) != cudaSuccess)
        THROW exception::CUDAError("Cannot allocate the log reduction buffer");
    synchronize();
    const detail::AgentData* a = nullptr;
    for (const auto& x : getModelData()->agents)
        if (x->name == agent) a = x.get();
    if (!a) THROW exception::InvalidAgentName(exception::format("No agent '%s'", agent.c_str()));
    const detail::Variable* var = a->find(variable);
    if (!var) THROW exception::InvalidAgentVar(exception::format("Agent '%s' has no variable '%s'", agent.c_str(), variable.c_str()));
    std::map<LoggingConfig::NameReduction, LogValue> out;
    detail::reduce_column_of(var->type, getDeviceVariable(agent, variable, state), getDeviceCount(agent, state), r,
                             getStream(), log_scratch, out, variable);
    return out[{variable, r}];
}

void CUDASimulation::processExitLog(double total_seconds) {
    // CUDASimulation::processExitLog (CUDASimulation.cu:1985-2022)
    if (!exit_log) return;
    if (!log_scratch && cudaMalloc(&log_scratch, detail::log_scratch_bytes()) != cudaSuccess)
        THROW exception::CUDAError("Cannot allocate the log reduction buffer");
    synchronize();
    ExitLogFrame frame;
    frame.step_count = getStepCounter();
    frame.total_time = total_seconds;
    detail::fill_log_frame(*exit_log, *this, log_scratch, frame);
    run_log.random_seed = SimulationConfig().random_seed;
    run_log.exit = std::move(frame);
}

}  // namespace flamegpu
