#ifndef INCLUDE_FLAMEGPU_SIMULATION_CUDASIMULATION_H_
#define INCLUDE_FLAMEGPU_SIMULATION_CUDASIMULATION_H_
// CUDASimulation (include/flamegpu/simulation/CUDASimulation.h:177-418 in the
// reference) on GB300: every step is one captured CUDA graph per buffer
// parity (auto spatial sort, message index builds, agent function launches
// and birth/death compaction, with populations kept on the device); the
// host synchronises only when a population could outgrow its buffers or when
// results are read back.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <memory>
#include <random>
#include <string>
#include <tuple>
#include <typeinfo>
#include <utility>
#include <array>
#include <vector>

#include "flamegpu/model/ModelDescription.h"
#include "flamegpu/simulation/AgentVector.h"
#include "flamegpu/simulation/LoggingConfig.h"

namespace flamegpu {

namespace detail {
struct SimulationImpl;
}

/** An agent created by a host function (HostNewAgentAPI,
 * include/flamegpu/runtime/agent/HostNewAgentAPI.h): its variables start at
 * their defaults; it joins its population when the host function returns, with
 * a fresh id. */
class HostNewAgentAPI {
 public:
    HostNewAgentAPI(AgentVector* v, flamegpu::size_type i) : agent_((*v)[i]) {}
    template <typename T>
    void setVariable(const std::string& name, T value) { agent_.setVariable<T>(name, value); }
    template <typename T, flamegpu::size_type N>
    void setVariable(const std::string& name, const std::array<T, N>& value) { agent_.setVariable<T, N>(name, value); }
    template <typename T, flamegpu::size_type N = 0>
    void setVariable(const std::string& name, flamegpu::size_type element, T value) {
        agent_.setVariable<T, N>(name, element, value);
    }
    template <typename T>
    T getVariable(const std::string& name) const { return agent_.getVariable<T>(name); }
    template <typename T, flamegpu::size_type N>
    std::array<T, N> getVariable(const std::string& name) const { return agent_.getVariable<T, N>(name); }

 private:
    AgentVector::Agent agent_;
};

/** Host-side API of init/step/exit/host-layer functions: environment
 * properties, agent counts, reductions of agent variables (computed on the
 * device) and agent creation. */
namespace detail {
/** The host copy of one macro property while host functions hold it: read
 *  from the device when the first handle is made, written back when the last
 *  one goes (if a handle wrote to it). */
struct HostMacroData {
    std::vector<char> host;
    void* device = nullptr;
    cudaStream_t stream = nullptr;
    bool dirty = false;
    ~HostMacroData();
};
}  // namespace detail

/**
 * HostMacroProperty<T, I, J, K, W> (include/flamegpu/runtime/environment/
 * HostMacroProperty.cuh:96-260): a host function's view of an environment
 * macro property. operator[] selects along the first dimension; a view of one
 * element converts to T and supports assignment, +=, -=, *=, /= and the
 * increment and decrement operators; zero() clears the whole property.
 */
template <typename T, flamegpu::size_type I = 1, flamegpu::size_type J = 1, flamegpu::size_type K = 1,
          flamegpu::size_type W = 1>
class HostMacroProperty {
 public:
    HostMacroProperty(std::shared_ptr<detail::HostMacroData> d, size_t first) : data(std::move(d)), at(first) {}
    HostMacroProperty<T, J, K, W, 1> operator[](flamegpu::size_type i) const {
        if (I == 1 && J == 1 && K == 1 && W == 1)
            THROW exception::OutOfBoundsException("Indexing a macro property element that has no further dimension");
        if (i >= I)
            THROW exception::OutOfBoundsException(exception::format("Macro property index %u is past its dimension of %u",
                                                                    static_cast<unsigned>(i), static_cast<unsigned>(I)));
        return HostMacroProperty<T, J, K, W, 1>(data, at + static_cast<size_t>(i) * J * K * W);
    }
    operator T() const { return value(); }
    HostMacroProperty& operator=(T v) {
        ref() = v;
        return *this;
    }
    HostMacroProperty& operator+=(T v) { ref() += v; return *this; }
    HostMacroProperty& operator-=(T v) { ref() -= v; return *this; }
    HostMacroProperty& operator*=(T v) { ref() *= v; return *this; }
    HostMacroProperty& operator/=(T v) { ref() /= v; return *this; }
    T operator++() { return ++ref(); }
    T operator--() { return --ref(); }
    T operator++(int) { return ref()++; }
    T operator--(int) { return ref()--; }
    /** Every element of this view set to 0. */
    void zero() {
        std::memset(data->host.data() + at * sizeof(T), 0, sizeof(T) * I * J * K * W);
        data->dirty = true;
    }

 private:
    T value() const {
        scalar_only();
        T v;
        std::memcpy(&v, data->host.data() + at * sizeof(T), sizeof(T));
        return v;
    }
    T& ref() {
        scalar_only();
        data->dirty = true;
        return *reinterpret_cast<T*>(data->host.data() + at * sizeof(T));
    }
    static void scalar_only() {
        if (I != 1 || J != 1 || K != 1 || W != 1)
            THROW exception::InvalidOperation("A macro property with dimensions is used as one value; index it first");
    }
    std::shared_ptr<detail::HostMacroData> data;
    size_t at;
};

/** DeviceAgentVector (include/flamegpu/runtime/agent/DeviceAgentVector.h): a
 *  host function's view of an agent population (HostAgentAPI::getPopulationData). */
typedef AgentVector& DeviceAgentVector;

class HostAPI {
 public:
    class Environment {
     public:
        explicit Environment(detail::SimulationImpl* s) : sim(s) {}
        template <typename T>
        T getProperty(const std::string& name) const {
            T v;
            get(name, typeid(T), sizeof(T), &v);
            return v;
        }
        template <typename T>
        T setProperty(const std::string& name, T value) {
            T old;
            get(name, typeid(T), sizeof(T), &old);
            set(name, typeid(T), sizeof(T), &value);
            return old;
        }
        /** Array properties (HostEnvironment.cuh:208-262): the whole array, one
         *  element (N = 0: any length), or as a vector; set returns the old value(s). */
        template <typename T, flamegpu::size_type N>
        std::array<T, N> getProperty(const std::string& name) const {
            std::array<T, N> v;
            for (flamegpu::size_type i = 0; i < N; ++i) element(name, typeid(T), sizeof(T), N, i, &v[i], nullptr);
            return v;
        }
        template <typename T, flamegpu::size_type N = 0>
        T getProperty(const std::string& name, flamegpu::size_type index) const {
            T v;
            element(name, typeid(T), sizeof(T), N, index, &v, nullptr);
            return v;
        }
        template <typename T>
        std::vector<T> getPropertyArray(const std::string& name) const {
            std::vector<T> v(elements(name));
            for (size_t i = 0; i < v.size(); ++i) element(name, typeid(T), sizeof(T), 0, static_cast<flamegpu::size_type>(i), &v[i], nullptr);
            return v;
        }
        template <typename T, flamegpu::size_type N>
        std::array<T, N> setProperty(const std::string& name, const std::array<T, N>& value) {
            std::array<T, N> old;
            for (flamegpu::size_type i = 0; i < N; ++i) element(name, typeid(T), sizeof(T), N, i, &old[i], &value[i]);
            return old;
        }
        template <typename T, flamegpu::size_type N = 0>
        T setProperty(const std::string& name, flamegpu::size_type index, T value) {
            T old;
            element(name, typeid(T), sizeof(T), N, index, &old, &value);
            return old;
        }
        template <typename T>
        std::vector<T> setPropertyArray(const std::string& name, const std::vector<T>& value) {
            if (value.size() != elements(name))
                THROW exception::OutOfBoundsException(exception::format("Environment property '%s' has another length", name.c_str()));
            std::vector<T> old(value.size());
            for (size_t i = 0; i < value.size(); ++i)
                element(name, typeid(T), sizeof(T), 0, static_cast<flamegpu::size_type>(i), &old[i], &value[i]);
            return old;
        }

        /** Set a property from raw bytes (size checked). */
        void setRaw(const std::string& name, const void* value, size_t size);

        /** HostEnvironment::getMacroProperty (HostEnvironment.cuh:148-160): the
         *  macro property's values, read back from the device; what the
         *  returned view writes reaches the device when the last view of the
         *  property is gone. */
        template <typename T, flamegpu::size_type I = 1, flamegpu::size_type J = 1, flamegpu::size_type K = 1,
                  flamegpu::size_type W = 1>
        HostMacroProperty<T, I, J, K, W> getMacroProperty(const std::string& name) const {
            const uint32_t dims[4] = {I, J, K, W};
            return HostMacroProperty<T, I, J, K, W>(macro(name, typeid(T), sizeof(T), dims), 0);
        }

     private:
        std::shared_ptr<detail::HostMacroData> macro(const std::string& name, const std::type_info& t, size_t size,
                                                     const uint32_t (&dims)[4]) const;
        void get(const std::string& name, const std::type_info& t, size_t size, void* out) const;
        void set(const std::string& name, const std::type_info& t, size_t size, const void* in);
        // element index of an array property (length n, 0: any): read into out, then written from in if given
        void element(const std::string& name, const std::type_info& t, size_t size, flamegpu::size_type n,
                     flamegpu::size_type index, void* out, const void* in) const;
        size_t elements(const std::string& name) const;
        detail::SimulationImpl* sim;
    };
    /** HostRandom (include/flamegpu/runtime/random/HostRandom.cuh:22-66): host-side
     *  draws from one std::mt19937_64 per simulation, seeded with its random seed
     *  (setSeed reseeds it). */
    class Random {
     public:
        explicit Random(detail::SimulationImpl* s) : sim(s) {}
        template <typename T>
        T uniform() const {
            static_assert(std::is_floating_point<T>::value, "HostRandom::uniform<T>() takes a floating point type");
            return std::uniform_real_distribution<T>(T(0), T(1))(engine());
        }
        template <typename T>
        T normal() const {
            static_assert(std::is_floating_point<T>::value, "HostRandom::normal<T>() takes a floating point type");
            return std::normal_distribution<T>(T(0), T(1))(engine());
        }
        template <typename T>
        T logNormal(T mean, T stddev) const {
            static_assert(std::is_floating_point<T>::value, "HostRandom::logNormal<T>() takes a floating point type");
            return std::lognormal_distribution<T>(mean, stddev)(engine());
        }
        /** An integer in [min, max] (HostRandom.cuh:96-140). */
        template <typename T>
        T uniform(T min, T max) const {
            static_assert(std::is_integral<T>::value, "HostRandom::uniform<T>(min, max) takes an integer type");
            using W = typename std::conditional<std::is_signed<T>::value, int64_t, uint64_t>::type;
            return static_cast<T>(std::uniform_int_distribution<W>(static_cast<W>(min), static_cast<W>(max))(engine()));
        }
        template <typename T = unsigned int>
        unsigned int poisson(double mean = 1.0) const {
            return static_cast<unsigned int>(std::poisson_distribution<unsigned int>(mean)(engine()));
        }
        void setSeed(uint64_t seed);
        uint64_t getSeed() const;

     private:
        std::mt19937_64& engine() const;
        detail::SimulationImpl* sim;
    };
    /** HostAgentAPI (include/flamegpu/runtime/agent/HostAgentAPI.cuh:134-227). */
    class AgentAPI {
     public:
        AgentAPI(detail::SimulationImpl* s, std::string a, std::string st) : sim(s), agent(std::move(a)), state(std::move(st)) {}
        unsigned int count() const;
        /** A new agent of this type and state (HostAgentAPI::newAgent, :160). */
        HostNewAgentAPI newAgent();
        /** HostAgentAPI::getPopulationData (HostAgentAPI.cuh:227-236): the
         *  population, read back from the device. What the host function
         *  changes in it, agents added (fresh ids for those without one) and
         *  removed included, replaces the population when the host function
         *  returns, before the agents made with newAgent() join it. */
        AgentVector& getPopulationData();
        /** Sum of a variable over the population (:174-185): accumulated on
         * the device in a fixed order (double for floating point, 64-bit
         * integers otherwise), returned as OutT. */
        template <typename InT>
        InT sum(const std::string& variable) const { return sum<InT, InT>(variable); }
        template <typename InT, typename OutT>
        OutT sum(const std::string& variable) const {
            return convert<OutT>(reduce_log(variable, typeid(InT), LoggingConfig::Sum));
        }
        /** Smallest / largest value of a variable (:206-216; 0 for an empty population). */
        template <typename InT>
        InT min(const std::string& variable) const { return convert<InT>(reduce_log(variable, typeid(InT), LoggingConfig::Min)); }
        template <typename InT>
        InT max(const std::string& variable) const { return convert<InT>(reduce_log(variable, typeid(InT), LoggingConfig::Max)); }
        /** Mean and population standard deviation (:196). */
        template <typename InT>
        std::pair<double, double> meanStandardDeviation(const std::string& variable) const {
            return {convert<double>(reduce_log(variable, typeid(InT), LoggingConfig::Mean)),
                    convert<double>(reduce_log(variable, typeid(InT), LoggingConfig::StandardDev))};
        }
        // The templates below launch kernels, so their definitions are in
        // flamegpu/runtime/HostReductions.cuh (included by flamegpu.h when
        // compiled by nvcc).
        /** Agents whose variable equals value (:226-227). */
        template <typename InT>
        unsigned int count(const std::string& variable, InT value) const;
        /** Counts of the variable's values in histogramBins equal bins over
         * [lowerBound, upperBound); values outside are not counted (:240-243). */
        template <typename InT>
        std::vector<unsigned int> histogramEven(const std::string& variable, unsigned int histogramBins,
                                                InT lowerBound, InT upperBound) const;
        template <typename InT, typename OutT>
        std::vector<OutT> histogramEven(const std::string& variable, unsigned int histogramBins, InT lowerBound,
                                        InT upperBound) const;
        /** Reduction of the variable by a FLAMEGPU_CUSTOM_REDUCTION operator,
         * init combined once with the result (init alone for no agents) (:254-255). */
        template <typename InT, typename ReductionT>
        InT reduce(const std::string& variable, ReductionT reductionOperator, InT init) const;
        /** The same over each value transformed by a FLAMEGPU_CUSTOM_TRANSFORM operator (:267-268). */
        template <typename InT, typename OutT, typename TransformT, typename ReductionT>
        OutT transformReduce(const std::string& variable, TransformT transformOperator, ReductionT reductionOperator,
                             OutT init) const;

        /** HostAgentAPI::Order (HostAgentAPI.cuh:131). */
        enum Order { Asc = 0, Desc = 1 };
        /** Sorts the population by a scalar variable (HostAgentAPI.cuh:287-290):
         *  stable, ascending or descending, on bits [beginBit, endBit) of the key. */
        template <typename VarT>
        void sort(const std::string& variable, Order order, int beginBit = 0, int endBit = sizeof(VarT) * 8) {
            static_assert(std::is_arithmetic<VarT>::value && sizeof(VarT) <= 8, "HostAgentAPI::sort takes a scalar type");
            const uint32_t kind = std::is_floating_point<VarT>::value ? 2u : (std::is_signed<VarT>::value ? 1u : 0u);
            sort_by(variable, typeid(VarT), kind, sizeof(VarT), order == Desc, beginBit, endBit);
        }
        /** By variable1, ties by variable2 (HostAgentAPI.cuh:301-302). */
        template <typename Var1T, typename Var2T>
        void sort(const std::string& variable1, Order order1, const std::string& variable2, Order order2) {
            sort<Var2T>(variable2, order2);
            sort<Var1T>(variable1, order1);
        }

     private:
        void sort_by(const std::string& variable, const std::type_info& t, uint32_t kind, uint32_t bytes, bool descending,
                     int begin_bit, int end_bit);
        LogValue reduce_log(const std::string& variable, const std::type_info& t, LoggingConfig::Reduction r) const;
        // The device column of a scalar variable of type t (the checks of the
        // reductions), the population count on the device, and the stream.
        const void* device_column(const std::string& variable, const std::type_info& t, const uint32_t** d_n,
                                  cudaStream_t* stream) const;
        template <typename OutT>
        static OutT convert(const LogValue& v) {
            const auto t = v.type;
            if (t == std::type_index(typeid(double))) return static_cast<OutT>(v.as<double>("reduction"));
            if (t == std::type_index(typeid(float))) return static_cast<OutT>(v.as<float>("reduction"));
            if (t == std::type_index(typeid(int64_t))) return static_cast<OutT>(v.as<int64_t>("reduction"));
            if (t == std::type_index(typeid(uint64_t))) return static_cast<OutT>(v.as<uint64_t>("reduction"));
            if (t == std::type_index(typeid(int32_t))) return static_cast<OutT>(v.as<int32_t>("reduction"));
            if (t == std::type_index(typeid(uint32_t))) return static_cast<OutT>(v.as<uint32_t>("reduction"));
            if (t == std::type_index(typeid(int16_t))) return static_cast<OutT>(v.as<int16_t>("reduction"));
            if (t == std::type_index(typeid(uint16_t))) return static_cast<OutT>(v.as<uint16_t>("reduction"));
            if (t == std::type_index(typeid(int8_t))) return static_cast<OutT>(v.as<int8_t>("reduction"));
            return static_cast<OutT>(v.as<uint8_t>("reduction"));
        }
        detail::SimulationImpl* sim;
        std::string agent, state;
    };
    explicit HostAPI(detail::SimulationImpl* s) : environment(s), random(s), sim(s) {}
    AgentAPI agent(const std::string& name, const std::string& state = "default") { return AgentAPI(sim, name, state); }
    unsigned int getStepCounter() const;
    Environment environment;
    Random random;

 private:
    detail::SimulationImpl* sim;
};

/** The reference's names of the host API's parts. */
using HostAgentAPI = HostAPI::AgentAPI;
using HostEnvironment = HostAPI::Environment;
using HostRandom = HostAPI::Random;

class CUDASimulation {
 public:
    /** Simulation::Config (include/flamegpu/simulation/Simulation.h:37-70). */
    struct SimConfig {
        unsigned int steps = 1;
        uint64_t random_seed = 0;
        std::string input_file;  // state file (JSON) loaded by applyConfig()
        // kept and written to state files as the reference's Simulation::Config
        // (include/flamegpu/simulation/Simulation.h:55-63) holds them
        std::string step_log_file;
        std::string exit_log_file;
        std::string common_log_file;
        bool truncate_log_files = false;
        unsigned int verbosity = 1;  // Verbosity::Quiet 0, Default 1, Verbose 2
        bool verbose = false;
        bool timing = false;
    };
    /** CUDASimulation::Config (CUDASimulation.h:100-128) plus the GB300 switches. */
    struct Config {
        int device_id = 0;
        bool inLayerConcurrency = true;
        bool use_graphs = true;       // capture each step into a CUDA graph and replay it
        bool check_each_step = false; // synchronise and check device errors after every step()
        bool profile_ops = false;     // issue steps eagerly and time every operation with CUDA events
        // Capture a pair of timing events around every operation into the step
        // graphs; harvestOperationTimes() adds the times of the last replay of
        // each graph to the operation profile. Steps stay graph replays.
        bool time_ops_in_graphs = false;
        // One operation (a label of the operation profile, e.g. "fn:inputdata")
        // timed the same way while steps stay replayed several per graph:
        // only its launches are bracketed by events, every replay's are read
        // by harvestOperationTimes(). Empty: off.
        std::string time_op_label;
        unsigned int message_stage_bytes = 96u * 1024u;  // shared memory per block for spatial neighbour windows (0: off)
        // Largest population an agent list may reach, births included: buffers
        // never grow past it, and a step that could exceed it (checked when the
        // buffers would have to grow) throws exception::OutOfMemory (0: no limit
        // below 2^31). Bounds the memory of a served run.
        unsigned int max_agents = 0;
        // Priority of the simulation's streams (cudaStreamCreateWithPriority: a
        // lower number runs first when kernels of several streams are waiting).
        int stream_priority = 0;
        // Threads per agent-function block: 32, 64 or 128 (0: 128). The
        // reference picks a block size per launch with
        // cudaOccupancyMaxPotentialBlockSize (CUDASimulation.cu:988).
        unsigned int agent_block = 0;
    };

    explicit CUDASimulation(const ModelDescription& model, int argc = 0, const char** argv = nullptr);
    ~CUDASimulation();
    CUDASimulation(const CUDASimulation&) = delete;
    CUDASimulation& operator=(const CUDASimulation&) = delete;

    SimConfig& SimulationConfig();
    Config& CUDAConfig();
    /** Applies the configuration; loads SimulationConfig().input_file if set. */
    void applyConfig();
    /** Simulation::exportData (include/flamegpu/simulation/Simulation.h): writes
     *  the configuration, step counter, environment and every population to a
     *  JSON state file in the reference's layout. */
    void exportData(const std::string& path);
    /** Reads a JSON state file (the reference's layout): the populations it
     *  holds replace those lists, environment properties, the step counter and
     *  the seed/steps configuration it names are set (GB300 extension; the
     *  reference reads it through SimulationConfig().input_file). */
    void loadState(const std::string& path);

    void setPopulationData(AgentVector& population, const std::string& state = "default");
    void getPopulationData(AgentVector& population, const std::string& state = "default");
    /** setPopulationData from named host columns (GB300 extension): every
     *  variable, _id included and set, given as n elements; the columns are
     *  copied straight to the device (asynchronously, then waited for). */
    void setPopulationColumns(const std::string& agent, const std::string& state, uint32_t n,
                              const std::vector<std::pair<std::string, const void*>>& host_columns);
    /** getPopulationData into named host columns of room for `cap` agents
     *  (GB300 extension); returns the population. */
    uint32_t getPopulationColumns(const std::string& agent, const std::string& state,
                                  const std::vector<std::pair<std::string, void*>>& host_columns, uint32_t cap);

    /** One step (all layers). Returns false if an exit condition requests a stop. */
    bool step();
    /** n steps (GB300 extension). When no host work runs between steps (no
     *  host layers, step functions or step log, no births or state changes
     *  whose capacity the host checks), up to 16 steps are replayed as one
     *  captured graph; the results are those of n calls of step(). */
    void step(unsigned int n);
    /** SimulationConfig().steps steps. */
    void simulate();
    unsigned int getStepCounter() const;
    void resetStepCounter();

    double getElapsedTimeSimulation() const;
    /** Agents summed over the steps run so far (all agent types and states,
     *  each step counted with the populations that entered it); waits for the
     *  steps issued. An extension (the reference has no such counter). */
    unsigned long long getAgentStepCount();
    std::vector<double> getElapsedTimeSteps() const;
    double getElapsedTimeStep(unsigned int step) const;

    template <typename T>
    void setEnvironmentProperty(const std::string& name, T value) {
        HostAPI::Environment e(impl.get());
        e.setProperty<T>(name, value);
    }
    template <typename T>
    T getEnvironmentProperty(const std::string& name) {
        HostAPI::Environment e(impl.get());
        return e.getProperty<T>(name);
    }

    // ---- GB300 extensions (device-resident access) ----
    /** Stream every step is issued on. */
    cudaStream_t getStream() const;
    /** Waits for the simulation's stream; throws exception::DeviceError for recorded device errors. */
    void synchronize();
    /** Agents in a state list (synchronises). */
    unsigned int getAgentCount(const std::string& agent, const std::string& state = "default");
    /** Device pointer to the current column of an agent variable (valid until the next step). */
    void* getDeviceVariable(const std::string& agent, const std::string& variable, const std::string& state = "default");
    /** One reduction of an agent variable over its population, on the device
     *  (the step / exit logs' reductions; HostAgentAPI's sum, min, max and
     *  mean / standard deviation use it). GB300 extension. */
    LogValue reduceAgentVariable(const std::string& agent, const std::string& variable, LoggingConfig::Reduction r,
                                 const std::string& state = "default");
    /** Override the bounds and radius of a spatial message list before stepping
     *  (per-run spatial grids of an ensemble). */
    void setSpatialMessageBounds(const std::string& message, const std::vector<float>& min,
                                 const std::vector<float>& max, float radius);
    /** Replace a state list's population from device columns (every variable,
     *  including _id, n rows each); the agent type's next id becomes next_id. */
    void setPopulationDevice(const std::string& agent, const std::string& state, unsigned int n,
                             const std::vector<std::pair<std::string, const void*>>& columns, id_t next_id);
    /** Device pointer to the device-resident agent count of a state list. */
    const unsigned int* getDeviceCount(const std::string& agent, const std::string& state = "default");
    /** Graph replays issued so far (0 when graphs are disabled). */
    unsigned long long getGraphLaunches() const;
    /** Kernel launches issued by the last step (counted at capture / issue). */
    unsigned int getKernelsPerStep() const;
    /** Per-operation device time since the last call ("fn:<name>", "build:<message>",
     *  "sort:<agent>", "compact:<agent>" -> total ms, count); needs CUDAConfig().profile_ops. */
    std::vector<std::tuple<std::string, double, unsigned long long>> takeOperationProfile();
    /** With CUDAConfig().time_ops_in_graphs: waits for the stream, then adds the
     *  operation times of the last replay of each graph replayed since the
     *  previous call to the profile that takeOperationProfile() returns. */
    void harvestOperationTimes();

    /** CUDASimulation::setStepLog / setExitLog / getRunLog (include/flamegpu/simulation/Simulation.h,
     *  CUDASimulation.cu:1949-2022): environment properties, agent counts and
     *  variable reductions logged every `frequency` steps (and once before the
     *  first step of simulate()) and at the end of simulate(). */
    void setStepLog(const StepLoggingConfig& cfg);
    void setExitLog(const LoggingConfig& cfg);
    const RunLog& getRunLog() const { return run_log; }
    /** The run log in the layout of the reference's JSONLogger
     *  (src/flamegpu/io/JSONLogger.cu:80-200): config, performance_specs and
     *  the frames' times (with_times: logStepTime / logExitTime), steps, exit.
     *  An agent's "count" is written as the number (the reference's
     *  j["count"][n] turns it into an array of n + 1 nulls). */
    std::string runLogJSON(bool with_times = true) const;
    /** Raw bytes of an environment property (GB300 extension). */
    void getEnvironmentRaw(const std::string& name, void* out, size_t bytes);
    /** Logs the frame of the step just completed when it is due (called by the step). */
    void processStepLog(double step_seconds);
    /** Logs the exit frame (called at the end of simulate()). */
    void processExitLog(double total_seconds);

    detail::SimulationImpl* getImpl() const { return impl.get(); }
    const std::shared_ptr<detail::ModelData>& getModelData() const;

 private:
    std::unique_ptr<detail::SimulationImpl> impl;
    std::unique_ptr<StepLoggingConfig> step_log;
    std::unique_ptr<LoggingConfig> exit_log;
    RunLog run_log;
    char* log_scratch = nullptr;  // device buffer of the log reductions
};

}  // namespace flamegpu

#endif  // INCLUDE_FLAMEGPU_SIMULATION_CUDASIMULATION_H_
