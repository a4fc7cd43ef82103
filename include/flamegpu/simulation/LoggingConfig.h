#ifndef INCLUDE_FLAMEGPU_SIMULATION_LOGGINGCONFIG_H_
#define INCLUDE_FLAMEGPU_SIMULATION_LOGGINGCONFIG_H_
// Step / exit logging with the reference's names
// (include/flamegpu/simulation/LoggingConfig.h, AgentLoggingConfig.h,
// LogFrame.h, RunLog.h): per logged step, environment properties, agent counts
// and reductions (mean, standard deviation, min, max, sum) of agent variables.
// Reductions run on the device (deterministic two-level reductions); sums are
// double for floating-point variables and 64-bit for integer ones, as the
// reference's sum_input_t (AgentLoggingConfig_SumReturn.h:14-60).
#include <cstdint>
#include <cstring>
#include <list>
#include <map>
#include <memory>
#include <string>
#include <type_traits>
#include <typeindex>
#include <utility>
#include <vector>

#include "flamegpu/exception/FLAMEGPUException.h"
#include "flamegpu/model/ModelDescription.h"

namespace flamegpu {

template <typename T>
struct sum_input_t {
    typedef typename std::conditional<std::is_floating_point<T>::value, double,
                                      typename std::conditional<std::is_signed<T>::value, int64_t, uint64_t>::type>::type
        result_t;
};

class LoggingConfig {
 public:
    enum Reduction { Mean, StandardDev, Min, Max, Sum };
    static constexpr const char* toString(const Reduction& r) {
        switch (r) {
            case Mean: return "mean";
            case StandardDev: return "standard_deviation";
            case Min: return "min";
            case Max: return "max";
            case Sum: return "sum";
            default: return "unknown";
        }
    }
    struct NameReduction {
        std::string name;
        Reduction reduction;
        bool operator<(const NameReduction& o) const {
            return name < o.name || (name == o.name && reduction < o.reduction);
        }
    };
    struct AgentEntry {
        bool count = false;
        std::vector<NameReduction> reductions;
    };

    /** LoggingConfig(model) (LoggingConfig.h:83). */
    explicit LoggingConfig(const ModelDescription& model) : model_(model.getData()) {}
    class AgentLoggingConfig;
    /** LoggingConfig::agent (LoggingConfig.h:97): what to log of one agent state. */
    AgentLoggingConfig agent(const std::string& agent_name, const std::string& state = "");
    /** LoggingConfig::logEnvironment (LoggingConfig.h:105). */
    void logEnvironment(const std::string& property_name);
    /** LoggingConfig::logTiming (LoggingConfig.h:110). */
    void logTiming(bool log_timing) { timing_ = log_timing; }

    // read by the simulation
    const std::shared_ptr<detail::ModelData>& model() const { return model_; }
    const std::map<std::pair<std::string, std::string>, AgentEntry>& agents() const { return agents_; }
    const std::vector<std::string>& environment() const { return environment_; }
    bool timing() const { return timing_; }

 protected:
    std::shared_ptr<detail::ModelData> model_;
    std::map<std::pair<std::string, std::string>, AgentEntry> agents_;
    std::vector<std::string> environment_;
    bool timing_ = false;
};

/** AgentLoggingConfig (AgentLoggingConfig.h:22-100): reductions of one agent state. */
class LoggingConfig::AgentLoggingConfig {
 public:
    AgentLoggingConfig(LoggingConfig* cfg, const detail::AgentData* agent, std::pair<std::string, std::string> key)
        : cfg_(cfg), agent_(agent), key_(std::move(key)) {}
    void logCount() { cfg_->agents_[key_].count = true; }
    template <typename T>
    void logMean(const std::string& variable) { add<T>(variable, Mean); }
    template <typename T>
    void logStandardDev(const std::string& variable) { add<T>(variable, StandardDev); }
    template <typename T>
    void logMin(const std::string& variable) { add<T>(variable, Min); }
    template <typename T>
    void logMax(const std::string& variable) { add<T>(variable, Max); }
    template <typename T>
    void logSum(const std::string& variable) { add<T>(variable, Sum); }

 private:
    template <typename T>
    void add(const std::string& variable, Reduction r) {
        const detail::Variable* v = agent_->find(variable);
        if (!v)
            THROW exception::InvalidAgentVar(exception::format("Agent '%s' has no variable '%s'", agent_->name.c_str(),
                                                               variable.c_str()));
        if (v->type != std::type_index(typeid(T)))
            THROW exception::InvalidVarType(exception::format("Variable '%s' is not of the logged type", variable.c_str()));
        if (v->elements != 1)
            THROW exception::InvalidVarType(exception::format("Variable '%s' is an array; reductions need scalars",
                                                              variable.c_str()));
        cfg_->agents_[key_].reductions.push_back({variable, r});
    }
    LoggingConfig* cfg_;
    const detail::AgentData* agent_;
    std::pair<std::string, std::string> key_;
};

inline LoggingConfig::AgentLoggingConfig LoggingConfig::agent(const std::string& agent_name, const std::string& state) {
    const detail::AgentData* a = nullptr;
    for (const auto& x : model_->agents)
        if (x->name == agent_name) a = x.get();
    if (!a) THROW exception::InvalidAgentName(exception::format("Model has no agent '%s'", agent_name.c_str()));
    const std::string st = state.empty() ? a->initial_state : state;
    bool has = false;
    for (const auto& s : a->states) has = has || s == st;
    if (!has) THROW exception::InvalidAgentState(exception::format("Agent '%s' has no state '%s'", agent_name.c_str(), st.c_str()));
    agents_[{agent_name, st}];
    return AgentLoggingConfig(this, a, {agent_name, st});
}

inline void LoggingConfig::logEnvironment(const std::string& property_name) {
    for (const auto& p : model_->environment)
        if (p.name == property_name) {
            environment_.push_back(property_name);
            return;
        }
    THROW exception::InvalidEnvProperty(exception::format("Environment has no property '%s'", property_name.c_str()));
}

/** StepLoggingConfig (StepLoggingConfig.h): a LoggingConfig applied every `frequency` steps. */
class StepLoggingConfig : public LoggingConfig {
 public:
    explicit StepLoggingConfig(const ModelDescription& model) : LoggingConfig(model) {}
    explicit StepLoggingConfig(const LoggingConfig& other) : LoggingConfig(other) {}
    void setFrequency(unsigned int steps) { frequency_ = steps ? steps : 1; }
    unsigned int frequency() const { return frequency_; }

 private:
    unsigned int frequency_ = 1;
};

/** One logged value: raw bytes of its C++ type. */
struct LogValue {
    std::type_index type = std::type_index(typeid(void));
    std::vector<char> bytes;
    uint32_t elements = 1;
    template <typename T>
    T as(const std::string& what) const {
        if (type != std::type_index(typeid(T)) || bytes.size() < sizeof(T))
            THROW exception::InvalidVarType(exception::format("Logged value '%s' has another type", what.c_str()));
        T v;
        std::memcpy(&v, bytes.data(), sizeof(T));
        return v;
    }
};

/** AgentLogFrame (LogFrame.h:112-200): the logged count and reductions of one agent state. */
class AgentLogFrame {
 public:
    AgentLogFrame() = default;
    AgentLogFrame(const std::map<LoggingConfig::NameReduction, LogValue>* data, unsigned int count)
        : data_(data), count_(count) {}
    unsigned int getCount() const {
        if (count_ == ~0u) THROW exception::InvalidOperation("Agent count was not logged");
        return count_;
    }
    template <typename T>
    T getMin(const std::string& variable) const { return get(variable, LoggingConfig::Min).as<T>(variable); }
    template <typename T>
    T getMax(const std::string& variable) const { return get(variable, LoggingConfig::Max).as<T>(variable); }
    template <typename T>
    typename sum_input_t<T>::result_t getSum(const std::string& variable) const {
        return get(variable, LoggingConfig::Sum).as<typename sum_input_t<T>::result_t>(variable);
    }
    double getMean(const std::string& variable) const { return get(variable, LoggingConfig::Mean).as<double>(variable); }
    double getStandardDev(const std::string& variable) const {
        return get(variable, LoggingConfig::StandardDev).as<double>(variable);
    }

 private:
    const LogValue& get(const std::string& variable, LoggingConfig::Reduction r) const {
        auto it = data_->find({variable, r});
        if (it == data_->end())
            THROW exception::InvalidAgentVar(exception::format("Variable '%s' was not logged with '%s'", variable.c_str(),
                                                               LoggingConfig::toString(r)));
        return it->second;
    }
    const std::map<LoggingConfig::NameReduction, LogValue>* data_ = nullptr;
    unsigned int count_ = ~0u;
};

/** LogFrame (LogFrame.h:20-110): what was logged at one step. */
class LogFrame {
 public:
    LogFrame() = default;
    unsigned int getStepCount() const { return step_count; }
    bool hasEnvironmentProperty(const std::string& name) const { return environment.count(name) != 0; }
    template <typename T>
    T getEnvironmentProperty(const std::string& name) const {
        auto it = environment.find(name);
        if (it == environment.end())
            THROW exception::InvalidEnvProperty(exception::format("Environment property '%s' was not logged", name.c_str()));
        return it->second.as<T>(name);
    }
    AgentLogFrame getAgent(const std::string& agent_name, const std::string& state = "default") const {
        auto it = agents.find({agent_name, state});
        if (it == agents.end())
            THROW exception::InvalidAgentState(exception::format("Agent '%s' state '%s' was not logged", agent_name.c_str(),
                                                                 state.c_str()));
        return AgentLogFrame(&it->second.first, it->second.second);
    }

    unsigned int step_count = 0;
    std::map<std::string, LogValue> environment;
    std::map<std::pair<std::string, std::string>, std::pair<std::map<LoggingConfig::NameReduction, LogValue>, unsigned int>>
        agents;
};

class StepLogFrame : public LogFrame {
 public:
    double getStepTime() const { return step_time; }
    double step_time = 0.0;
};

class ExitLogFrame : public LogFrame {
 public:
    double getTotalTime() const { return total_time; }
    // run-time compilation (none here: 0), init and exit function seconds
    double getRTCTime() const { return rtc_time; }
    double getInitTime() const { return init_time; }
    double getExitTime() const { return exit_time; }
    double total_time = 0.0;
    double rtc_time = 0.0, init_time = 0.0, exit_time = 0.0;
};

/** RunLog (RunLog.h): the step frames and exit frame of one run. */
class RunLog {
 public:
    const std::list<StepLogFrame>& getStepLog() const { return step; }
    const ExitLogFrame& getExitLog() const { return exit; }
    unsigned int getStepLogFrequency() const { return step_log_frequency; }
    uint64_t getRandomSeed() const { return random_seed; }

    std::list<StepLogFrame> step;
    ExitLogFrame exit;
    unsigned int step_log_frequency = 0;
    uint64_t random_seed = 0;
};

}  // namespace flamegpu

#endif  // INCLUDE_FLAMEGPU_SIMULATION_LOGGINGCONFIG_H_
