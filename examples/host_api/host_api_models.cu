// Host-function test models, written against the FLAME GPU 2 API: agents
// created by init functions (HostAgentAPI::newAgent) and reductions of agent
// variables in exit functions (sum, min, max, meanStandardDeviation).
//
// Registered models:
//   ensemble_counter  the model of the reference's TestCUDAEnsemble.simulate
//                     (tests/test_cases/simulation/test_cuda_ensemble.cu:251-316):
//                     an init function creates POPULATION_TO_GENERATE agents
//                     with counter 0, one function adds 1 to each counter per
//                     step, the exit function adds the sum of the counters to a
//                     process-wide total (fg_test_counter_total).
//   ensemble_offset   the model of the reference's ensemble example
//                     (examples/cpp/ensemble/src/main.cu:6-24): x = init + i *
//                     init_offset at creation, x += offset every step, the exit
//                     function writes sum(x) into the property "result" and
//                     adds it and "init" to process-wide totals
//                     (fg_test_offset_totals).
//   host_probe        an init function creates N agents (x = i, f = i / 2,
//                     u = i % 7); the exit function writes count, sum, min,
//                     max, mean and standard deviation into properties.
// Parameters (all models): [0] population to generate.
#include <atomic>
#include <cstdint>

#include "flamegpu/flamegpu.h"
#include "flamegpu_gb300/fg_sim.h"

namespace {
std::atomic<uint64_t> g_counter_total{0};
std::atomic<int64_t> g_offset_result{0};
std::atomic<int64_t> g_offset_init{0};
}  // namespace

extern "C" uint64_t fg_test_counter_total(int reset) {
    return reset ? g_counter_total.exchange(0) : g_counter_total.load();
}
extern "C" void fg_test_offset_totals(int64_t* init_sum, int64_t* result_sum, int reset) {
    *init_sum = reset ? g_offset_init.exchange(0) : g_offset_init.load();
    *result_sum = reset ? g_offset_result.exchange(0) : g_offset_result.load();
}

FLAMEGPU_AGENT_FUNCTION(count_step, flamegpu::MessageNone, flamegpu::MessageNone) {
    FLAMEGPU->setVariable<uint32_t>("counter", FLAMEGPU->getVariable<uint32_t>("counter") + 1);
    return flamegpu::ALIVE;
}
FLAMEGPU_INIT_FUNCTION(counter_init) {
    const uint32_t n = FLAMEGPU->environment.getProperty<uint32_t>("POPULATION_TO_GENERATE");
    auto agent = FLAMEGPU->agent("Agent");
    for (uint32_t i = 0; i < n; ++i) agent.newAgent().setVariable<uint32_t>("counter", 0);
}
FLAMEGPU_EXIT_FUNCTION(counter_exit) {
    g_counter_total += FLAMEGPU->agent("Agent").sum<uint32_t, uint64_t>("counter");
}

FLAMEGPU_AGENT_FUNCTION(add_offset, flamegpu::MessageNone, flamegpu::MessageNone) {
    FLAMEGPU->setVariable<int>("x", FLAMEGPU->getVariable<int>("x") + FLAMEGPU->environment.getProperty<int>("offset"));
    return flamegpu::ALIVE;
}
FLAMEGPU_INIT_FUNCTION(offset_init) {
    const uint32_t n = FLAMEGPU->environment.getProperty<uint32_t>("POPULATION_TO_GENERATE");
    const int init = FLAMEGPU->environment.getProperty<int>("init");
    const int init_offset = FLAMEGPU->environment.getProperty<int>("init_offset");
    auto agent = FLAMEGPU->agent("Agent");
    for (uint32_t i = 0; i < n; ++i) agent.newAgent().setVariable<int>("x", init + static_cast<int>(i) * init_offset);
}
FLAMEGPU_EXIT_FUNCTION(offset_exit) {
    const int result = FLAMEGPU->agent("Agent").sum<int>("x");
    FLAMEGPU->environment.setProperty<int>("result", result);
    g_offset_result += result;
    g_offset_init += FLAMEGPU->environment.getProperty<int>("init");
}

FLAMEGPU_AGENT_FUNCTION(probe_nothing, flamegpu::MessageNone, flamegpu::MessageNone) { return flamegpu::ALIVE; }
FLAMEGPU_INIT_FUNCTION(probe_init) {
    const uint32_t n = FLAMEGPU->environment.getProperty<uint32_t>("POPULATION_TO_GENERATE");
    auto agent = FLAMEGPU->agent("a");
    for (uint32_t i = 0; i < n; ++i) {
        auto a = agent.newAgent();
        a.setVariable<int>("x", static_cast<int>(i) - 100);
        a.setVariable<float>("f", static_cast<float>(i) * 0.5f);
        a.setVariable<uint32_t>("u", i % 7u);
    }
}
FLAMEGPU_EXIT_FUNCTION(probe_exit) {
    auto a = FLAMEGPU->agent("a");
    FLAMEGPU->environment.setProperty<uint32_t>("count", a.count());
    FLAMEGPU->environment.setProperty<int64_t>("sum_x", a.sum<int, int64_t>("x"));
    FLAMEGPU->environment.setProperty<int>("sum_x_int", a.sum<int>("x"));
    FLAMEGPU->environment.setProperty<int>("min_x", a.min<int>("x"));
    FLAMEGPU->environment.setProperty<int>("max_x", a.max<int>("x"));
    FLAMEGPU->environment.setProperty<uint32_t>("max_u", a.max<uint32_t>("u"));
    FLAMEGPU->environment.setProperty<double>("sum_f", a.sum<float, double>("f"));
    const auto ms = a.meanStandardDeviation<float>("f");
    FLAMEGPU->environment.setProperty<double>("mean_f", ms.first);
    FLAMEGPU->environment.setProperty<double>("sd_f", ms.second);
}

namespace {

void* make_counter(const double* p, int32_t np) {
    auto* m = new flamegpu::ModelDescription("test");
    m->Environment().newProperty<uint32_t>("POPULATION_TO_GENERATE", np > 0 ? static_cast<uint32_t>(p[0]) : 32u, true);
    flamegpu::AgentDescription agent = m->newAgent("Agent");
    agent.newVariable<uint32_t>("counter", 0);
    flamegpu::AgentFunctionDescription f = agent.newFunction("count_step", count_step);
    m->newLayer().addAgentFunction(f);
    m->addInitFunction(counter_init);
    m->addExitFunction(counter_exit);
    return m;
}

void* make_offset(const double* p, int32_t np) {
    auto* m = new flamegpu::ModelDescription("ensemble_offset");
    flamegpu::EnvironmentDescription env = m->Environment();
    env.newProperty<uint32_t>("POPULATION_TO_GENERATE", np > 0 ? static_cast<uint32_t>(p[0]) : 1000u, true);
    env.newProperty<int>("init", 0);
    env.newProperty<int>("init_offset", 0);
    env.newProperty<int>("offset", 1);
    env.newProperty<int>("result", 0);
    flamegpu::AgentDescription agent = m->newAgent("Agent");
    agent.newVariable<int>("x");
    flamegpu::AgentFunctionDescription f = agent.newFunction("add_offset", add_offset);
    m->newLayer().addAgentFunction(f);
    m->addInitFunction(offset_init);
    m->addExitFunction(offset_exit);
    return m;
}

void* make_probe(const double* p, int32_t np) {
    auto* m = new flamegpu::ModelDescription("host_probe");
    flamegpu::EnvironmentDescription env = m->Environment();
    env.newProperty<uint32_t>("POPULATION_TO_GENERATE", np > 0 ? static_cast<uint32_t>(p[0]) : 1000u, true);
    env.newProperty<uint32_t>("count", 0u);
    env.newProperty<int64_t>("sum_x", 0);
    env.newProperty<int>("sum_x_int", 0);
    env.newProperty<int>("min_x", 0);
    env.newProperty<int>("max_x", 0);
    env.newProperty<uint32_t>("max_u", 0u);
    env.newProperty<double>("sum_f", 0.0);
    env.newProperty<double>("mean_f", 0.0);
    env.newProperty<double>("sd_f", 0.0);
    flamegpu::AgentDescription a = m->newAgent("a");
    a.newVariable<int>("x", 0);
    a.newVariable<float>("f", 0.0f);
    a.newVariable<uint32_t>("u", 0u);
    flamegpu::AgentFunctionDescription f = a.newFunction("probe_nothing", probe_nothing);
    m->newLayer().addAgentFunction(f);
    m->addInitFunction(probe_init);
    m->addExitFunction(probe_exit);
    return m;
}

struct Register {
    Register() {
        fgs_register_model("ensemble_counter", &make_counter);
        fgs_register_model("ensemble_offset", &make_offset);
        fgs_register_model("host_probe", &make_probe);
    }
} reg;

}  // namespace
