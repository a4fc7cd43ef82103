// A host function editing a population through HostAgentAPI::getPopulationData
// (DeviceAgentVector), written against the FLAME GPU 2 API: the calls of the
// reference's tests tests/test_cases/runtime/agent/test_device_agent_vector.cu
// (read, update, erase, push_back inside a host function).
//
// Registered model "host_population": agent "agent" (x, y: int).
//   layer 1, host function: every agent's x += 1; the agents whose new x is a
//            multiple of 5 are erased; three agents with x = 1000, 1001, 1002
//            (no id: fresh ids) are appended.
//   layer 2, agent function: y = 2 * x.
//   step function: reads the population back and counts agents whose y is not
//            2 * x (fg_test_host_population_errors()).
#include <cstdint>
#include <mutex>

#include "flamegpu/flamegpu.h"
#include "flamegpu_gb300/fg_sim.h"

namespace {
std::mutex g_mu;
unsigned int g_errors = 0;
}  // namespace

FLAMEGPU_HOST_FUNCTION(hp_edit) {
    flamegpu::DeviceAgentVector av = FLAMEGPU->agent("agent").getPopulationData();
    for (auto a : av) a.setVariable<int>("x", a.getVariable<int>("x") + 1);
    for (flamegpu::size_type i = av.size(); i-- > 0;)
        if (av[i].getVariable<int>("x") % 5 == 0) av.erase(i);
    for (int k = 0; k < 3; ++k) {
        av.push_back();
        av.back().setVariable<int>("x", 1000 + k);
    }
}
FLAMEGPU_AGENT_FUNCTION(hp_double, flamegpu::MessageNone, flamegpu::MessageNone) {
    FLAMEGPU->setVariable<int>("y", 2 * FLAMEGPU->getVariable<int>("x"));
    return flamegpu::ALIVE;
}
FLAMEGPU_STEP_FUNCTION(hp_check) {
    std::lock_guard<std::mutex> lock(g_mu);
    flamegpu::DeviceAgentVector av = FLAMEGPU->agent("agent").getPopulationData();
    for (const auto& a : av)
        if (a.getVariable<int>("y") != 2 * a.getVariable<int>("x")) ++g_errors;
    if (av.size() != FLAMEGPU->agent("agent").count()) ++g_errors;
}

// The view reaches the device before a reduction or sort reads the population,
// and a sort reorders the view (test_device_agent_vector.cu HostReduceAutoSync).
FLAMEGPU_STEP_FUNCTION(hp_autosync) {
    std::lock_guard<std::mutex> lock(g_mu);
    flamegpu::HostAgentAPI agent = FLAMEGPU->agent("agent");
    flamegpu::DeviceAgentVector av = agent.getPopulationData();
    long long want = 0;
    for (auto a : av) {
        a.setVariable<int>("x", a.getVariable<int>("x") + 10);
        want += a.getVariable<int>("x");
    }
    if (agent.sum<int, long long>("x") != want) ++g_errors;
    av.push_back();
    av.back().setVariable<int>("x", -5);
    if (agent.count() != av.size()) ++g_errors;
    if (agent.min<int>("x") != -5) ++g_errors;
    agent.sort<int>("x", flamegpu::HostAgentAPI::Desc);
    for (flamegpu::size_type i = 1; i < av.size(); ++i)
        if (av[i - 1].getVariable<int>("x") < av[i].getVariable<int>("x")) ++g_errors;
    if (av.back().getVariable<int>("x") != -5) ++g_errors;
}

// test_device_agent_vector.cu Insert: n copies of agent 0 inserted n / 2 from the end.
FLAMEGPU_STEP_FUNCTION(hp_insert) {
    flamegpu::DeviceAgentVector av = FLAMEGPU->agent("agent").getPopulationData();
    const flamegpu::size_type n = av.size();
    if (n == 0) return;
    flamegpu::AgentInstance ai(av[0]);
    av.insert(av.size() - n / 2, n, ai);
}

namespace {
void* make_host_population_insert(const double*, int32_t) {
    auto* m = new flamegpu::ModelDescription("host_population_insert");
    flamegpu::AgentDescription a = m->newAgent("agent");
    a.newVariable<int>("x", 0);
    a.newVariable<int>("y", 0);
    m->addStepFunction(hp_insert);
    return m;
}
void* make_host_population_sync(const double*, int32_t) {
    auto* m = new flamegpu::ModelDescription("host_population_sync");
    flamegpu::AgentDescription a = m->newAgent("agent");
    a.newVariable<int>("x", 0);
    a.newVariable<int>("y", 0);
    m->addStepFunction(hp_autosync);
    return m;
}
void* make_host_population(const double*, int32_t) {
    auto* m = new flamegpu::ModelDescription("host_population");
    flamegpu::AgentDescription a = m->newAgent("agent");
    a.newVariable<int>("x", 0);
    a.newVariable<int>("y", 0);
    m->newLayer().addHostFunction(hp_edit);
    m->newLayer().addAgentFunction(a.newFunction("double", hp_double));
    m->addStepFunction(hp_check);
    return m;
}
struct Register {
    Register() {
        fgs_register_model("host_population", &make_host_population);
        fgs_register_model("host_population_sync", &make_host_population_sync);
        fgs_register_model("host_population_insert", &make_host_population_insert);
    }
} reg;
}  // namespace

extern "C" unsigned int fg_test_host_population_errors(int reset) {
    std::lock_guard<std::mutex> lock(g_mu);
    const unsigned int e = g_errors;
    if (reset) g_errors = 0;
    return e;
}
