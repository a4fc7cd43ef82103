// Host-triggered agent sorts (HostAgentAPI::sort, HostAgentAPI.cuh:287-302),
// written against the FLAME GPU 2 API. Registered model:
//   host_sort  params: [mode]. Agent "agent" with k (its row before the
//              sort), f (float), d (double), i (int32_t), u (uint64_t),
//              c (int8_t), h (uint16_t); a step function sorts the
//              population: 0 f ascending, 1 f descending, 2 i ascending then
//              f descending, 3 u descending, 4 c ascending, 5 d ascending on
//              bits [4, 60), 6 h descending.
#include <cstdint>

#include "flamegpu/flamegpu.h"
#include "flamegpu_gb300/fg_sim.h"

FLAMEGPU_STEP_FUNCTION(host_sort_step) {
    flamegpu::HostAgentAPI a = FLAMEGPU->agent("agent");
    switch (FLAMEGPU->environment.getProperty<int>("mode")) {
        case 0: a.sort<float>("f", flamegpu::HostAgentAPI::Asc); break;
        case 1: a.sort<float>("f", flamegpu::HostAgentAPI::Desc); break;
        case 2: a.sort<int32_t, float>("i", flamegpu::HostAgentAPI::Asc, "f", flamegpu::HostAgentAPI::Desc); break;
        case 3: a.sort<uint64_t>("u", flamegpu::HostAgentAPI::Desc); break;
        case 4: a.sort<int8_t>("c", flamegpu::HostAgentAPI::Asc); break;
        case 5: a.sort<double>("d", flamegpu::HostAgentAPI::Asc, 4, 60); break;
        default: a.sort<uint16_t>("h", flamegpu::HostAgentAPI::Desc); break;
    }
}

FLAMEGPU_AGENT_FUNCTION(host_sort_nothing, flamegpu::MessageNone, flamegpu::MessageNone) { return flamegpu::ALIVE; }

namespace {

void* make_host_sort(const double* p, int32_t np) {
    auto* m = new flamegpu::ModelDescription("host_sort");
    m->Environment().newProperty<int>("mode", np > 0 ? static_cast<int>(p[0]) : 0);
    flamegpu::AgentDescription a = m->newAgent("agent");
    a.newVariable<uint32_t>("k");
    a.newVariable<float>("f");
    a.newVariable<double>("d");
    a.newVariable<int32_t>("i");
    a.newVariable<uint64_t>("u");
    a.newVariable<int8_t>("c");
    a.newVariable<uint16_t>("h");
    m->newLayer().addAgentFunction(a.newFunction("nothing", host_sort_nothing));
    m->addStepFunction(host_sort_step);
    return m;
}

struct Register {
    Register() { fgs_register_model("host_sort", &make_host_sort); }
} reg;

}  // namespace
