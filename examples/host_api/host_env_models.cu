// Host environment arrays and host random numbers, written against the FLAME
// GPU 2 API as the reference's host_functions example uses them
// (examples/cpp/host_functions/src/main.cu:8-62: HostAgentAPI, array
// environment properties by element, histogramEven, FLAMEGPU->random).
//
// Registered model:
//   host_env_random  environment "u64" (uint64_t[3] = {11, 12, 13}), "arr"
//                    (int[4] = {1, 2, 3, 4}) and result properties; agent
//                    "agent" (x). The init function sums "u64" element by
//                    element and as an array, sets arr[2] = 30 and checks the
//                    old value, replaces "arr" from a vector, and records
//                    the agent count through a HostAgentAPI. The step function
//                    draws one of each host random kind into properties
//                    (r_uniform, r_normal, r_lognormal, r_int in [1, 10],
//                    r_poisson) and the histogram of x over 8 bins of
//                    [-0.5, 1023.5) into "hist".
#include <array>
#include <cstdint>
#include <vector>

#include "flamegpu/flamegpu.h"
#include "flamegpu_gb300/fg_sim.h"

FLAMEGPU_INIT_FUNCTION(env_init) {
    const uint64_t e0 = FLAMEGPU->environment.getProperty<uint64_t, 3>("u64", 0);
    const uint64_t e1 = FLAMEGPU->environment.getProperty<uint64_t, 3>("u64", 1);
    const uint64_t e2 = FLAMEGPU->environment.getProperty<uint64_t>("u64", 2);
    const std::array<uint64_t, 3> all = FLAMEGPU->environment.getProperty<uint64_t, 3>("u64");
    FLAMEGPU->environment.setProperty<uint64_t>("u64_sum", e0 + e1 + e2);
    FLAMEGPU->environment.setProperty<uint64_t>("u64_sum_array", all[0] + all[1] + all[2]);
    const int old = FLAMEGPU->environment.setProperty<int, 4>("arr", 2, 30);
    FLAMEGPU->environment.setProperty<int>("arr_old2", old);
    const std::vector<int> before = FLAMEGPU->environment.getPropertyArray<int>("arr");
    FLAMEGPU->environment.setProperty<int>("arr_sum_before", before[0] + before[1] + before[2] + before[3]);
    FLAMEGPU->environment.setPropertyArray<int>("arr", std::vector<int>{5, 6, 7, 8});
    flamegpu::HostAgentAPI agent = FLAMEGPU->agent("agent");
    FLAMEGPU->environment.setProperty<uint32_t>("count", agent.count());
}

FLAMEGPU_STEP_FUNCTION(env_step) {
    FLAMEGPU->environment.setProperty<double>("r_uniform", FLAMEGPU->random.uniform<double>());
    FLAMEGPU->environment.setProperty<double>("r_normal", FLAMEGPU->random.normal<double>());
    FLAMEGPU->environment.setProperty<double>("r_lognormal", FLAMEGPU->random.logNormal<double>(1.0, 1.0));
    FLAMEGPU->environment.setProperty<int>("r_int", FLAMEGPU->random.uniform<int>(1, 10));
    FLAMEGPU->environment.setProperty<uint32_t>("r_poisson", FLAMEGPU->random.poisson(3.0));
    const std::vector<unsigned int> h = FLAMEGPU->agent("agent").histogramEven<float>("x", 8, -0.5f, 1023.5f);
    for (int b = 0; b < 8; ++b) FLAMEGPU->environment.setProperty<uint32_t, 8>("hist", b, h[b]);
}

FLAMEGPU_AGENT_FUNCTION(env_nothing, flamegpu::MessageNone, flamegpu::MessageNone) { return flamegpu::ALIVE; }

namespace {

void* make_host_env_random(const double*, int32_t) {
    auto* m = new flamegpu::ModelDescription("host_env_random");
    flamegpu::EnvironmentDescription env = m->Environment();
    env.newProperty<uint64_t, 3>("u64", {11, 12, 13});
    env.newProperty<int, 4>("arr", {1, 2, 3, 4});
    env.newProperty<uint64_t>("u64_sum", 0);
    env.newProperty<uint64_t>("u64_sum_array", 0);
    env.newProperty<int>("arr_old2", 0);
    env.newProperty<int>("arr_sum_before", 0);
    env.newProperty<uint32_t>("count", 0u);
    env.newProperty<double>("r_uniform", -1.0);
    env.newProperty<double>("r_normal", 0.0);
    env.newProperty<double>("r_lognormal", 0.0);
    env.newProperty<int>("r_int", 0);
    env.newProperty<uint32_t>("r_poisson", 0u);
    env.newProperty<uint32_t, 8>("hist", {0, 0, 0, 0, 0, 0, 0, 0});
    flamegpu::AgentDescription a = m->newAgent("agent");
    a.newVariable<float>("x");
    m->newLayer().addAgentFunction(a.newFunction("nothing", env_nothing));
    m->addInitFunction(env_init);
    m->addStepFunction(env_step);
    return m;
}

struct Register {
    Register() { fgs_register_model("host_env_random", &make_host_env_random); }
} reg;

}  // namespace
