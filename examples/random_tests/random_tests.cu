// Device random numbers (FLAMEGPU->random), written against the FLAME GPU 2
// API: every kind of draw of AgentRandom
// (include/flamegpu/runtime/random/AgentRandom.cuh:24-60) stored per agent,
// for the distribution and reproducibility checks of tests/test_random_gpu.py.
//
// Registered models:
//   random_draws      params: small and large Poisson means (default 3.5, 250).
//                     Agent "agent"; its function "draw" stores, every step:
//                     u_f / u_d uniform float / double, u_i uniform int in
//                     [-3, 7], u_r uniform float in [2, 5), n_f / n_d normal,
//                     ln_f logNormal(0, 0.5), p_s / p_l Poisson with the two
//                     means, p_1 Poisson with the default mean (1).
//   random_bad_range  one function calls uniform<int>(5, 1) (min > max): a
//                     device error with seatbelts on (AgentRandom.cuh:129-137).
#include "flamegpu/flamegpu.h"
#include "flamegpu_gb300/fg_sim.h"

FLAMEGPU_AGENT_FUNCTION(random_draw, flamegpu::MessageNone, flamegpu::MessageNone) {
    FLAMEGPU->setVariable<float>("u_f", FLAMEGPU->random.uniform<float>());
    FLAMEGPU->setVariable<double>("u_d", FLAMEGPU->random.uniform<double>());
    FLAMEGPU->setVariable<int>("u_i", FLAMEGPU->random.uniform<int>(-3, 7));
    FLAMEGPU->setVariable<float>("u_r", FLAMEGPU->random.uniform<float>(2.0f, 5.0f));
    FLAMEGPU->setVariable<float>("n_f", FLAMEGPU->random.normal<float>());
    FLAMEGPU->setVariable<double>("n_d", FLAMEGPU->random.normal<double>());
    FLAMEGPU->setVariable<float>("ln_f", FLAMEGPU->random.logNormal<float>(0.0f, 0.5f));
    FLAMEGPU->setVariable<unsigned int>("p_s", FLAMEGPU->random.poisson(FLAMEGPU->environment.getProperty<double>("P_SMALL")));
    FLAMEGPU->setVariable<unsigned int>("p_l", FLAMEGPU->random.poisson(FLAMEGPU->environment.getProperty<double>("P_LARGE")));
    FLAMEGPU->setVariable<unsigned int>("p_1", FLAMEGPU->random.poisson());
    return flamegpu::ALIVE;
}

FLAMEGPU_AGENT_FUNCTION(random_bad_range, flamegpu::MessageNone, flamegpu::MessageNone) {
    FLAMEGPU->setVariable<int>("u_i", FLAMEGPU->random.uniform<int>(5, 1));
    return flamegpu::ALIVE;
}

namespace {

void* make_random_draws(const double* p, int32_t np) {
    auto* m = new flamegpu::ModelDescription("random_draws");
    m->Environment().newProperty<double>("P_SMALL", np > 0 ? p[0] : 3.5);
    m->Environment().newProperty<double>("P_LARGE", np > 1 ? p[1] : 250.0);
    flamegpu::AgentDescription a = m->newAgent("agent");
    a.newVariable<float>("u_f");
    a.newVariable<double>("u_d");
    a.newVariable<int>("u_i");
    a.newVariable<float>("u_r");
    a.newVariable<float>("n_f");
    a.newVariable<double>("n_d");
    a.newVariable<float>("ln_f");
    a.newVariable<unsigned int>("p_s");
    a.newVariable<unsigned int>("p_l");
    a.newVariable<unsigned int>("p_1");
    m->newLayer().addAgentFunction(a.newFunction("draw", random_draw));
    return m;
}

void* make_random_bad_range(const double*, int32_t) {
    auto* m = new flamegpu::ModelDescription("random_bad_range");
    flamegpu::AgentDescription a = m->newAgent("agent");
    a.newVariable<int>("u_i");
    m->newLayer().addAgentFunction(a.newFunction("bad", random_bad_range));
    return m;
}

struct Register {
    Register() {
        fgs_register_model("random_draws", &make_random_draws);
        fgs_register_model("random_bad_range", &make_random_bad_range);
    }
} reg;

}  // namespace
