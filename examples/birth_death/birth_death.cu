// Birth/death compaction stress model, written against the FLAME GPU 2 API.
// 8 float variables f0..f7 and an int counter; per step every agent
// increments its counter, dies with probability P_DEATH, and a survivor
// spawns one child with probability P_BIRTH that copies f0..f7 (counter 0)
// and receives a fresh id. Decisions come from a counter-based hash of
// (SEED, agent id, step, stream) — SplitMix64's finaliser (Steele, Lea &
// Flood 2014) — so the same model gives the same decisions on any build.
// Registered as "birth_death"; parameters: p_death, p_birth, seed.
// Benchmark model: built with seatbelts off, as the reference builds its
// benchmarks (FLAMEGPU_SEATBELTS=OFF, src/CMakeLists.txt:78). The test models
// keep the device checks on.
#ifndef FLAMEGPU_SEATBELTS
#define FLAMEGPU_SEATBELTS 0
#endif
#include "flamegpu/flamegpu.h"
#include "flamegpu_gb300/fg_sim.h"

namespace {
FLAMEGPU_HOST_DEVICE_FUNCTION uint64_t bd_mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
FLAMEGPU_HOST_DEVICE_FUNCTION float bd_uniform(uint64_t seed, uint64_t key, uint32_t step, uint32_t stream) {
    const uint64_t h = bd_mix64(bd_mix64(bd_mix64(seed) ^ key) ^ ((static_cast<uint64_t>(step) << 8) | stream));
    return static_cast<float>(h >> 40) * (1.0f / 16777216.0f);
}
}  // namespace

FLAMEGPU_AGENT_FUNCTION(live, flamegpu::MessageNone, flamegpu::MessageNone) {
    const uint64_t seed = FLAMEGPU->environment.getProperty<uint64_t>("SEED");
    const uint64_t key = FLAMEGPU->getID();
    const uint32_t step = FLAMEGPU->getStepCounter();
    FLAMEGPU->setVariable<int>("counter", FLAMEGPU->getVariable<int>("counter") + 1);
    if (bd_uniform(seed, key, step, 0) < FLAMEGPU->environment.getProperty<float>("P_DEATH")) return flamegpu::DEAD;
    if (bd_uniform(seed, key, step, 1) < FLAMEGPU->environment.getProperty<float>("P_BIRTH")) {
        FLAMEGPU->agent_out.setVariable<float>("f0", FLAMEGPU->getVariable<float>("f0"));
        FLAMEGPU->agent_out.setVariable<float>("f1", FLAMEGPU->getVariable<float>("f1"));
        FLAMEGPU->agent_out.setVariable<float>("f2", FLAMEGPU->getVariable<float>("f2"));
        FLAMEGPU->agent_out.setVariable<float>("f3", FLAMEGPU->getVariable<float>("f3"));
        FLAMEGPU->agent_out.setVariable<float>("f4", FLAMEGPU->getVariable<float>("f4"));
        FLAMEGPU->agent_out.setVariable<float>("f5", FLAMEGPU->getVariable<float>("f5"));
        FLAMEGPU->agent_out.setVariable<float>("f6", FLAMEGPU->getVariable<float>("f6"));
        FLAMEGPU->agent_out.setVariable<float>("f7", FLAMEGPU->getVariable<float>("f7"));
        FLAMEGPU->agent_out.setVariable<int>("counter", 0);
    }
    return flamegpu::ALIVE;
}

namespace {
void* make_birth_death(const double* p, int32_t np) {
    auto P = [&](int i, double d) { return i < np ? p[i] : d; };
    auto* model = new flamegpu::ModelDescription("BirthDeath");
    flamegpu::EnvironmentDescription env = model->Environment();
    env.newProperty<float>("P_DEATH", static_cast<float>(P(0, 0.30)));
    env.newProperty<float>("P_BIRTH", static_cast<float>(P(1, 0.20)));
    env.newProperty<uint64_t>("SEED", static_cast<uint64_t>(P(2, 1.0)));
    flamegpu::AgentDescription a = model->newAgent("agent");
    const char* names[8] = {"f0", "f1", "f2", "f3", "f4", "f5", "f6", "f7"};
    for (const char* n : names) a.newVariable<float>(n);
    a.newVariable<int>("counter", 0);
    auto f = a.newFunction("live", live);
    f.setAllowAgentDeath(true);
    f.setAgentOutput(a);
    model->newLayer().addAgentFunction(f);
    return model;
}
struct Register {
    Register() { fgs_register_model("birth_death", &make_birth_death); }
} reg;
}  // namespace
