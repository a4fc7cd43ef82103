// Predator-prey on MessageSpatial2D, written against the FLAME GPU 2 API.
// (FLAME GPU 2 ships no such example; the model is specified here.)
//
// Agents "prey" (x, y, crowd) and "predator" (x, y), positions in [0, EDGE].
// Per step:
//   layer 1  predator_output: predators output their location (radius R);
//            prey_output: prey output theirs
//   layer 2  prey_crowd: each prey counts the other prey closer than R
//   layer 3  prey_step: a prey with any predator message closer than R dies;
//            otherwise it moves by a uniform step in [-STEP, STEP] per axis
//            (clamped to the domain) and, if fewer than MAX_CROWD other prey
//            were within R, gives birth with probability P_PREY_BIRTH to a
//            prey at its new position.
//            predator_step: a predator dies with probability P_PRED_DEATH,
//            otherwise it moves like a prey.
// The crowding limit is a local carrying capacity: without it, predators
// clear the prey around themselves within a few steps, predation falls, and
// the prey population grows by about 4% a step without bound.
// Randomness: SplitMix64 finaliser (Steele, Lea & Flood 2014) over (SEED, id,
// step, stream), the same hash the oracle uses.
// Registered as "predprey2d"; parameters: edge, radius, p_prey_birth,
// p_pred_death, step, seed, max_crowd.
#ifndef FLAMEGPU_SEATBELTS
#define FLAMEGPU_SEATBELTS 0  // benchmark model: device checks off, as in the reference's benchmark builds
#endif
#include "flamegpu/flamegpu.h"
#include "flamegpu_gb300/fg_sim.h"

namespace {
FLAMEGPU_HOST_DEVICE_FUNCTION uint64_t pp_mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
FLAMEGPU_HOST_DEVICE_FUNCTION float pp_uniform(uint64_t seed, uint64_t key, uint32_t step, uint32_t stream) {
    const uint64_t h = pp_mix64(pp_mix64(pp_mix64(seed) ^ key) ^ ((static_cast<uint64_t>(step) << 8) | stream));
    return static_cast<float>(h >> 40) * (1.0f / 16777216.0f);
}
FLAMEGPU_HOST_DEVICE_FUNCTION float pp_clamp(float v, float lo, float hi) { return v < lo ? lo : (v > hi ? hi : v); }
}  // namespace

FLAMEGPU_AGENT_FUNCTION(predator_output, flamegpu::MessageNone, flamegpu::MessageSpatial2D) {
    FLAMEGPU->message_out.setVariable<flamegpu::id_t>("id", FLAMEGPU->getID());
    FLAMEGPU->message_out.setLocation(FLAMEGPU->getVariable<float>("x"), FLAMEGPU->getVariable<float>("y"));
    return flamegpu::ALIVE;
}

FLAMEGPU_AGENT_FUNCTION(prey_output, flamegpu::MessageNone, flamegpu::MessageSpatial2D) {
    FLAMEGPU->message_out.setVariable<flamegpu::id_t>("id", FLAMEGPU->getID());
    FLAMEGPU->message_out.setLocation(FLAMEGPU->getVariable<float>("x"), FLAMEGPU->getVariable<float>("y"));
    return flamegpu::ALIVE;
}

FLAMEGPU_AGENT_FUNCTION(prey_crowd, flamegpu::MessageSpatial2D, flamegpu::MessageNone) {
    const float x = FLAMEGPU->getVariable<float>("x");
    const float y = FLAMEGPU->getVariable<float>("y");
    const float r = FLAMEGPU->environment.getProperty<float>("RADIUS");
    const flamegpu::id_t me = FLAMEGPU->getID();
    uint32_t crowd = 0;
    for (const auto& m : FLAMEGPU->message_in(x, y)) {
        const float dx = m.getVariable<float>("x") - x;
        const float dy = m.getVariable<float>("y") - y;
        if (dx * dx + dy * dy < r * r && m.getVariable<flamegpu::id_t>("id") != me) ++crowd;
    }
    FLAMEGPU->setVariable<uint32_t>("crowd", crowd);
    return flamegpu::ALIVE;
}

FLAMEGPU_AGENT_FUNCTION(prey_step, flamegpu::MessageSpatial2D, flamegpu::MessageNone) {
    const float x = FLAMEGPU->getVariable<float>("x");
    const float y = FLAMEGPU->getVariable<float>("y");
    const float r = FLAMEGPU->environment.getProperty<float>("RADIUS");
    for (const auto& m : FLAMEGPU->message_in(x, y)) {
        const float dx = m.getVariable<float>("x") - x;
        const float dy = m.getVariable<float>("y") - y;
        if (dx * dx + dy * dy < r * r) return flamegpu::DEAD;  // eaten
    }
    const uint64_t seed = FLAMEGPU->environment.getProperty<uint64_t>("SEED");
    const uint64_t key = FLAMEGPU->getID();
    const uint32_t step = FLAMEGPU->getStepCounter();
    const float st = FLAMEGPU->environment.getProperty<float>("STEP");
    const float edge = FLAMEGPU->environment.getProperty<float>("EDGE");
    const float nx = pp_clamp(x + st * (2.0f * pp_uniform(seed, key, step, 2) - 1.0f), 0.0f, edge);
    const float ny = pp_clamp(y + st * (2.0f * pp_uniform(seed, key, step, 3) - 1.0f), 0.0f, edge);
    FLAMEGPU->setVariable<float>("x", nx);
    FLAMEGPU->setVariable<float>("y", ny);
    if (pp_uniform(seed, key, step, 1) < FLAMEGPU->environment.getProperty<float>("P_PREY_BIRTH") &&
        FLAMEGPU->getVariable<uint32_t>("crowd") < FLAMEGPU->environment.getProperty<uint32_t>("MAX_CROWD")) {
        FLAMEGPU->agent_out.setVariable<float>("x", nx);
        FLAMEGPU->agent_out.setVariable<float>("y", ny);
    }
    return flamegpu::ALIVE;
}

FLAMEGPU_AGENT_FUNCTION(predator_step, flamegpu::MessageNone, flamegpu::MessageNone) {
    const uint64_t seed = FLAMEGPU->environment.getProperty<uint64_t>("SEED");
    const uint64_t key = FLAMEGPU->getID();
    const uint32_t step = FLAMEGPU->getStepCounter();
    if (pp_uniform(seed, key, step, 4) < FLAMEGPU->environment.getProperty<float>("P_PRED_DEATH")) return flamegpu::DEAD;
    const float st = FLAMEGPU->environment.getProperty<float>("STEP");
    const float edge = FLAMEGPU->environment.getProperty<float>("EDGE");
    const float x = FLAMEGPU->getVariable<float>("x");
    const float y = FLAMEGPU->getVariable<float>("y");
    FLAMEGPU->setVariable<float>("x", pp_clamp(x + st * (2.0f * pp_uniform(seed, key, step, 5) - 1.0f), 0.0f, edge));
    FLAMEGPU->setVariable<float>("y", pp_clamp(y + st * (2.0f * pp_uniform(seed, key, step, 6) - 1.0f), 0.0f, edge));
    return flamegpu::ALIVE;
}

namespace {
void* make_predprey(const double* p, int32_t np) {
    auto P = [&](int i, double d) { return i < np ? p[i] : d; };
    const float edge = static_cast<float>(P(0, 64.0)), r = static_cast<float>(P(1, 1.0));
    auto* model = new flamegpu::ModelDescription("PredatorPrey2D");
    flamegpu::EnvironmentDescription env = model->Environment();
    env.newProperty<float>("EDGE", edge);
    env.newProperty<float>("RADIUS", r);
    env.newProperty<float>("P_PREY_BIRTH", static_cast<float>(P(2, 0.05)));
    env.newProperty<float>("P_PRED_DEATH", static_cast<float>(P(3, 0.02)));
    env.newProperty<float>("STEP", static_cast<float>(P(4, 0.5)));
    env.newProperty<uint64_t>("SEED", static_cast<uint64_t>(P(5, 4.0)));
    env.newProperty<uint32_t>("MAX_CROWD", static_cast<uint32_t>(P(6, 4.0)));
    for (const char* name : {"predator_location", "prey_location"}) {
        auto msg = model->newMessage<flamegpu::MessageSpatial2D>(name);
        msg.setMin(0.0f, 0.0f);
        msg.setMax(edge, edge);
        msg.setRadius(r);
        msg.newVariable<flamegpu::id_t>("id");
    }
    flamegpu::AgentDescription prey = model->newAgent("prey");
    prey.newVariable<float>("x");
    prey.newVariable<float>("y");
    prey.newVariable<uint32_t>("crowd", 0u);
    flamegpu::AgentDescription pred = model->newAgent("predator");
    pred.newVariable<float>("x");
    pred.newVariable<float>("y");
    auto fo = pred.newFunction("predator_output", predator_output);
    fo.setMessageOutput("predator_location");
    auto fpo = prey.newFunction("prey_output", prey_output);
    fpo.setMessageOutput("prey_location");
    auto fc = prey.newFunction("prey_crowd", prey_crowd);
    fc.setMessageInput("prey_location");
    auto fp = prey.newFunction("prey_step", prey_step);
    fp.setMessageInput("predator_location");
    fp.setAllowAgentDeath(true);
    fp.setAgentOutput(prey);
    auto fd = pred.newFunction("predator_step", predator_step);
    fd.setAllowAgentDeath(true);
    flamegpu::LayerDescription l1 = model->newLayer();
    l1.addAgentFunction(fo);
    l1.addAgentFunction(fpo);
    model->newLayer().addAgentFunction(fc);
    flamegpu::LayerDescription l3 = model->newLayer();
    l3.addAgentFunction(fp);
    l3.addAgentFunction(fd);
    return model;
}
struct Register {
    Register() { fgs_register_model("predprey2d", &make_predprey); }
} reg;
}  // namespace
