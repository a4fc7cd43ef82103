// Device agent creation, written against the FLAME GPU 2 API: the models of
// the reference's DeviceAgentCreationTest suite
// (tests/test_cases/runtime/agent/test_device_agent_creation.cu:23-1338).
//
// Registered models:
//   dac         params: kind, layout, condition
//               kind 0..3: MandatoryOutput, OptionalOutput, MandatoryOutputWithDeath,
//                          OptionalOutputWithDeath (:23-52); death allowed for 2, 3
//               layout 0: one agent, default state, births into it (SameState)
//                      1: states a, b; a -> a; births into b (DifferentState)
//                      2: states a, b; a -> b; births into b (SameState with a condition, :657-778)
//                      3: states a, b, c; a -> c; births into b (DifferentState with a condition, :779-892)
//                      4: agent2 runs, births into agent state b (DifferentAgent, :383-602)
//                      5: agent2 runs, births into agent, whose "default" is 15 (DefaultVariableValue, :604-653)
//               condition 1: EvenThreadsOnlyCdn (:654-656)
//   dac_array   params: default_works. ArrayVarDeviceBirth(_DefaultWorks) (:1108-1194)
//   dac_ids     params: agents. 0: AgentID_MultipleStatesUniqueIDs (:1196-1296),
//               1: AgentID_DeviceBirth_MultipleAgents (:1297-1338)
//   cross_birth births across agent types and states, for an order-exact
//               comparison with the oracle. Agents "prey" (default state) and
//               "hunter" (states roam, rest; v u32, x f32 each). Per step:
//                 spawn  prey: x += 1; a hunter child in roam (v + 1000, x / 2)
//                        if (id + step) % 3 == 0; dies if id % 11 == 0
//                 hunt   hunter roam -> rest if id is even: x += 2; a prey
//                        child (v + 7, x) if id % 5 == 0
//                 wake   hunter rest -> roam: x -= 1
#include "flamegpu/flamegpu.h"
#include "flamegpu_gb300/fg_sim.h"

FLAMEGPU_AGENT_FUNCTION(dac_mandatory, flamegpu::MessageNone, flamegpu::MessageNone) {
    const unsigned int id = FLAMEGPU->getVariable<unsigned int>("id") + 1;
    FLAMEGPU->agent_out.setVariable<float>("x", id + 12.0f);
    FLAMEGPU->agent_out.setVariable<unsigned int>("id", id);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(dac_optional, flamegpu::MessageNone, flamegpu::MessageNone) {
    const unsigned int id = FLAMEGPU->getVariable<unsigned int>("id") + 1;
    if (threadIdx.x % 2 == 0) {
        FLAMEGPU->agent_out.setVariable<float>("x", id + 12.0f);
        FLAMEGPU->agent_out.setVariable<unsigned int>("id", id);
    }
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(dac_mandatory_death, flamegpu::MessageNone, flamegpu::MessageNone) {
    const unsigned int id = FLAMEGPU->getVariable<unsigned int>("id") + 1;
    FLAMEGPU->agent_out.setVariable<float>("x", id + 12.0f);
    FLAMEGPU->agent_out.setVariable<unsigned int>("id", id);
    return flamegpu::DEAD;
}
FLAMEGPU_AGENT_FUNCTION(dac_optional_death, flamegpu::MessageNone, flamegpu::MessageNone) {
    const unsigned int id = FLAMEGPU->getVariable<unsigned int>("id") + 1;
    if (threadIdx.x % 2 == 0) {
        FLAMEGPU->agent_out.setVariable<float>("x", id + 12.0f);
        FLAMEGPU->agent_out.setVariable<unsigned int>("id", id);
    } else {
        return flamegpu::DEAD;
    }
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION_CONDITION(dac_even_threads) { return threadIdx.x % 2 == 0; }

FLAMEGPU_AGENT_FUNCTION(dac_array_birth, flamegpu::MessageNone, flamegpu::MessageNone) {
    const unsigned int i = FLAMEGPU->getVariable<unsigned int>("id") * 3;
    FLAMEGPU->agent_out.setVariable<unsigned int>("id", i);
    FLAMEGPU->agent_out.setVariable<int, 4>("array_var", 0, 3 + i);
    FLAMEGPU->agent_out.setVariable<int, 4>("array_var", 1, 5 + i);
    FLAMEGPU->agent_out.setVariable<int, 4>("array_var", 2, 9 + i);
    FLAMEGPU->agent_out.setVariable<int, 4>("array_var", 3, 17 + i);
    FLAMEGPU->agent_out.setVariable<float>("y", 14.0f + i);
    return flamegpu::DEAD;
}
FLAMEGPU_AGENT_FUNCTION(dac_array_birth_default, flamegpu::MessageNone, flamegpu::MessageNone) {
    const unsigned int i = FLAMEGPU->getVariable<unsigned int>("id") * 3;
    FLAMEGPU->agent_out.setVariable<unsigned int>("id", i);
    return flamegpu::DEAD;
}

FLAMEGPU_AGENT_FUNCTION(dac_copy_id, flamegpu::MessageNone, flamegpu::MessageNone) {
    FLAMEGPU->setVariable<flamegpu::id_t>("id_copy", FLAMEGPU->getID());
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(dac_id_birth, flamegpu::MessageNone, flamegpu::MessageNone) {
    FLAMEGPU->setVariable<flamegpu::id_t>("id_other", FLAMEGPU->agent_out.getID());
    FLAMEGPU->agent_out.setVariable<flamegpu::id_t>("id_other", FLAMEGPU->getID());
    return flamegpu::ALIVE;
}

FLAMEGPU_AGENT_FUNCTION(cb_spawn, flamegpu::MessageNone, flamegpu::MessageNone) {
    const flamegpu::id_t id = FLAMEGPU->getID();
    const float x = FLAMEGPU->getVariable<float>("x") + 1.0f;
    FLAMEGPU->setVariable<float>("x", x);
    if ((id + FLAMEGPU->getStepCounter()) % 3 == 0) {
        FLAMEGPU->agent_out.setVariable<unsigned int>("v", FLAMEGPU->getVariable<unsigned int>("v") + 1000u);
        FLAMEGPU->agent_out.setVariable<float>("x", x * 0.5f);
    }
    return id % 11 == 0 ? flamegpu::DEAD : flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION_CONDITION(cb_even) { return FLAMEGPU->getID() % 2 == 0; }
FLAMEGPU_AGENT_FUNCTION(cb_hunt, flamegpu::MessageNone, flamegpu::MessageNone) {
    const float x = FLAMEGPU->getVariable<float>("x") + 2.0f;
    FLAMEGPU->setVariable<float>("x", x);
    if (FLAMEGPU->getID() % 5 == 0) {
        FLAMEGPU->agent_out.setVariable<unsigned int>("v", FLAMEGPU->getVariable<unsigned int>("v") + 7u);
        FLAMEGPU->agent_out.setVariable<float>("x", x);
    }
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(cb_wake, flamegpu::MessageNone, flamegpu::MessageNone) {
    FLAMEGPU->setVariable<float>("x", FLAMEGPU->getVariable<float>("x") - 1.0f);
    return flamegpu::ALIVE;
}

namespace {

void* make_cross_birth(const double*, int32_t) {
    auto* m = new flamegpu::ModelDescription("CrossBirth");
    flamegpu::AgentDescription prey = m->newAgent("prey");
    prey.newVariable<unsigned int>("v");
    prey.newVariable<float>("x");
    flamegpu::AgentDescription hunter = m->newAgent("hunter");
    hunter.newVariable<unsigned int>("v");
    hunter.newVariable<float>("x");
    hunter.newState("roam");
    hunter.newState("rest");
    hunter.setInitialState("roam");
    flamegpu::AgentFunctionDescription spawn = prey.newFunction("spawn", cb_spawn);
    spawn.setAgentOutput(hunter, "roam");
    spawn.setAllowAgentDeath(true);
    flamegpu::AgentFunctionDescription hunt = hunter.newFunction("hunt", cb_hunt);
    hunt.setInitialState("roam");
    hunt.setEndState("rest");
    hunt.setFunctionCondition(cb_even);
    hunt.setAgentOutput(prey);
    flamegpu::AgentFunctionDescription wake = hunter.newFunction("wake", cb_wake);
    wake.setInitialState("rest");
    wake.setEndState("roam");
    m->newLayer().addAgentFunction(spawn);
    m->newLayer().addAgentFunction(hunt);
    m->newLayer().addAgentFunction(wake);
    return m;
}

flamegpu::AgentFunctionDescription dac_function(flamegpu::AgentDescription& a, int kind) {
    switch (kind) {
        case 1: return a.newFunction("output", dac_optional);
        case 2: return a.newFunction("output", dac_mandatory_death);
        case 3: return a.newFunction("output", dac_optional_death);
        default: return a.newFunction("output", dac_mandatory);
    }
}

void* make_dac(const double* p, int32_t np) {
    auto P = [&](int i, double d) { return i < np ? p[i] : d; };
    const int kind = static_cast<int>(P(0, 0)), layout = static_cast<int>(P(1, 0)), cond = static_cast<int>(P(2, 0));
    auto* m = new flamegpu::ModelDescription("DeviceAgentCreation");
    flamegpu::AgentDescription agent = m->newAgent("agent");
    agent.newVariable<float>("x");
    if (layout == 5) agent.newVariable<float>("default", 15.0f);
    agent.newVariable<unsigned int>("id");
    if (layout == 1 || layout == 2 || layout == 3 || layout == 4) {
        agent.newState("a");
        agent.newState("b");
    }
    if (layout == 3) agent.newState("c");
    flamegpu::AgentDescription runner = agent;
    if (layout >= 4) {
        runner = m->newAgent("agent2");
        runner.newVariable<float>("x");
        runner.newVariable<unsigned int>("id");
    }
    flamegpu::AgentFunctionDescription f = dac_function(runner, kind);
    if (kind >= 2) f.setAllowAgentDeath(true);
    if (cond) f.setFunctionCondition(dac_even_threads);
    switch (layout) {
        case 1:
            f.setInitialState("a");
            f.setEndState("a");
            f.setAgentOutput(agent, "b");
            break;
        case 2:
            f.setInitialState("a");
            f.setEndState("b");
            f.setAgentOutput(agent, "b");
            break;
        case 3:
            f.setInitialState("a");
            f.setEndState("c");
            f.setAgentOutput(agent, "b");
            break;
        case 4:
            f.setAgentOutput(agent, "b");
            break;
        default:
            f.setAgentOutput(agent);
    }
    m->newLayer().addAgentFunction(f);
    return m;
}

void* make_dac_array(const double* p, int32_t np) {
    const bool default_works = np > 0 && p[0] != 0.0;
    auto* m = new flamegpu::ModelDescription("model");
    flamegpu::AgentDescription a = m->newAgent("agent_name");
    a.newVariable<unsigned int>("id", UINT_MAX);
    if (default_works) {
        a.newVariable<int, 4>("array_var", {3, 5, 9, 17});
        a.newVariable<float>("y", 14.0f);
    } else {
        a.newVariable<int, 4>("array_var");
        a.newVariable<float>("y");
    }
    flamegpu::AgentFunctionDescription fn =
        default_works ? a.newFunction("out", dac_array_birth_default) : a.newFunction("out", dac_array_birth);
    fn.setAllowAgentDeath(true);
    fn.setAgentOutput(a);
    m->newLayer().addAgentFunction(fn);
    return m;
}

void* make_dac_ids(const double* p, int32_t np) {
    const bool agents = np > 0 && p[0] != 0.0;
    auto* m = new flamegpu::ModelDescription("test_agentid");
    if (agents) {
        flamegpu::AgentDescription A = m->newAgent("agentA");
        A.newVariable<flamegpu::id_t>("id_other", flamegpu::ID_NOT_SET);
        flamegpu::AgentDescription B = m->newAgent("agentB");
        B.newVariable<flamegpu::id_t>("id_other", flamegpu::ID_NOT_SET);
        flamegpu::AgentFunctionDescription f = A.newFunction("birth", dac_id_birth);
        f.setAgentOutput(B);
        m->newLayer().addAgentFunction(f);
        return m;
    }
    flamegpu::AgentDescription a = m->newAgent("agent");
    a.newVariable<flamegpu::id_t>("id_copy", flamegpu::ID_NOT_SET);
    a.newVariable<flamegpu::id_t>("id_other", flamegpu::ID_NOT_SET);
    a.newState("a");
    a.newState("b");
    flamegpu::AgentFunctionDescription b1 = a.newFunction("birth", dac_id_birth);
    b1.setAgentOutput(a, "a");
    b1.setInitialState("a");
    b1.setEndState("a");
    flamegpu::AgentFunctionDescription b2 = a.newFunction("birth2", dac_id_birth);
    b2.setAgentOutput(a, "b");
    b2.setInitialState("b");
    b2.setEndState("b");
    flamegpu::AgentFunctionDescription c1 = a.newFunction("copy_id", dac_copy_id);
    c1.setInitialState("a");
    c1.setEndState("a");
    flamegpu::AgentFunctionDescription c2 = a.newFunction("copy_id2", dac_copy_id);
    c2.setInitialState("b");
    c2.setEndState("b");
    m->newLayer().addAgentFunction(b1);
    m->newLayer().addAgentFunction(b2);
    flamegpu::LayerDescription l2 = m->newLayer();
    l2.addAgentFunction(c1);
    l2.addAgentFunction(c2);
    return m;
}

struct Register {
    Register() {
        fgs_register_model("dac", &make_dac);
        fgs_register_model("dac_array", &make_dac_array);
        fgs_register_model("dac_ids", &make_dac_ids);
        fgs_register_model("cross_birth", &make_cross_birth);
    }
} reg;

}  // namespace
