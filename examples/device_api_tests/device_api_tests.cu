// DeviceAPI identity and birth-id calls, written against the FLAME GPU 2 API:
// the models of the reference's tests
// tests/test_cases/runtime/test_device_api.cu:365-405 (check_agent_name_state:
// isAgent / isState) and of AgentOut::genID (DeviceAPI.cuh:548-557).
//
// Registered models:
//   agent_name_state  agent "agent" with states "state" and "state8"; its
//                     function (initial state "state", the agent's first)
//                     stores isAgent("agent"), isAgent("agent3"),
//                     isState("state"), isState("state5") as ints.
//   gen_id            agent "agent"; its function gives birth to one agent of
//                     its type, calls genID() and stores the child's getID()
//                     in "child" (the child's "parent" gets the parent's id).
#include "flamegpu/flamegpu.h"
#include "flamegpu_gb300/fg_sim.h"

FLAMEGPU_AGENT_FUNCTION(check_agent_name_state, flamegpu::MessageNone, flamegpu::MessageNone) {
    FLAMEGPU->setVariable<int>("correct_name", static_cast<int>(FLAMEGPU->isAgent("agent")));
    FLAMEGPU->setVariable<int>("wrong_name", static_cast<int>(FLAMEGPU->isAgent("agent3")));
    FLAMEGPU->setVariable<int>("correct_state", static_cast<int>(FLAMEGPU->isState("state")));
    FLAMEGPU->setVariable<int>("wrong_state", static_cast<int>(FLAMEGPU->isState("state5")));
    return flamegpu::ALIVE;
}

FLAMEGPU_AGENT_FUNCTION(birth_with_gen_id, flamegpu::MessageNone, flamegpu::MessageNone) {
    FLAMEGPU->agent_out.setVariable<flamegpu::id_t>("parent", FLAMEGPU->getID());
    FLAMEGPU->agent_out.genID();
    FLAMEGPU->setVariable<flamegpu::id_t>("child", FLAMEGPU->agent_out.getID());
    return flamegpu::ALIVE;
}

namespace {

void* make_agent_name_state(const double*, int32_t) {
    auto* m = new flamegpu::ModelDescription("model");
    flamegpu::AgentDescription agent = m->newAgent("agent");
    agent.newState("state");
    agent.newState("state8");
    agent.newVariable<int>("correct_name", -1);
    agent.newVariable<int>("wrong_name", -1);
    agent.newVariable<int>("correct_state", -1);
    agent.newVariable<int>("wrong_state", -1);
    m->newLayer().addAgentFunction(agent.newFunction("some_function", check_agent_name_state));
    return m;
}

void* make_gen_id(const double*, int32_t) {
    auto* m = new flamegpu::ModelDescription("gen_id");
    flamegpu::AgentDescription agent = m->newAgent("agent");
    agent.newVariable<flamegpu::id_t>("child", flamegpu::ID_NOT_SET);
    agent.newVariable<flamegpu::id_t>("parent", flamegpu::ID_NOT_SET);
    flamegpu::AgentFunctionDescription f = agent.newFunction("birth", birth_with_gen_id);
    f.setAgentOutput(agent);
    m->newLayer().addAgentFunction(f);
    return m;
}

struct Register {
    Register() {
        fgs_register_model("agent_name_state", &make_agent_name_state);
        fgs_register_model("gen_id", &make_gen_id);
    }
} reg;

}  // namespace
