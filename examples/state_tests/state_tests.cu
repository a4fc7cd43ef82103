// Agent function conditions and state transitions, written against the FLAME
// GPU 2 API. The first three models restate the reference's tests
// (tests/test_cases/runtime/test_agent_function_conditions.cu:19-150,
// tests/test_cases/runtime/agent/detail/test_agent_state_transition.cu:20-260);
// "state_mix" exercises conditions, death, birth and transitions together,
// for an order-exact comparison with the oracle.
//
// Registered models:
//   condition_split   SplitAgents: Start -> End if x == 1 (x + 1, y = 3..6),
//                     Start -> End2 if x != 1 (x - 1, y = 23..26), two layers
//   condition_none    AllDisabled: a condition no agent meets, then a plain function
//   state_chain       params: rounds. Start -> Start (x + 1), then Start -> End
//                     for agents with x == step + 2 ... (see chain_* below)
//   state_mix         states A, B; per step:
//                       mix_ab  A -> B if (id + step) % 3 == 0: x += 1; dies if
//                               id % 7 == 0; a child (v + 1000, x) if id % 5 == 0
//                       mix_ba  B -> A if id % 2 == 0: x *= 2
//                       mix_aa  A -> A if x > 10: x -= 10
#include "flamegpu/flamegpu.h"
#include "flamegpu_gb300/fg_sim.h"

namespace {
const char* kStart = "Start";
const char* kEnd = "End";
const char* kEnd2 = "End2";
}  // namespace

// ------------------------------------------------------------ condition_split

FLAMEGPU_AGENT_FUNCTION(split_fn1, flamegpu::MessageNone, flamegpu::MessageNone) {
    FLAMEGPU->setVariable<int>("x", FLAMEGPU->getVariable<int>("x") + 1);
    FLAMEGPU->setVariable<int, 4>("y", 0, 3);
    FLAMEGPU->setVariable<int, 4>("y", 1, 4);
    FLAMEGPU->setVariable<int, 4>("y", 2, 5);
    FLAMEGPU->setVariable<int, 4>("y", 3, 6);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(split_fn2, flamegpu::MessageNone, flamegpu::MessageNone) {
    FLAMEGPU->setVariable<int>("x", FLAMEGPU->getVariable<int>("x") - 1);
    FLAMEGPU->setVariable<int, 4>("y", 0, 23);
    FLAMEGPU->setVariable<int, 4>("y", 1, 24);
    FLAMEGPU->setVariable<int, 4>("y", 2, 25);
    FLAMEGPU->setVariable<int, 4>("y", 3, 26);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION_CONDITION(split_cond1) { return FLAMEGPU->getVariable<int>("x") == 1; }
FLAMEGPU_AGENT_FUNCTION_CONDITION(split_cond2) { return FLAMEGPU->getVariable<int>("x") != 1; }
FLAMEGPU_AGENT_FUNCTION_CONDITION(all_fail) { return false; }

// ---------------------------------------------------------------- state_chain

FLAMEGPU_AGENT_FUNCTION(chain_inc, flamegpu::MessageNone, flamegpu::MessageNone) {
    FLAMEGPU->setVariable<int>("x", FLAMEGPU->getVariable<int>("x") + 1);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(chain_move, flamegpu::MessageNone, flamegpu::MessageNone) {
    FLAMEGPU->setVariable<int>("x", FLAMEGPU->getVariable<int>("x") + 10);
    return flamegpu::ALIVE;
}
// the agents whose round has come: round r moves in step r - 1
FLAMEGPU_AGENT_FUNCTION_CONDITION(chain_due) {
    return FLAMEGPU->getVariable<int>("round") == static_cast<int>(FLAMEGPU->getStepCounter()) + 1;
}

// ------------------------------------------------------------------ state_mix

FLAMEGPU_AGENT_FUNCTION(mix_ab, flamegpu::MessageNone, flamegpu::MessageNone) {
    const flamegpu::id_t id = FLAMEGPU->getID();
    const float x = FLAMEGPU->getVariable<float>("x") + 1.0f;
    FLAMEGPU->setVariable<float>("x", x);
    if (id % 5 == 0) {
        FLAMEGPU->agent_out.setVariable<unsigned int>("v", FLAMEGPU->getVariable<unsigned int>("v") + 1000u);
        FLAMEGPU->agent_out.setVariable<float>("x", x);
    }
    return id % 7 == 0 ? flamegpu::DEAD : flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(mix_ba, flamegpu::MessageNone, flamegpu::MessageNone) {
    FLAMEGPU->setVariable<float>("x", FLAMEGPU->getVariable<float>("x") * 2.0f);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(mix_aa, flamegpu::MessageNone, flamegpu::MessageNone) {
    FLAMEGPU->setVariable<float>("x", FLAMEGPU->getVariable<float>("x") - 10.0f);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION_CONDITION(mix_ab_cond) {
    return (FLAMEGPU->getID() + FLAMEGPU->getStepCounter()) % 3 == 0;
}
FLAMEGPU_AGENT_FUNCTION_CONDITION(mix_ba_cond) { return FLAMEGPU->getID() % 2 == 0; }
FLAMEGPU_AGENT_FUNCTION_CONDITION(mix_aa_cond) { return FLAMEGPU->getVariable<float>("x") > 10.0f; }

namespace {

void* make_condition_split(const double*, int32_t) {
    auto* m = new flamegpu::ModelDescription("ConditionSplit");
    flamegpu::AgentDescription a = m->newAgent("Agent");
    a.newVariable<int>("x");
    a.newVariable<int, 4>("y");
    a.newState(kStart);
    a.newState(kEnd);
    a.newState(kEnd2);
    flamegpu::AgentFunctionDescription f1 = a.newFunction("Function1", split_fn1);
    f1.setInitialState(kStart);
    f1.setEndState(kEnd);
    f1.setFunctionCondition(split_cond1);
    flamegpu::AgentFunctionDescription f2 = a.newFunction("Function2", split_fn2);
    f2.setInitialState(kStart);
    f2.setEndState(kEnd2);
    f2.setFunctionCondition(split_cond2);
    m->newLayer().addAgentFunction(f1);
    m->newLayer().addAgentFunction(f2);
    return m;
}

void* make_condition_none(const double*, int32_t) {
    auto* m = new flamegpu::ModelDescription("ConditionNone");
    flamegpu::AgentDescription a = m->newAgent("Agent");
    a.newVariable<int>("x");
    a.newVariable<int, 4>("y");
    flamegpu::AgentFunctionDescription f1 = a.newFunction("Function1", split_fn1);
    f1.setFunctionCondition(all_fail);
    flamegpu::AgentFunctionDescription f2 = a.newFunction("Function2", split_fn2);
    m->newLayer().addAgentFunction(f1);
    m->newLayer().addAgentFunction(f2);
    return m;
}

void* make_state_chain(const double*, int32_t) {
    auto* m = new flamegpu::ModelDescription("StateChain");
    flamegpu::AgentDescription a = m->newAgent("Agent");
    a.newVariable<int>("x");
    a.newVariable<int>("round");
    a.newState(kStart);
    a.newState(kEnd);
    a.setInitialState(kStart);
    flamegpu::AgentFunctionDescription inc = a.newFunction("inc", chain_inc);
    inc.setInitialState(kStart);
    inc.setEndState(kStart);
    flamegpu::AgentFunctionDescription mv = a.newFunction("move", chain_move);
    mv.setInitialState(kStart);
    mv.setEndState(kEnd);
    mv.setFunctionCondition(chain_due);
    m->newLayer().addAgentFunction(inc);
    m->newLayer().addAgentFunction(mv);
    return m;
}

void* make_state_mix(const double*, int32_t) {
    auto* m = new flamegpu::ModelDescription("StateMix");
    flamegpu::AgentDescription a = m->newAgent("agent");
    a.newVariable<unsigned int>("v");
    a.newVariable<float>("x");
    a.newState("A");
    a.newState("B");
    a.setInitialState("A");
    flamegpu::AgentFunctionDescription ab = a.newFunction("mix_ab", mix_ab);
    ab.setInitialState("A");
    ab.setEndState("B");
    ab.setFunctionCondition(mix_ab_cond);
    ab.setAllowAgentDeath(true);
    ab.setAgentOutput(a, "B");
    flamegpu::AgentFunctionDescription ba = a.newFunction("mix_ba", mix_ba);
    ba.setInitialState("B");
    ba.setEndState("A");
    ba.setFunctionCondition(mix_ba_cond);
    flamegpu::AgentFunctionDescription aa = a.newFunction("mix_aa", mix_aa);
    aa.setInitialState("A");
    aa.setEndState("A");
    aa.setFunctionCondition(mix_aa_cond);
    m->newLayer().addAgentFunction(ab);
    m->newLayer().addAgentFunction(ba);
    m->newLayer().addAgentFunction(aa);
    return m;
}

struct Register {
    Register() {
        fgs_register_model("condition_split", &make_condition_split);
        fgs_register_model("condition_none", &make_condition_none);
        fgs_register_model("state_chain", &make_state_chain);
        fgs_register_model("state_mix", &make_state_mix);
    }
} reg;

}  // namespace
