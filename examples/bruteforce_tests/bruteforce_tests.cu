// Brute-force message test models, written against the FLAME GPU 2 API: the
// models of the reference's TestMessage_BruteForce cases
// (tests/test_cases/runtime/messaging/test_brute_force.cu).
//
// Registered models (parameters in brackets):
//   bf_sum [variant, optional]   Mandatory1 / Mandatory2 / Optional1 / Optional2
//                                (:73-276): agents output x (optional: only if
//                                x != 0); every agent sums the messages and
//                                multiplies them (clamped at +-1e6) in message
//                                order; variant 2 also adds 1 to its x.
//   bf_optional_none             OptionalNone (:277-314): no message is output.
//   bf_read_empty                ReadEmpty (:332-381): a list read before output.
//   bf_array                     ArrayVariable (:383-418): array message variables.
//   bf_persistence [persistent]  PersistenceOff / PersistenceOn (:436-627): an
//                                init function creates the agents, output only
//                                on even steps (function condition).
//   bf_reserved                  reserved_name (:316-330): a message variable
//                                named "_" (its factory throws ReservedName).
#include <climits>

#include "flamegpu/flamegpu.h"
#include "flamegpu_gb300/fg_sim.h"

namespace {
constexpr unsigned int kBfAgents = 128;  // AGENT_COUNT of the reference tests
}

FLAMEGPU_AGENT_FUNCTION(bf_out, flamegpu::MessageNone, flamegpu::MessageBruteForce) {
    FLAMEGPU->message_out.setVariable("x", FLAMEGPU->getVariable<int>("x"));
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(bf_out_optional, flamegpu::MessageNone, flamegpu::MessageBruteForce) {
    const int x = FLAMEGPU->getVariable<int>("x");
    if (x) FLAMEGPU->message_out.setVariable("x", x);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(bf_out_none, flamegpu::MessageNone, flamegpu::MessageBruteForce) { return flamegpu::ALIVE; }
FLAMEGPU_AGENT_FUNCTION(bf_in, flamegpu::MessageBruteForce, flamegpu::MessageNone) {
    int sum = FLAMEGPU->getVariable<int>("sum");
    int product = FLAMEGPU->getVariable<int>("product");
    for (auto& message : FLAMEGPU->message_in) {
        const int x = message.getVariable<int>("x");
        sum += x;
        product *= x;
        product = product > 1000000 ? 1 : product;
        product = product < -1000000 ? -1 : product;
    }
    FLAMEGPU->setVariable<int>("sum", sum);
    FLAMEGPU->setVariable<int>("product", product);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(bf_in2, flamegpu::MessageBruteForce, flamegpu::MessageNone) {
    int sum = FLAMEGPU->getVariable<int>("sum");
    int product = FLAMEGPU->getVariable<int>("product");
    for (auto& message : FLAMEGPU->message_in) {
        const int x = message.getVariable<int>("x");
        sum += x;
        product *= x;
        product = product > 1000000 ? 1 : product;
        product = product < -1000000 ? -1 : product;
    }
    FLAMEGPU->setVariable<int>("sum", sum);
    FLAMEGPU->setVariable<int>("product", product);
    FLAMEGPU->setVariable<int>("x", FLAMEGPU->getVariable<int>("x") + 1);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(bf_in_none, flamegpu::MessageBruteForce, flamegpu::MessageNone) {
    for (auto& message : FLAMEGPU->message_in)
        FLAMEGPU->setVariable("message_read", message.getVariable<unsigned int>("index_times_3"));
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(bf_count, flamegpu::MessageBruteForce, flamegpu::MessageNone) {
    unsigned int count = 0;
    for (const auto& message : FLAMEGPU->message_in) {
        (void)message;
        ++count;
    }
    FLAMEGPU->setVariable<unsigned int>("count", count);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(bf_array_out, flamegpu::MessageNone, flamegpu::MessageBruteForce) {
    const unsigned int index = FLAMEGPU->getVariable<unsigned int>("index");
    FLAMEGPU->message_out.setVariable<unsigned int>("index", index);
    FLAMEGPU->message_out.setVariable<unsigned int, 3>("v", 0, index * 3);
    FLAMEGPU->message_out.setVariable<unsigned int, 3>("v", 1, index * 7);
    FLAMEGPU->message_out.setVariable<unsigned int, 3>("v", 2, index * 11);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(bf_array_in, flamegpu::MessageBruteForce, flamegpu::MessageNone) {
    const unsigned int my_index = FLAMEGPU->getVariable<unsigned int>("index");
    for (auto& message : FLAMEGPU->message_in) {
        if (message.getVariable<unsigned int>("index") == my_index) {
            FLAMEGPU->setVariable<unsigned int, 3>("message_read", 0, message.getVariable<unsigned int, 3>("v", 0));
            FLAMEGPU->setVariable<unsigned int, 3>("message_read", 1, message.getVariable<unsigned int, 3>("v", 1));
            FLAMEGPU->setVariable<unsigned int, 3>("message_read", 2, message.getVariable<unsigned int, 3>("v", 2));
            break;
        }
    }
    return flamegpu::ALIVE;
}
FLAMEGPU_INIT_FUNCTION(bf_persist_init) {
    auto agent = FLAMEGPU->agent("Agent");
    for (uint32_t i = 0; i < kBfAgents; ++i) {
        auto instance = agent.newAgent();
        instance.setVariable<int>("id", static_cast<int>(i));
        instance.setVariable<unsigned int>("count", 0u);
        instance.setVariable<unsigned int>("sum", 0u);
    }
}
FLAMEGPU_AGENT_FUNCTION_CONDITION(bf_even_only) { return FLAMEGPU->getStepCounter() % 2 == 0; }
FLAMEGPU_AGENT_FUNCTION(bf_out_simple, flamegpu::MessageNone, flamegpu::MessageBruteForce) {
    FLAMEGPU->message_out.setVariable<int>("id", FLAMEGPU->getVariable<int>("id"));
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(bf_in_simple, flamegpu::MessageBruteForce, flamegpu::MessageNone) {
    unsigned int count = 0, sum = 0;
    for (auto& m : FLAMEGPU->message_in) {
        ++count;
        sum += m.getVariable<int>("id");
    }
    FLAMEGPU->setVariable<unsigned int>("count", count);
    FLAMEGPU->setVariable<unsigned int>("sum", sum);
    return flamegpu::ALIVE;
}

namespace {

void* make_sum(const double* p, int32_t n) {
    const int variant = n > 0 ? static_cast<int>(p[0]) : 1;
    const bool optional = n > 1 && p[1] != 0.0;
    auto* m = new flamegpu::ModelDescription("Model");
    flamegpu::MessageBruteForce::Description message = m->newMessage("Message");
    message.newVariable<int>("x");
    flamegpu::AgentDescription a = m->newAgent("Agent");
    a.newVariable<int>("x");
    a.newVariable<int>("sum");
    a.newVariable<int>("product");
    flamegpu::AgentFunctionDescription fo =
        optional ? a.newFunction("OutFunction", bf_out_optional) : a.newFunction("OutFunction", bf_out);
    if (optional) fo.setMessageOutputOptional(true);
    fo.setMessageOutput(message);
    flamegpu::AgentFunctionDescription fi =
        variant == 2 ? a.newFunction("InFunction", bf_in2) : a.newFunction("InFunction", bf_in);
    fi.setMessageInput(message);
    m->newLayer("OutLayer").addAgentFunction(fo);
    m->newLayer("InLayer").addAgentFunction(fi);
    return m;
}

void* make_optional_none(const double*, int32_t) {
    auto* m = new flamegpu::ModelDescription("Model");
    flamegpu::MessageBruteForce::Description message = m->newMessage("Message");
    message.newVariable<unsigned int>("index_times_3");
    flamegpu::AgentDescription a = m->newAgent("Agent");
    a.newVariable<unsigned int>("index");
    a.newVariable<unsigned int>("message_read", UINT_MAX);
    flamegpu::AgentFunctionDescription fo = a.newFunction("OutFunction", bf_out_none);
    fo.setMessageOutputOptional(true);
    fo.setMessageOutput(message);
    flamegpu::AgentFunctionDescription fi = a.newFunction("InFunction", bf_in_none);
    fi.setMessageInput(message);
    m->newLayer("OutLayer").addAgentFunction(fo);
    m->newLayer("InLayer").addAgentFunction(fi);
    return m;
}

void* make_read_empty(const double*, int32_t) {
    auto* m = new flamegpu::ModelDescription("Model");
    flamegpu::MessageBruteForce::Description message = m->newMessage<flamegpu::MessageBruteForce>("location");
    message.newVariable<int>("id");
    flamegpu::AgentDescription agent = m->newAgent("agent");
    agent.newVariable<unsigned int>("count", 0);
    agent.newFunction("in", bf_count).setMessageInput("location");
    m->newLayer().addAgentFunction(bf_count);
    return m;
}

void* make_array(const double*, int32_t) {
    auto* m = new flamegpu::ModelDescription("Model");
    flamegpu::MessageBruteForce::Description message = m->newMessage<flamegpu::MessageBruteForce>("Message");
    message.newVariable<unsigned int, 3>("v");
    message.newVariable<unsigned int>("index");
    flamegpu::AgentDescription a = m->newAgent("Agent");
    a.newVariable<unsigned int>("index");
    a.newVariable<unsigned int, 3>("message_read", {UINT_MAX, UINT_MAX, UINT_MAX});
    flamegpu::AgentFunctionDescription fo = a.newFunction("OutFunction", bf_array_out);
    fo.setMessageOutput(message);
    flamegpu::AgentFunctionDescription fi = a.newFunction("InFunction", bf_array_in);
    fi.setMessageInput(message);
    m->newLayer("OutLayer").addAgentFunction(fo);
    m->newLayer("InLayer").addAgentFunction(fi);
    return m;
}

void* make_persistence(const double* p, int32_t n) {
    const bool persistent = n > 0 && p[0] != 0.0;
    auto* m = new flamegpu::ModelDescription("TestMessage_BruteForce");
    {
        flamegpu::MessageBruteForce::Description message = m->newMessage<flamegpu::MessageBruteForce>("msg");
        message.newVariable<int>("id");
        if (persistent) message.setPersistent(true);
    }
    {
        flamegpu::AgentDescription agent = m->newAgent("Agent");
        agent.newVariable<int>("id");
        agent.newVariable<unsigned int>("count", 0);
        agent.newVariable<unsigned int>("sum", 0);
        auto af = agent.newFunction("out", bf_out_simple);
        af.setMessageOutput("msg");
        af.setMessageOutputOptional(true);
        af.setFunctionCondition(bf_even_only);
        agent.newFunction("in", bf_in_simple).setMessageInput("msg");
    }
    m->newLayer().addAgentFunction(bf_out_simple);
    m->newLayer().addAgentFunction(bf_in_simple);
    m->addInitFunction(bf_persist_init);
    return m;
}

void* make_reserved(const double*, int32_t) {
    auto* m = new flamegpu::ModelDescription("Model");
    flamegpu::MessageBruteForce::Description message = m->newMessage("Message");
    try {
        message.newVariable<int>("_");
    } catch (...) {
        delete m;
        throw;
    }
    return m;
}

struct Register {
    Register() {
        fgs_register_model("bf_sum", &make_sum);
        fgs_register_model("bf_optional_none", &make_optional_none);
        fgs_register_model("bf_read_empty", &make_read_empty);
        fgs_register_model("bf_array", &make_array);
        fgs_register_model("bf_persistence", &make_persistence);
        fgs_register_model("bf_reserved", &make_reserved);
    }
} reg;

}  // namespace
