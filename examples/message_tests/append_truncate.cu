// Message list truncate / append semantics, written against the FLAME GPU 2
// API: the models of the reference's TestMessage_AppendTruncate
// (tests/test_cases/runtime/messaging/test_append_truncate.cu:22-320).
// The first output to a list in a step truncates it, later outputs in the
// same step append.
//
// Registered models (brute-force message "Message" with int x):
//   at_truncate        Out (x = 0), then In (count)
//   at_append          Out (x = 0), Out2 (x = 1), then In2 (count0, count1)
//   at_opt_truncate    optional Out: agents with do_out output and flip do_out
//   at_opt_append      optional Out (flips do_out), optional Out2 (do_out), In2
//   at_append_resize   agents "a" output x = 1, agents "b" x = 2, one agent
//                      "c" counts each value
#include "flamegpu/flamegpu.h"
#include "flamegpu_gb300/fg_sim.h"

FLAMEGPU_AGENT_FUNCTION(at_out, flamegpu::MessageNone, flamegpu::MessageBruteForce) {
    FLAMEGPU->message_out.setVariable("x", 0);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(at_out2, flamegpu::MessageNone, flamegpu::MessageBruteForce) {
    FLAMEGPU->message_out.setVariable("x", 1);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(at_in, flamegpu::MessageBruteForce, flamegpu::MessageNone) {
    unsigned int count = 0;
    for (const auto& message : FLAMEGPU->message_in) {
        (void)message;
        ++count;
    }
    FLAMEGPU->setVariable<unsigned int>("count", count);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(at_in2, flamegpu::MessageBruteForce, flamegpu::MessageNone) {
    unsigned int c0 = 0, c1 = 0;
    for (const auto& message : FLAMEGPU->message_in) {
        const int x = message.getVariable<int>("x");
        if (x == 0) ++c0;
        else if (x == 1) ++c1;
    }
    FLAMEGPU->setVariable<unsigned int>("count0", c0);
    FLAMEGPU->setVariable<unsigned int>("count1", c1);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(at_opt_out, flamegpu::MessageNone, flamegpu::MessageBruteForce) {
    if (FLAMEGPU->getVariable<unsigned int>("do_out") > 0) {
        FLAMEGPU->message_out.setVariable("x", 0);
        FLAMEGPU->setVariable<unsigned int>("do_out", 0);
    } else {
        FLAMEGPU->setVariable<unsigned int>("do_out", 1);
    }
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(at_opt_out2, flamegpu::MessageNone, flamegpu::MessageBruteForce) {
    if (FLAMEGPU->getVariable<unsigned int>("do_out") > 0) FLAMEGPU->message_out.setVariable("x", 1);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(at_out_1, flamegpu::MessageNone, flamegpu::MessageBruteForce) {
    FLAMEGPU->message_out.setVariable("x", 1);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(at_out_2, flamegpu::MessageNone, flamegpu::MessageBruteForce) {
    FLAMEGPU->message_out.setVariable("x", 2);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(at_in3, flamegpu::MessageBruteForce, flamegpu::MessageNone) {
    unsigned int c0 = 0, c1 = 0, c2 = 0;
    for (const auto& message : FLAMEGPU->message_in) {
        const int x = message.getVariable<int>("x");
        if (x == 1) ++c1;
        else if (x == 2) ++c2;
        else ++c0;
    }
    FLAMEGPU->setVariable<unsigned int>("c0", c0);
    FLAMEGPU->setVariable<unsigned int>("c1", c1);
    FLAMEGPU->setVariable<unsigned int>("c2", c2);
    return flamegpu::ALIVE;
}

namespace {

void* make_truncate(const double*, int32_t) {
    auto* m = new flamegpu::ModelDescription("Truncate");
    auto msg = m->newMessage("Message");
    msg.newVariable<int>("x");
    flamegpu::AgentDescription a = m->newAgent("Agent");
    a.newVariable<unsigned int>("count");
    auto fo = a.newFunction("out", at_out);
    fo.setMessageOutput(msg);
    auto fi = a.newFunction("in", at_in);
    fi.setMessageInput(msg);
    m->newLayer().addAgentFunction(fo);
    m->newLayer().addAgentFunction(fi);
    return m;
}

void* make_append(const double*, int32_t) {
    auto* m = new flamegpu::ModelDescription("Append");
    auto msg = m->newMessage("Message");
    msg.newVariable<int>("x");
    flamegpu::AgentDescription a = m->newAgent("Agent");
    a.newVariable<unsigned int>("count0");
    a.newVariable<unsigned int>("count1");
    auto fo = a.newFunction("out", at_out);
    fo.setMessageOutput(msg);
    auto fo2 = a.newFunction("out2", at_out2);
    fo2.setMessageOutput(msg);
    auto fi = a.newFunction("in", at_in2);
    fi.setMessageInput(msg);
    m->newLayer().addAgentFunction(fo);
    m->newLayer().addAgentFunction(fo2);
    m->newLayer().addAgentFunction(fi);
    return m;
}

void* make_opt_truncate(const double*, int32_t) {
    auto* m = new flamegpu::ModelDescription("OptionalTruncate");
    auto msg = m->newMessage("Message");
    msg.newVariable<int>("x");
    flamegpu::AgentDescription a = m->newAgent("Agent");
    a.newVariable<unsigned int>("count");
    a.newVariable<unsigned int>("do_out");
    auto fo = a.newFunction("out", at_opt_out);
    fo.setMessageOutputOptional(true);
    fo.setMessageOutput(msg);
    auto fi = a.newFunction("in", at_in);
    fi.setMessageInput(msg);
    m->newLayer().addAgentFunction(fo);
    m->newLayer().addAgentFunction(fi);
    return m;
}

void* make_opt_append(const double*, int32_t) {
    auto* m = new flamegpu::ModelDescription("OptionalAppend");
    auto msg = m->newMessage("Message");
    msg.newVariable<int>("x");
    flamegpu::AgentDescription a = m->newAgent("Agent");
    a.newVariable<unsigned int>("count0");
    a.newVariable<unsigned int>("count1");
    a.newVariable<unsigned int>("do_out");
    auto fo = a.newFunction("out", at_opt_out);
    fo.setMessageOutputOptional(true);
    fo.setMessageOutput(msg);
    auto fo2 = a.newFunction("out2", at_opt_out2);
    fo2.setMessageOutputOptional(true);
    fo2.setMessageOutput(msg);
    auto fi = a.newFunction("in", at_in2);
    fi.setMessageInput(msg);
    m->newLayer().addAgentFunction(fo);
    m->newLayer().addAgentFunction(fo2);
    m->newLayer().addAgentFunction(fi);
    return m;
}

void* make_append_resize(const double*, int32_t) {
    auto* m = new flamegpu::ModelDescription("AppendResize");
    auto msg = m->newMessage("Message");
    msg.newVariable<int>("x");
    flamegpu::AgentDescription a = m->newAgent("a");
    auto f1 = a.newFunction("Out_1", at_out_1);
    f1.setMessageOutput(msg);
    flamegpu::AgentDescription b = m->newAgent("b");
    auto f2 = b.newFunction("Out_2", at_out_2);
    f2.setMessageOutput(msg);
    flamegpu::AgentDescription c = m->newAgent("c");
    c.newVariable<unsigned int>("c0", 0u);
    c.newVariable<unsigned int>("c1", 0u);
    c.newVariable<unsigned int>("c2", 0u);
    auto fi = c.newFunction("In", at_in3);
    fi.setMessageInput(msg);
    m->newLayer().addAgentFunction(f1);
    m->newLayer().addAgentFunction(f2);
    m->newLayer().addAgentFunction(fi);
    return m;
}

struct Register {
    Register() {
        fgs_register_model("at_truncate", &make_truncate);
        fgs_register_model("at_append", &make_append);
        fgs_register_model("at_opt_truncate", &make_opt_truncate);
        fgs_register_model("at_opt_append", &make_opt_append);
        fgs_register_model("at_append_resize", &make_append_resize);
    }
} reg;

}  // namespace
