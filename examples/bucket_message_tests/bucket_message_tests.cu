// Bucket message test models, written against the FLAME GPU 2 API: the models
// of the reference's tests tests/test_cases/runtime/messaging/test_bucket.cu.
//
// Registered model "bucket_messages", parameters [variant, persistent]:
//   agent "agent" (id, do_output, count1, count2, sum, index, v[3] read back
//   as message_read[3]) over a bucket message list "bucket":
//     0 Mandatory: bounds [12, 12 + 512]; every agent outputs its id with the
//       key 12 + id / 2, then reads the bucket 12 + (id - 1) / 2 (id 0 reads
//       its own): count1 = messages iterated, count2 = size(), sum = ids.
//     1 Optional: as 0, only agents with do_output set output.
//     2 OptionalNone: no agent outputs.
//     3 Mandatory_Range: as 0, reading the four buckets from
//       12 + (id / 8) * 4 with message_in(begin, end); count2 = the size of
//       bucket 12 + id / 2.
//     4 ArrayVariable: bounds [0, 1024]; every agent outputs v = index * (3,
//       7, 11) with the key index, then reads its own bucket.
//     5 Persistence: bounds [0, 1024]; on even steps every agent outputs its
//       id to bucket 0, then every agent reads bucket 0 (count1, sum); with
//       parameter 1 set the list is persistent.
//     6 BadKey: every agent outputs with the key 12 + 513, past the bounds
//       [12, 12 + 512] (a device error).
//     7 NoUpperBound: the list has no upper bound (the simulation cannot be
//       built).
//   fg_test_bucket_description() runs the reference's description checks
//   (DescriptionValidation) and returns one bit per check that held.
#include <cstdint>

#include "flamegpu/flamegpu.h"
#include "flamegpu_gb300/fg_sim.h"

FLAMEGPU_AGENT_FUNCTION(bk_out_mandatory, flamegpu::MessageNone, flamegpu::MessageBucket) {
    const int id = FLAMEGPU->getVariable<int>("id");
    FLAMEGPU->message_out.setVariable<int>("id", id);
    FLAMEGPU->message_out.setKey(12 + id / 2);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(bk_out_optional, flamegpu::MessageNone, flamegpu::MessageBucket) {
    if (FLAMEGPU->getVariable<int>("do_output")) {
        const int id = FLAMEGPU->getVariable<int>("id");
        FLAMEGPU->message_out.setVariable<int>("id", id);
        FLAMEGPU->message_out.setKey(12 + id / 2);
    }
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(bk_out_none, flamegpu::MessageNone, flamegpu::MessageBucket) { return flamegpu::ALIVE; }
FLAMEGPU_AGENT_FUNCTION(bk_out_bad, flamegpu::MessageNone, flamegpu::MessageBucket) {
    FLAMEGPU->message_out.setVariable<int>("id", FLAMEGPU->getVariable<int>("id"));
    FLAMEGPU->message_out.setKey(12 + 513);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(bk_in, flamegpu::MessageBucket, flamegpu::MessageNone) {
    const int id = FLAMEGPU->getVariable<int>("id");
    const int id_m1 = id == 0 ? 0 : id - 1;
    unsigned int count = 0, sum = 0;
    for (auto& m : FLAMEGPU->message_in(12 + id_m1 / 2)) {
        ++count;
        sum += m.getVariable<int>("id");
    }
    FLAMEGPU->setVariable<unsigned int>("count1", count);
    FLAMEGPU->setVariable<unsigned int>("count2", FLAMEGPU->message_in(12 + id_m1 / 2).size());
    FLAMEGPU->setVariable<unsigned int>("sum", sum);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(bk_in_range, flamegpu::MessageBucket, flamegpu::MessageNone) {
    const int id = FLAMEGPU->getVariable<int>("id");
    const int begin = 12 + (id / 8) * 4;
    unsigned int count = 0, sum = 0;
    for (auto& m : FLAMEGPU->message_in(begin, begin + 4)) {
        ++count;
        sum += m.getVariable<int>("id");
    }
    FLAMEGPU->setVariable<unsigned int>("count1", count);
    FLAMEGPU->setVariable<unsigned int>("count2", FLAMEGPU->message_in(12 + id / 2).size());
    FLAMEGPU->setVariable<unsigned int>("sum", sum);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(bk_array_out, flamegpu::MessageNone, flamegpu::MessageBucket) {
    const unsigned int index = FLAMEGPU->getVariable<unsigned int>("index");
    FLAMEGPU->message_out.setVariable<unsigned int, 3>("v", 0, index * 3);
    FLAMEGPU->message_out.setVariable<unsigned int, 3>("v", 1, index * 7);
    FLAMEGPU->message_out.setVariable<unsigned int, 3>("v", 2, index * 11);
    FLAMEGPU->message_out.setKey(static_cast<int>(index));
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(bk_array_in, flamegpu::MessageBucket, flamegpu::MessageNone) {
    const unsigned int index = FLAMEGPU->getVariable<unsigned int>("index");
    for (auto& m : FLAMEGPU->message_in(static_cast<int>(index))) {
        FLAMEGPU->setVariable<unsigned int, 3>("message_read", 0, m.getVariable<unsigned int, 3>("v", 0));
        FLAMEGPU->setVariable<unsigned int, 3>("message_read", 1, m.getVariable<unsigned int, 3>("v", 1));
        FLAMEGPU->setVariable<unsigned int, 3>("message_read", 2, m.getVariable<unsigned int, 3>("v", 2));
    }
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION_CONDITION(bk_even_only) { return FLAMEGPU->getStepCounter() % 2 == 0; }
FLAMEGPU_AGENT_FUNCTION(bk_out_simple, flamegpu::MessageNone, flamegpu::MessageBucket) {
    FLAMEGPU->message_out.setVariable<int>("id", FLAMEGPU->getVariable<int>("id"));
    FLAMEGPU->message_out.setKey(0);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(bk_in_simple, flamegpu::MessageBucket, flamegpu::MessageNone) {
    unsigned int count = 0, sum = 0;
    for (auto& m : FLAMEGPU->message_in(0)) {
        ++count;
        sum += m.getVariable<int>("id");
    }
    FLAMEGPU->setVariable<unsigned int>("count1", count);
    FLAMEGPU->setVariable<unsigned int>("sum", sum);
    return flamegpu::ALIVE;
}

namespace {

double param(const double* p, int32_t np, int i, double d) { return i < np ? p[i] : d; }

void two_layers(flamegpu::ModelDescription* m, flamegpu::AgentFunctionDescription fo, flamegpu::AgentFunctionDescription fi) {
    fo.setMessageOutput("bucket");
    fi.setMessageInput("bucket");
    m->newLayer().addAgentFunction(fo);
    m->newLayer().addAgentFunction(fi);
}

void* make_bucket_messages(const double* p, int32_t np) {
    const int variant = static_cast<int>(param(p, np, 0, 0));
    auto* m = new flamegpu::ModelDescription("BucketMessageTest");
    flamegpu::MessageBucket::Description msg = m->newMessage<flamegpu::MessageBucket>("bucket");
    if (variant == 4 || variant == 5) msg.setBounds(0, 1024);
    else if (variant != 7) msg.setBounds(12, 12 + 512);
    msg.newVariable<int>("id");
    msg.newVariable<unsigned int, 3>("v");
    if (variant == 5 && param(p, np, 1, 0) != 0.0) msg.setPersistent(true);
    flamegpu::AgentDescription a = m->newAgent("agent");
    a.newVariable<int>("id");
    a.newVariable<int>("do_output", 0);
    a.newVariable<unsigned int>("index", 0u);
    a.newVariable<unsigned int>("count1", 0u);
    a.newVariable<unsigned int>("count2", 0u);
    a.newVariable<unsigned int>("sum", 0u);
    a.newVariable<unsigned int, 3>("message_read", {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu});
    switch (variant) {
        case 1: two_layers(m, a.newFunction("out", bk_out_optional), a.newFunction("in", bk_in));
                m->Agent("agent").Function("out").setMessageOutputOptional(true); break;
        case 2: two_layers(m, a.newFunction("out", bk_out_none), a.newFunction("in", bk_in));
                m->Agent("agent").Function("out").setMessageOutputOptional(true); break;
        case 3: two_layers(m, a.newFunction("out", bk_out_mandatory), a.newFunction("in", bk_in_range)); break;
        case 4: two_layers(m, a.newFunction("out", bk_array_out), a.newFunction("in", bk_array_in)); break;
        case 5: {
            flamegpu::AgentFunctionDescription fo = a.newFunction("out", bk_out_simple);
            fo.setMessageOutputOptional(true);
            fo.setFunctionCondition(bk_even_only);
            two_layers(m, fo, a.newFunction("in", bk_in_simple));
            break;
        }
        case 6: two_layers(m, a.newFunction("out", bk_out_bad), a.newFunction("in", bk_in)); break;
        default: two_layers(m, a.newFunction("out", bk_out_mandatory), a.newFunction("in", bk_in)); break;
    }
    return m;
}

struct Register {
    Register() { fgs_register_model("bucket_messages", &make_bucket_messages); }
} reg;

template <typename F>
bool throws_invalid_argument(F f) {
    try {
        f();
    } catch (const flamegpu::exception::InvalidArgument&) {
        return true;
    } catch (...) {
        return false;
    }
    return false;
}
template <typename F>
bool no_throw(F f) {
    try {
        f();
    } catch (...) {
        return false;
    }
    return true;
}

}  // namespace

// The checks of test_bucket.cu DescriptionValidation, in order; bit k is set
// when check k held.
extern "C" uint32_t fg_test_bucket_description() {
    flamegpu::ModelDescription model("BucketMessageTest");
    flamegpu::MessageBucket::Description message = model.newMessage<flamegpu::MessageBucket>("buckets");
    uint32_t ok = 0;
    int k = 0;
    auto check = [&](bool held) { ok |= (held ? 1u : 0u) << k++; };
    check(throws_invalid_argument([&] { message.setUpperBound(0); }));  // lower bound 0: no buckets
    check(no_throw([&] { message.setLowerBound(10); }));
    check(no_throw([&] { message.setUpperBound(11); }));
    check(throws_invalid_argument([&] { message.setUpperBound(0); }));   // upper < lower
    check(no_throw([&] { message.setUpperBound(12); }));
    check(throws_invalid_argument([&] { message.setLowerBound(13); }));  // lower > upper
    check(throws_invalid_argument([&] { message.setBounds(12, 12); }));  // lower == upper
    check(throws_invalid_argument([&] { message.setBounds(13, 12); }));  // lower > upper
    check(no_throw([&] { message.setBounds(12, 13); }));
    check(no_throw([&] { message.newVariable<int>("somevar"); }));
    check(message.getLowerBound() == 12 && message.getUpperBound() == 13);
    return ok;
}
