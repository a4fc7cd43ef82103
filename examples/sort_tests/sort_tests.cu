// Automatic spatial agent sort and empty message lists, written against the
// FLAME GPU 2 API: the models of the reference's tests
// tests/test_cases/runtime/agent/detail/test_spatial_agent_sort.cu:15-240
// (AutomaticSpatialAgentSort.*) and
// tests/test_cases/runtime/messaging/test_spatial_3d.cu:495-540 (ReadEmpty).
//
// Registered models:
//   sort_order  params: variant. Agent "agent" (initial_order int) reading a
//               Spatial3D (or 2D) message list over [-5, 5], radius 0.2, with a
//               function that does nothing:
//                 0 SortingDisabled (x, y, z; sort period 0)
//                 1 SortEveryStep (x, y, z)
//                 2 SortEveryStep_no_default (x, y, z; the only state "foobar")
//                 3 SortEveryStep_vec2 (a packed "xy" float[2], Spatial2D)
//                 4 SortEveryStep_vec3 (a packed "xyz" float[3])
//   read_empty  ReadEmpty: one agent counts the messages around (0, 0, 0) of a
//               list nothing has output (bounds [-3, 3], radius 2)
#include "flamegpu/flamegpu.h"
#include "flamegpu_gb300/fg_sim.h"

FLAMEGPU_AGENT_FUNCTION(sort_dummy_3d, flamegpu::MessageSpatial3D, flamegpu::MessageNone) { return flamegpu::ALIVE; }
FLAMEGPU_AGENT_FUNCTION(sort_dummy_2d, flamegpu::MessageSpatial2D, flamegpu::MessageNone) { return flamegpu::ALIVE; }
FLAMEGPU_AGENT_FUNCTION(read_empty_count, flamegpu::MessageSpatial3D, flamegpu::MessageNone) {
    unsigned int count = 0;
    for (const auto& message : FLAMEGPU->message_in(0, 0, 0)) {
        (void)message;
        count++;
    }
    FLAMEGPU->setVariable<unsigned int>("count", count);
    return flamegpu::ALIVE;
}

namespace {

void* make_sort_order(const double* p, int32_t np) {
    const int variant = np > 0 ? static_cast<int>(p[0]) : 1;
    auto* m = new flamegpu::ModelDescription("model");
    flamegpu::AgentDescription a = m->newAgent("agent");
    a.newVariable<int>("initial_order");
    if (variant == 2) a.newState("foobar");
    if (variant == 3) {
        a.newVariable<float, 2>("xy");
    } else if (variant == 4) {
        a.newVariable<float, 3>("xyz");
    } else {
        a.newVariable<float>("x");
        a.newVariable<float>("y");
        a.newVariable<float>("z");
    }
    if (variant == 0) a.setSortPeriod(0);
    if (variant == 3) {
        auto msg = m->newMessage<flamegpu::MessageSpatial2D>("location");
        msg.setMin(-5, -5);
        msg.setMax(5, 5);
        msg.setRadius(0.2f);
        auto f = a.newFunction("dummySpatialFunc", sort_dummy_2d);
        f.setMessageInput("location");
        m->newLayer().addAgentFunction(f);
    } else {
        auto msg = m->newMessage<flamegpu::MessageSpatial3D>("location");
        msg.setMin(-5, -5, -5);
        msg.setMax(5, 5, 5);
        msg.setRadius(0.2f);
        auto f = a.newFunction("dummySpatialFunc", sort_dummy_3d);
        f.setMessageInput("location");
        m->newLayer().addAgentFunction(f);
    }
    return m;
}

void* make_read_empty(const double*, int32_t) {
    auto* m = new flamegpu::ModelDescription("Model");
    auto msg = m->newMessage<flamegpu::MessageSpatial3D>("location");
    msg.setMin(-3, -3, -3);
    msg.setMax(3, 3, 3);
    msg.setRadius(2);
    msg.newVariable<flamegpu::id_t>("id");
    flamegpu::AgentDescription a = m->newAgent("agent");
    a.newVariable<unsigned int>("count", 0);
    auto f = a.newFunction("in", read_empty_count);
    f.setMessageInput("location");
    m->newLayer().addAgentFunction(f);
    return m;
}

struct Register {
    Register() {
        fgs_register_model("sort_order", &make_sort_order);
        fgs_register_model("read_empty", &make_read_empty);
    }
} reg;

}  // namespace
