// Array message test models, written against the FLAME GPU 2 API: the models
// of the reference's tests tests/test_cases/runtime/messaging/test_array.cu,
// test_array_2d.cu and test_array_3d.cu.
//
// Registered models, parameters [variant, dim x, dim y, dim z, radius]
// (dimensions past the model's own are ignored):
//   array1d, array2d, array3d  agent "agent" (index, x, y, z, message_write,
//       message_read, value_success) over an array message list "message"
//       (index, v, v2[3]); two layers, output then input:
//     0 Mandatory: every agent outputs index * 3 at the cell of message_write,
//       then reads the message at its own index's cell (at()).
//     1 Optional: as 0, only agents whose message_write is even output.
//     2 OptionalNone: no agent outputs.
//     3 Duplicate: as 0, but message_write 13 is output to cell 0 as well.
//     4 Moore, wrapped: every agent outputs at its (x, y, z); reads its
//       wrapped Moore neighbourhood (radius), counting the messages and
//       checking their values against their coordinates.
//     5 Moore, clamped: the same with message_in(x, y, z, radius).
//     6 von Neumann, wrapped (2D / 3D).  7 von Neumann, clamped (2D / 3D).
//     8 ReadEmpty: one function reads cell 0 of a list nothing output.
#include <cstdint>

#include "flamegpu/flamegpu.h"
#include "flamegpu_gb300/fg_sim.h"

namespace {

template <int D>
struct Coord {
    template <typename API>
    __device__ static void of(API* F, uint32_t i, uint32_t (&c)[3]) {
        const uint32_t dx = F->environment.template getProperty<uint32_t>("DIM_X");
        const uint32_t dy = F->environment.template getProperty<uint32_t>("DIM_Y");
        c[0] = i % dx;
        c[1] = D > 1 ? (i / dx) % dy : 0u;
        c[2] = D > 2 ? i / (dx * dy) : 0u;
    }
};

template <typename Out>
__device__ void set_index(const Out& o, const uint32_t (&c)[3], std::integral_constant<int, 1>) { o.setIndex(c[0]); }
template <typename Out>
__device__ void set_index(const Out& o, const uint32_t (&c)[3], std::integral_constant<int, 2>) { o.setIndex(c[0], c[1]); }
template <typename Out>
__device__ void set_index(const Out& o, const uint32_t (&c)[3], std::integral_constant<int, 3>) {
    o.setIndex(c[0], c[1], c[2]);
}
template <typename In>
__device__ auto at(const In& in, const uint32_t (&c)[3], std::integral_constant<int, 1>) { return in.at(c[0]); }
template <typename In>
__device__ auto at(const In& in, const uint32_t (&c)[3], std::integral_constant<int, 2>) { return in.at(c[0], c[1]); }
template <typename In>
__device__ auto at(const In& in, const uint32_t (&c)[3], std::integral_constant<int, 3>) { return in.at(c[0], c[1], c[2]); }

// variant 0 / 1 / 3 output
template <int D, bool OPTIONAL, bool BAD, typename API>
__device__ flamegpu::AGENT_STATUS out_write(API* F) {
    uint32_t w = F->template getVariable<uint32_t>("message_write");
    if (OPTIONAL && w % 2 != 0) return flamegpu::ALIVE;
    F->message_out.template setVariable<uint32_t>("index", w * 3);
    if (BAD && w == 13) w = 0;
    uint32_t c[3];
    Coord<D>::of(F, w, c);
    set_index(F->message_out, c, std::integral_constant<int, D>());
    return flamegpu::ALIVE;
}
// variants 4 - 7 output: the agent's own cell, values from its coordinates
template <int D, typename API>
__device__ flamegpu::AGENT_STATUS out_xyz(API* F) {
    const uint32_t c[3] = {F->template getVariable<uint32_t>("x"), F->template getVariable<uint32_t>("y"),
                           F->template getVariable<uint32_t>("z")};
    F->message_out.template setVariable<uint32_t>("index", F->template getVariable<uint32_t>("index"));
    F->message_out.template setVariable<uint32_t>("v", c[0] * 3);
    F->message_out.template setVariable<uint32_t, 3>("v2", 0, c[0] * 3);
    F->message_out.template setVariable<uint32_t, 3>("v2", 1, c[1] * 7);
    F->message_out.template setVariable<uint32_t, 3>("v2", 2, c[2] * 11);
    set_index(F->message_out, c, std::integral_constant<int, D>());
    return flamegpu::ALIVE;
}
// variants 0 - 3 input: the message at the agent's own index
template <int D, typename API>
__device__ flamegpu::AGENT_STATUS in_at(API* F) {
    uint32_t c[3];
    Coord<D>::of(F, F->template getVariable<uint32_t>("index"), c);
    const auto m = at(F->message_in, c, std::integral_constant<int, D>());
    F->template setVariable<uint32_t>("message_read", m.template getVariable<uint32_t>("index"));
    return flamegpu::ALIVE;
}
// variants 4 - 7 input: count the neighbourhood and check each message's values
template <int D, typename Filter, typename API>
__device__ void count_check(API* F, const Filter& filter) {
    uint32_t count = 0;
    bool ok = true;
    for (const auto& m : filter) {
        ++count;
        const uint32_t mz = D > 2 ? m.getZ() : 0u;
        const uint32_t my = D > 1 ? m.getY() : 0u;
        ok = ok && m.template getVariable<uint32_t, 3>("v2", 0) == m.getX() * 3 &&
             m.template getVariable<uint32_t, 3>("v2", 1) == my * 7 &&
             m.template getVariable<uint32_t, 3>("v2", 2) == mz * 11 && m.template getVariable<uint32_t>("v") == m.getX() * 3;
    }
    F->template setVariable<uint32_t>("message_read", count);
    F->template setVariable<uint32_t>("value_success", ok ? 1u : 0u);
}

}  // namespace

#define FG_ARRAY_FUNCTIONS(D, MSG)                                                                          \
    FLAMEGPU_AGENT_FUNCTION(out_mandatory_##D, flamegpu::MessageNone, MSG) { return out_write<D, false, false>(FLAMEGPU); } \
    FLAMEGPU_AGENT_FUNCTION(out_optional_##D, flamegpu::MessageNone, MSG) { return out_write<D, true, false>(FLAMEGPU); }   \
    FLAMEGPU_AGENT_FUNCTION(out_none_##D, flamegpu::MessageNone, MSG) { return flamegpu::ALIVE; }                           \
    FLAMEGPU_AGENT_FUNCTION(out_bad_##D, flamegpu::MessageNone, MSG) { return out_write<D, false, true>(FLAMEGPU); }         \
    FLAMEGPU_AGENT_FUNCTION(out_xyz_##D, flamegpu::MessageNone, MSG) { return out_xyz<D>(FLAMEGPU); }                       \
    FLAMEGPU_AGENT_FUNCTION(in_at_##D, MSG, flamegpu::MessageNone) { return in_at<D>(FLAMEGPU); }

FG_ARRAY_FUNCTIONS(1, flamegpu::MessageArray)
FG_ARRAY_FUNCTIONS(2, flamegpu::MessageArray2D)
FG_ARRAY_FUNCTIONS(3, flamegpu::MessageArray3D)

FLAMEGPU_AGENT_FUNCTION(in_moore_w_1, flamegpu::MessageArray, flamegpu::MessageNone) {
    count_check<1>(FLAMEGPU, FLAMEGPU->message_in.wrap(FLAMEGPU->getVariable<uint32_t>("x"),
                                                       FLAMEGPU->environment.getProperty<uint32_t>("RADIUS")));
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(in_moore_1, flamegpu::MessageArray, flamegpu::MessageNone) {
    count_check<1>(FLAMEGPU, FLAMEGPU->message_in(FLAMEGPU->getVariable<uint32_t>("x"),
                                                  FLAMEGPU->environment.getProperty<uint32_t>("RADIUS")));
    return flamegpu::ALIVE;
}
#define FG_ARRAY_SEARCH_2D(NAME, CALL)                                                                       \
    FLAMEGPU_AGENT_FUNCTION(NAME, flamegpu::MessageArray2D, flamegpu::MessageNone) {                         \
        count_check<2>(FLAMEGPU, FLAMEGPU->message_in CALL(FLAMEGPU->getVariable<uint32_t>("x"),             \
                                                           FLAMEGPU->getVariable<uint32_t>("y"),             \
                                                           FLAMEGPU->environment.getProperty<uint32_t>("RADIUS"))); \
        return flamegpu::ALIVE;                                                                              \
    }
#define FG_ARRAY_SEARCH_3D(NAME, CALL)                                                                       \
    FLAMEGPU_AGENT_FUNCTION(NAME, flamegpu::MessageArray3D, flamegpu::MessageNone) {                         \
        count_check<3>(FLAMEGPU, FLAMEGPU->message_in CALL(FLAMEGPU->getVariable<uint32_t>("x"),             \
                                                           FLAMEGPU->getVariable<uint32_t>("y"),             \
                                                           FLAMEGPU->getVariable<uint32_t>("z"),             \
                                                           FLAMEGPU->environment.getProperty<uint32_t>("RADIUS"))); \
        return flamegpu::ALIVE;                                                                              \
    }
FG_ARRAY_SEARCH_2D(in_moore_w_2, .wrap)
FG_ARRAY_SEARCH_2D(in_moore_2, )
FG_ARRAY_SEARCH_2D(in_vn_w_2, .vn_wrap)
FG_ARRAY_SEARCH_2D(in_vn_2, .vn)
FG_ARRAY_SEARCH_3D(in_moore_w_3, .wrap)
FG_ARRAY_SEARCH_3D(in_moore_3, )
FG_ARRAY_SEARCH_3D(in_vn_w_3, .vn_wrap)
FG_ARRAY_SEARCH_3D(in_vn_3, .vn)

FLAMEGPU_AGENT_FUNCTION(read_empty_2, flamegpu::MessageArray2D, flamegpu::MessageNone) {
    FLAMEGPU->setVariable<uint32_t>("message_read", FLAMEGPU->message_in.at(0, 0).getVariable<uint32_t>("v"));
    return flamegpu::ALIVE;
}

namespace {

double param(const double* p, int32_t np, int i, double d) { return i < np ? p[i] : d; }

// The model of every variant but its two functions: environment (dimensions,
// radius), the message list and the agent.
template <int D, typename MSG>
flamegpu::ModelDescription* base_model(const double* p, int32_t np) {
    const uint32_t dims[3] = {static_cast<uint32_t>(param(p, np, 1, 12)), static_cast<uint32_t>(param(p, np, 2, 13)),
                              static_cast<uint32_t>(param(p, np, 3, 5))};
    auto* m = new flamegpu::ModelDescription("array_messages");
    flamegpu::EnvironmentDescription env = m->Environment();
    env.newProperty<uint32_t>("DIM_X", dims[0]);
    env.newProperty<uint32_t>("DIM_Y", D > 1 ? dims[1] : 1u);
    env.newProperty<uint32_t>("RADIUS", static_cast<uint32_t>(param(p, np, 4, 1)));
    auto msg = m->newMessage<MSG>("message");
    if constexpr (D == 1) msg.setLength(dims[0]);
    else if constexpr (D == 2) msg.setDimensions(dims[0], dims[1]);
    else msg.setDimensions(dims[0], dims[1], dims[2]);
    msg.template newVariable<uint32_t>("index");
    msg.template newVariable<uint32_t>("v");
    msg.template newVariable<uint32_t, 3>("v2");
    flamegpu::AgentDescription a = m->newAgent("agent");
    for (const char* v : {"index", "x", "y", "z", "message_write", "value_success"}) a.newVariable<uint32_t>(v, 0u);
    a.newVariable<uint32_t>("message_read", 0xFFFFFFFFu);
    return m;
}

void two_layers(flamegpu::ModelDescription* m, flamegpu::AgentFunctionDescription fo, flamegpu::AgentFunctionDescription fi) {
    fo.setMessageOutput("message");
    fi.setMessageInput("message");
    m->newLayer().addAgentFunction(fo);
    m->newLayer().addAgentFunction(fi);
}

void* make_array1d(const double* p, int32_t np) {
    auto* m = base_model<1, flamegpu::MessageArray>(p, np);
    flamegpu::AgentDescription a = m->Agent("agent");
    switch (static_cast<int>(param(p, np, 0, 0))) {
        case 1: two_layers(m, a.newFunction("out", out_optional_1), a.newFunction("in", in_at_1));
                m->Agent("agent").Function("out").setMessageOutputOptional(true); break;
        case 2: two_layers(m, a.newFunction("out", out_none_1), a.newFunction("in", in_at_1));
                m->Agent("agent").Function("out").setMessageOutputOptional(true); break;
        case 3: two_layers(m, a.newFunction("out", out_bad_1), a.newFunction("in", in_at_1)); break;
        case 4: two_layers(m, a.newFunction("out", out_xyz_1), a.newFunction("in", in_moore_w_1)); break;
        case 5: two_layers(m, a.newFunction("out", out_xyz_1), a.newFunction("in", in_moore_1)); break;
        default: two_layers(m, a.newFunction("out", out_mandatory_1), a.newFunction("in", in_at_1)); break;
    }
    return m;
}

void* make_array2d(const double* p, int32_t np) {
    auto* m = base_model<2, flamegpu::MessageArray2D>(p, np);
    flamegpu::AgentDescription a = m->Agent("agent");
    switch (static_cast<int>(param(p, np, 0, 0))) {
        case 1: two_layers(m, a.newFunction("out", out_optional_2), a.newFunction("in", in_at_2));
                m->Agent("agent").Function("out").setMessageOutputOptional(true); break;
        case 2: two_layers(m, a.newFunction("out", out_none_2), a.newFunction("in", in_at_2));
                m->Agent("agent").Function("out").setMessageOutputOptional(true); break;
        case 3: two_layers(m, a.newFunction("out", out_bad_2), a.newFunction("in", in_at_2)); break;
        case 4: two_layers(m, a.newFunction("out", out_xyz_2), a.newFunction("in", in_moore_w_2)); break;
        case 5: two_layers(m, a.newFunction("out", out_xyz_2), a.newFunction("in", in_moore_2)); break;
        case 6: two_layers(m, a.newFunction("out", out_xyz_2), a.newFunction("in", in_vn_w_2)); break;
        case 7: two_layers(m, a.newFunction("out", out_xyz_2), a.newFunction("in", in_vn_2)); break;
        case 8: {
            flamegpu::AgentFunctionDescription fi = a.newFunction("in", read_empty_2);
            fi.setMessageInput("message");
            m->newLayer().addAgentFunction(fi);
            break;
        }
        default: two_layers(m, a.newFunction("out", out_mandatory_2), a.newFunction("in", in_at_2)); break;
    }
    return m;
}

void* make_array3d(const double* p, int32_t np) {
    auto* m = base_model<3, flamegpu::MessageArray3D>(p, np);
    flamegpu::AgentDescription a = m->Agent("agent");
    switch (static_cast<int>(param(p, np, 0, 0))) {
        case 1: two_layers(m, a.newFunction("out", out_optional_3), a.newFunction("in", in_at_3));
                m->Agent("agent").Function("out").setMessageOutputOptional(true); break;
        case 2: two_layers(m, a.newFunction("out", out_none_3), a.newFunction("in", in_at_3));
                m->Agent("agent").Function("out").setMessageOutputOptional(true); break;
        case 3: two_layers(m, a.newFunction("out", out_bad_3), a.newFunction("in", in_at_3)); break;
        case 4: two_layers(m, a.newFunction("out", out_xyz_3), a.newFunction("in", in_moore_w_3)); break;
        case 5: two_layers(m, a.newFunction("out", out_xyz_3), a.newFunction("in", in_moore_3)); break;
        case 6: two_layers(m, a.newFunction("out", out_xyz_3), a.newFunction("in", in_vn_w_3)); break;
        case 7: two_layers(m, a.newFunction("out", out_xyz_3), a.newFunction("in", in_vn_3)); break;
        default: two_layers(m, a.newFunction("out", out_mandatory_3), a.newFunction("in", in_at_3)); break;
    }
    return m;
}

struct Register {
    Register() {
        fgs_register_model("array1d", &make_array1d);
        fgs_register_model("array2d", &make_array2d);
        fgs_register_model("array3d", &make_array3d);
    }
} reg;

}  // namespace
