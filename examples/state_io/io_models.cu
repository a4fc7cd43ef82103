// State-file test models, written against the FLAME GPU 2 API: the models of
// the reference's IO tests (tests/test_cases/io/test_io.cu).
//
// Registered models:
//   io_types    MiniSim (:255-300): agent "a" with one variable of every
//               scalar type and NaN / infinity floats and doubles, agent "b"
//               (states "1", "2") with three-element arrays of every type,
//               environment properties of every type, as arrays, and NaN /
//               infinities. No macro properties (not supported here).
//   io_agentid  IOTest2 (:622-735): agent "agent" with an id_t variable
//               id_other; one function that does nothing.
#include <cmath>
#include <limits>

#include "flamegpu/flamegpu.h"
#include "flamegpu_gb300/fg_sim.h"

FLAMEGPU_AGENT_FUNCTION(io_nothing, flamegpu::MessageNone, flamegpu::MessageNone) { return flamegpu::ALIVE; }

namespace {

void* make_io_types(const double*, int32_t) {
    auto* m = new flamegpu::ModelDescription("test_model");
    flamegpu::AgentDescription a = m->newAgent("a");
    a.newVariable<float>("float");
    a.newVariable<double>("double");
    a.newVariable<int64_t>("int64_t");
    a.newVariable<uint64_t>("uint64_t");
    a.newVariable<int32_t>("int32_t");
    a.newVariable<uint32_t>("uint32_t");
    a.newVariable<int16_t>("int16_t");
    a.newVariable<uint16_t>("uint16_t");
    a.newVariable<int8_t>("int8_t");
    a.newVariable<uint8_t>("uint8_t");
    a.newVariable<float>("float_qnan");
    a.newVariable<float>("float_snan");
    a.newVariable<float>("float_inf");
    a.newVariable<float>("float_inf_neg");
    a.newVariable<double>("double_qnan");
    a.newVariable<double>("double_snan");
    a.newVariable<double>("double_inf");
    a.newVariable<double>("double_inf_neg");
    flamegpu::AgentDescription b = m->newAgent("b");
    b.newState("1");
    b.newState("2");
    b.newVariable<float, 3>("float");
    b.newVariable<double, 3>("double");
    b.newVariable<int64_t, 3>("int64_t");
    b.newVariable<uint64_t, 3>("uint64_t");
    b.newVariable<int32_t, 3>("int32_t");
    b.newVariable<uint32_t, 3>("uint32_t");
    b.newVariable<int16_t, 3>("int16_t");
    b.newVariable<uint16_t, 3>("uint16_t");
    b.newVariable<int8_t, 3>("int8_t");
    b.newVariable<uint8_t, 3>("uint8_t");
    flamegpu::EnvironmentDescription e = m->Environment();
    e.newProperty<float>("float", 12.0f);
    e.newProperty<double>("double", 13.0);
    e.newProperty<int64_t>("int64_t", 14);
    e.newProperty<uint64_t>("uint64_t", 15u);
    e.newProperty<int32_t>("int32_t", 16);
    e.newProperty<uint32_t>("uint32_t", 17u);
    e.newProperty<int16_t>("int16_t", 18);
    e.newProperty<uint16_t>("uint16_t", 19u);
    e.newProperty<int8_t>("int8_t", 20);
    e.newProperty<uint8_t>("uint8_t", 21u);
    e.newProperty<float, 3>("float_a", {12.0f, 0.0f, 1.0f});
    e.newProperty<double, 3>("double_a", {13.0, 0.0, 1.0});
    e.newProperty<int64_t, 3>("int64_t_a", {14, 0, 1});
    e.newProperty<uint64_t, 3>("uint64_t_a", {15u, 0u, 1u});
    e.newProperty<int32_t, 3>("int32_t_a", {16, 0, 1});
    e.newProperty<uint32_t, 3>("uint32_t_a", {17u, 0u, 1u});
    e.newProperty<int16_t, 3>("int16_t_a", {18, 0, 1});
    e.newProperty<uint16_t, 3>("uint16_t_a", {19u, 0u, 1u});
    e.newProperty<int8_t, 3>("int8_t_a", {20, 0, 1});
    e.newProperty<uint8_t, 3>("uint8_t_a", {21u, 0u, 1u});
    e.newProperty<float>("float_qnan", std::numeric_limits<float>::quiet_NaN());
    e.newProperty<float>("float_snan", std::numeric_limits<float>::signaling_NaN());
    e.newProperty<float>("float_inf", std::numeric_limits<float>::infinity());
    e.newProperty<float>("float_inf_neg", -std::numeric_limits<float>::infinity());
    e.newProperty<double>("double_qnan", std::numeric_limits<double>::quiet_NaN());
    e.newProperty<double>("double_snan", std::numeric_limits<double>::signaling_NaN());
    e.newProperty<double>("double_inf", std::numeric_limits<double>::infinity());
    e.newProperty<double>("double_inf_neg", -std::numeric_limits<double>::infinity());
    flamegpu::AgentFunctionDescription fa = a.newFunction("nothing_a", io_nothing);
    m->newLayer().addAgentFunction(fa);
    return m;
}

void* make_io_agentid(const double*, int32_t) {
    auto* m = new flamegpu::ModelDescription("test_agentid");
    flamegpu::AgentDescription a = m->newAgent("agent");
    a.newVariable<flamegpu::id_t>("id_other", flamegpu::ID_NOT_SET);
    flamegpu::AgentFunctionDescription f = a.newFunction("nothing", io_nothing);
    m->newLayer().addAgentFunction(f);
    return m;
}

struct Register {
    Register() {
        fgs_register_model("io_types", &make_io_types);
        fgs_register_model("io_agentid", &make_io_agentid);
    }
} reg;

}  // namespace
