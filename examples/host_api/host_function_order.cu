// Host function order and exit conditions, written against the FLAME GPU 2
// API: the model of the reference's tests
// tests/test_cases/simulation/test_host_functions.cu (MiniSim).
//
// Registered model "host_function_order", parameter [with_second]: an init,
// a step and an exit function, an exit condition that returns EXIT the
// second time it runs, and a host layer function, each recording its kind
// (0 Init, 1 Step, 2 Exit, 3 HostLayer, 4 ExitCondition; 5-9 the second
// functions of each kind, added when with_second is set; the second exit
// condition always continues). fg_test_function_order() copies the record
// out; fg_test_host_function_duplicates() adds each kind of function twice
// and returns one bit per InvalidHostFunc raised.
#include <cstdint>
#include <cstring>
#include <mutex>
#include <vector>

#include "flamegpu/flamegpu.h"
#include "flamegpu_gb300/fg_sim.h"

namespace {
enum FunctionType { Init, Step, Exit, HostLayer, ExitCondition, Init2, Step2, Exit2, HostLayer2, ExitCondition2 };
std::mutex g_mu;
std::vector<int32_t> g_order;
void record(FunctionType t) {
    std::lock_guard<std::mutex> lock(g_mu);
    g_order.push_back(t);
}
}  // namespace

FLAMEGPU_INIT_FUNCTION(hfo_init) { record(Init); }
FLAMEGPU_STEP_FUNCTION(hfo_step) { record(Step); }
FLAMEGPU_EXIT_FUNCTION(hfo_exit) { record(Exit); }
FLAMEGPU_HOST_FUNCTION(hfo_host) { record(HostLayer); }
FLAMEGPU_EXIT_CONDITION(hfo_exit_condition) {
    record(ExitCondition);
    std::lock_guard<std::mutex> lock(g_mu);
    int seen = 0;
    for (int32_t a : g_order) seen += a == ExitCondition ? 1 : 0;
    return seen > 1 ? flamegpu::EXIT : flamegpu::CONTINUE;
}
FLAMEGPU_INIT_FUNCTION(hfo_init2) { record(Init2); }
FLAMEGPU_STEP_FUNCTION(hfo_step2) { record(Step2); }
FLAMEGPU_EXIT_FUNCTION(hfo_exit2) { record(Exit2); }
FLAMEGPU_HOST_FUNCTION(hfo_host2) { record(HostLayer2); }
FLAMEGPU_EXIT_CONDITION(hfo_exit_condition2) {
    record(ExitCondition2);
    return flamegpu::CONTINUE;
}

namespace {
void* make_host_function_order(const double* p, int32_t np) {
    const bool second = np > 0 && p[0] != 0.0;
    auto* m = new flamegpu::ModelDescription("model");
    m->newAgent("agent");
    flamegpu::LayerDescription layer = m->newLayer("hostfn_layer");
    m->addInitFunction(hfo_init);
    m->addStepFunction(hfo_step);
    m->addExitFunction(hfo_exit);
    m->addExitCondition(hfo_exit_condition);
    layer.addHostFunction(hfo_host);
    if (second) {
        m->addInitFunction(hfo_init2);
        m->addStepFunction(hfo_step2);
        m->addExitFunction(hfo_exit2);
        m->addExitCondition(hfo_exit_condition2);
        layer.addHostFunction(hfo_host2);
    }
    {
        std::lock_guard<std::mutex> lock(g_mu);
        g_order.clear();
    }
    return m;
}
struct Register {
    Register() { fgs_register_model("host_function_order", &make_host_function_order); }
} reg;

template <typename F>
bool raises_invalid_host_func(F f) {
    try {
        f();
    } catch (const flamegpu::exception::InvalidHostFunc&) {
        return true;
    } catch (...) {
        return false;
    }
    return false;
}
}  // namespace

extern "C" int32_t fg_test_function_order(int32_t* out, int32_t cap) {
    std::lock_guard<std::mutex> lock(g_mu);
    const int32_t n = static_cast<int32_t>(g_order.size());
    std::memcpy(out, g_order.data(), sizeof(int32_t) * static_cast<size_t>(n < cap ? n : cap));
    return n;
}

// test_host_functions.cu:206-223: adding a function of each kind twice raises
// InvalidHostFunc; one host function may be in two layers.
extern "C" uint32_t fg_test_host_function_duplicates() {
    flamegpu::ModelDescription m("model");
    flamegpu::LayerDescription l1 = m.newLayer("hostfn_layer");
    flamegpu::LayerDescription l2 = m.newLayer("hostfn_layer2");
    m.addInitFunction(hfo_init);
    m.addStepFunction(hfo_step);
    m.addExitFunction(hfo_exit);
    m.addExitCondition(hfo_exit_condition);
    l1.addHostFunction(hfo_host);
    uint32_t ok = 0;
    ok |= raises_invalid_host_func([&] { m.addInitFunction(hfo_init); }) ? 1u : 0u;
    ok |= raises_invalid_host_func([&] { l1.addHostFunction(hfo_host); }) ? 2u : 0u;
    ok |= raises_invalid_host_func([&] { m.addStepFunction(hfo_step); }) ? 4u : 0u;
    ok |= raises_invalid_host_func([&] { m.addExitCondition(hfo_exit_condition); }) ? 8u : 0u;
    ok |= raises_invalid_host_func([&] { m.addExitFunction(hfo_exit); }) ? 16u : 0u;
    try {
        l2.addHostFunction(hfo_host);
        ok |= 32u;
    } catch (...) {
    }
    return ok;
}
