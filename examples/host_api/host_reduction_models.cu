// Host reductions that run on the device, written against the FLAME GPU 2 API:
// the operations of the reference's host-reduction tests
// (tests/test_cases/runtime/agent/host_reduction/test_count.cu,
// test_histogram_even.cu, test_reduce.cu, test_transform_reduce.cu) over
// every scalar type.
//
// Registered model:
//   host_reductions  agent "agent" with one variable of each type: f (float),
//                    d (double), i8, u8, i16, u16, i32, u32, i64, u64. A step
//                    function computes, per variable, count(v, 0),
//                    histogramEven<T, unsigned int>(v, 10, 0, 20),
//                    histogramEven<T, int> of the same, reduce<T>(v, max, 0),
//                    reduce<T>(v, sum, 7) and transformReduce<T, int32_t>(v,
//                    "<= 0 ? 1 : 0", sum, 0), into slots that
//                    fg_test_host_reductions() copies out (16 8-byte slots
//                    per variable, values stored bit for bit).
#include <cstdint>
#include <cstring>
#include <mutex>
#include <vector>

#include "flamegpu/flamegpu.h"
#include "flamegpu_gb300/fg_sim.h"

namespace {

FLAMEGPU_CUSTOM_REDUCTION(hr_max, a, b) { return a > b ? a : b; }
FLAMEGPU_CUSTOM_REDUCTION(hr_sum, a, b) { return a + b; }
FLAMEGPU_CUSTOM_TRANSFORM(hr_non_positive, a) { return a <= 0 ? 1 : 0; }

constexpr int kSlots = 16;
constexpr int kVars = 10;
std::mutex g_mu;
uint64_t g_slots[kVars * kSlots];

template <typename T>
uint64_t bits(T v) {
    uint64_t o = 0;
    std::memcpy(&o, &v, sizeof(T));
    return o;
}

template <typename T>
void reduce_one(flamegpu::HostAPI* api, const char* var, int k) {
    auto a = api->agent("agent");
    uint64_t* s = g_slots + k * kSlots;
    s[0] = a.count<T>(var, static_cast<T>(0));
    s[1] = bits<T>(a.reduce<T>(var, hr_max, static_cast<T>(0)));
    s[2] = bits<T>(a.reduce<T>(var, hr_sum, static_cast<T>(7)));
    s[3] = bits<int32_t>(a.transformReduce<T, int32_t>(var, hr_non_positive, hr_sum, 0));
    const std::vector<unsigned int> h = a.histogramEven<T>(var, 10, static_cast<T>(0), static_cast<T>(20));
    const std::vector<int> hi = a.histogramEven<T, int>(var, 10, static_cast<T>(0), static_cast<T>(20));
    for (int b = 0; b < 10; ++b) s[4 + b] = h[b];
    // the two histograms agree (counts as unsigned int and as int)
    bool same = h.size() == hi.size();
    for (size_t b = 0; same && b < h.size(); ++b) same = static_cast<int>(h[b]) == hi[b];
    s[14] = same ? 1u : 0u;
}

FLAMEGPU_AGENT_FUNCTION(hr_nothing, flamegpu::MessageNone, flamegpu::MessageNone) { return flamegpu::ALIVE; }

FLAMEGPU_STEP_FUNCTION(hr_step) {
    std::lock_guard<std::mutex> lock(g_mu);
    reduce_one<float>(FLAMEGPU, "f", 0);
    reduce_one<double>(FLAMEGPU, "d", 1);
    reduce_one<int8_t>(FLAMEGPU, "i8", 2);
    reduce_one<uint8_t>(FLAMEGPU, "u8", 3);
    reduce_one<int16_t>(FLAMEGPU, "i16", 4);
    reduce_one<uint16_t>(FLAMEGPU, "u16", 5);
    reduce_one<int32_t>(FLAMEGPU, "i32", 6);
    reduce_one<uint32_t>(FLAMEGPU, "u32", 7);
    reduce_one<int64_t>(FLAMEGPU, "i64", 8);
    reduce_one<uint64_t>(FLAMEGPU, "u64", 9);
}

void* make_host_reductions(const double*, int32_t) {
    auto* m = new flamegpu::ModelDescription("host_reductions");
    flamegpu::AgentDescription a = m->newAgent("agent");
    a.newVariable<float>("f");
    a.newVariable<double>("d");
    a.newVariable<int8_t>("i8");
    a.newVariable<uint8_t>("u8");
    a.newVariable<int16_t>("i16");
    a.newVariable<uint16_t>("u16");
    a.newVariable<int32_t>("i32");
    a.newVariable<uint32_t>("u32");
    a.newVariable<int64_t>("i64");
    a.newVariable<uint64_t>("u64");
    m->newLayer().addAgentFunction(a.newFunction("nothing", hr_nothing));
    m->addStepFunction(hr_step);
    return m;
}

struct Register {
    Register() { fgs_register_model("host_reductions", &make_host_reductions); }
} reg;

}  // namespace

extern "C" void fg_test_host_reductions(uint64_t* out) {
    std::lock_guard<std::mutex> lock(g_mu);
    std::memcpy(out, g_slots, sizeof(g_slots));
}
