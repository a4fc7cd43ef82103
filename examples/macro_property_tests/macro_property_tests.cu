// Environment macro property test models, written against the FLAME GPU 2
// API: the models of the reference's tests
// tests/test_cases/runtime/environment/test_device_macro_property.cu and
// test_host_macro_property.cu.
//
// Registered model "macro_properties", parameter [variant]; agent "agent"
// (a, b, c, i, j, k, w: unsigned int; cd: double; id: int; x_i64, x_u64,
// x_i32, x_u32, x_f64, x_f32 of those types):
//   0 add      init: int, double exchange(1); write: += a; read: b = int, cd = double
//   1 add2     init: int exchange(1); write: b = int + a; check: c = int
//   2 add3     init: int exchange(1); write: b = int.addAtomic(a); check: c = int
//   3 sub      init: int exchange(25); write: -= a; read: b = int
//   4 sub2     init: int exchange(25); write: b = int - a; check: c = int
//   5 sub3     init: int exchange(25); write: b = int.subAtomic(a); check: c = int
//   6 post++   init: int exchange(1); write: b = int++; read: c = int
//   7 pre++    as 6 with b = ++int
//   8 post--   as 6 with b = int--
//   9 pre--    as 6 with b = --int
//  10 min      init: int exchange(25); write: b = int.min(a); read: c = int
//  11 max      as 10 with max
//  12 cas      init: int exchange(25); write: b = int.CAS(a, 100); read: c = int
//  13 exchange every 4- and 8-byte type: init exchange(15); read into x_<type>
//  14 host ReadTest: agents exchange a into int[i][j][k][w] (2 x 3 x 4 x 5);
//     a host layer checks every element against its row-major position
//  15 host WriteTest: a host layer writes 1 + position; agents set a = 12
//     where 2 + int[i][j][k][w] == a + 1 (a = 2 + position), else 0
//  16 host ZeroTest: as 15, then a host layer calls zero(); agents set a = 1
//     where the element is 0, else 0
//  17 host ArithmeticTest: host layers set int, uint, int8, uint8, int64,
//     uint64, id, float, double to 10, then check the reference's arithmetic
//  18 contention: every agent adds 1 to count, id to total (double), and
//     takes min and max of id; a second layer reads them into a, cd, b, c
//  19 index past the first dimension of int[2][3][4][5] (a device error)
//  20 WriteRead: += then a read of int in one agent function (a device error)
//  21 ReadWrite: a read then += of int in one agent function (a device error)
//   fg_test_macro_errors() returns the host layers' failed checks.
#include <cstdint>
#include <mutex>

#include "flamegpu/flamegpu.h"
#include "flamegpu_gb300/fg_sim.h"

namespace {
std::mutex g_mu;
unsigned int g_errors = 0;
void fail_if(bool bad) {
    if (bad) ++g_errors;
}
}  // namespace

using flamegpu::MessageNone;

#define MP(T, ...) FLAMEGPU->environment.getMacroProperty<T, ##__VA_ARGS__>
#define UINT_MP MP(unsigned int)("int")

FLAMEGPU_AGENT_FUNCTION(mp_init1, MessageNone, MessageNone) {
    UINT_MP.exchange(1);
    MP(double)("double").exchange(1);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(mp_init25, MessageNone, MessageNone) {
    UINT_MP.exchange(25);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(mp_add, MessageNone, MessageNone) {
    UINT_MP += FLAMEGPU->getVariable<unsigned int>("a");
    MP(double)("double") += static_cast<double>(FLAMEGPU->getVariable<unsigned int>("a"));
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(mp_read_add, MessageNone, MessageNone) {
    FLAMEGPU->setVariable<unsigned int>("b", UINT_MP);
    FLAMEGPU->setVariable<double>("cd", MP(double)("double"));
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(mp_add2, MessageNone, MessageNone) {
    FLAMEGPU->setVariable<unsigned int>("b", UINT_MP + FLAMEGPU->getVariable<unsigned int>("a"));
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(mp_add3, MessageNone, MessageNone) {
    FLAMEGPU->setVariable<unsigned int>("b", UINT_MP.addAtomic(FLAMEGPU->getVariable<unsigned int>("a")));
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(mp_sub, MessageNone, MessageNone) {
    UINT_MP -= FLAMEGPU->getVariable<unsigned int>("a");
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(mp_sub2, MessageNone, MessageNone) {
    FLAMEGPU->setVariable<unsigned int>("b", UINT_MP - FLAMEGPU->getVariable<unsigned int>("a"));
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(mp_sub3, MessageNone, MessageNone) {
    FLAMEGPU->setVariable<unsigned int>("b", UINT_MP.subAtomic(FLAMEGPU->getVariable<unsigned int>("a")));
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(mp_read_b, MessageNone, MessageNone) {
    FLAMEGPU->setVariable<unsigned int>("b", UINT_MP);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(mp_read_c, MessageNone, MessageNone) {
    FLAMEGPU->setVariable<unsigned int>("c", UINT_MP);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(mp_postinc, MessageNone, MessageNone) {
    FLAMEGPU->setVariable<unsigned int>("b", UINT_MP++);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(mp_preinc, MessageNone, MessageNone) {
    FLAMEGPU->setVariable<unsigned int>("b", ++UINT_MP);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(mp_postdec, MessageNone, MessageNone) {
    FLAMEGPU->setVariable<unsigned int>("b", UINT_MP--);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(mp_predec, MessageNone, MessageNone) {
    FLAMEGPU->setVariable<unsigned int>("b", --UINT_MP);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(mp_min, MessageNone, MessageNone) {
    FLAMEGPU->setVariable<unsigned int>("b", UINT_MP.min(FLAMEGPU->getVariable<unsigned int>("a")));
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(mp_max, MessageNone, MessageNone) {
    FLAMEGPU->setVariable<unsigned int>("b", UINT_MP.max(FLAMEGPU->getVariable<unsigned int>("a")));
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(mp_cas, MessageNone, MessageNone) {
    FLAMEGPU->setVariable<unsigned int>("b", UINT_MP.CAS(FLAMEGPU->getVariable<unsigned int>("a"), 100));
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(mp_exchange_init, MessageNone, MessageNone) {
    MP(int64_t)("i64").exchange(15);
    MP(uint64_t)("u64").exchange(15u);
    MP(int32_t)("i32").exchange(15);
    MP(uint32_t)("u32").exchange(15u);
    MP(double)("f64").exchange(15);
    MP(float)("f32").exchange(15);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(mp_exchange_read, MessageNone, MessageNone) {
    FLAMEGPU->setVariable<int64_t>("x_i64", MP(int64_t)("i64"));
    FLAMEGPU->setVariable<uint64_t>("x_u64", MP(uint64_t)("u64"));
    FLAMEGPU->setVariable<int32_t>("x_i32", MP(int32_t)("i32"));
    FLAMEGPU->setVariable<uint32_t>("x_u32", MP(uint32_t)("u32"));
    FLAMEGPU->setVariable<double>("x_f64", MP(double)("f64"));
    FLAMEGPU->setVariable<float>("x_f32", MP(float)("f32"));
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(mp_agent_write4, MessageNone, MessageNone) {
    auto t = FLAMEGPU->environment.getMacroProperty<unsigned int, 2, 3, 4, 5>("int4");
    t[FLAMEGPU->getVariable<unsigned int>("i")][FLAMEGPU->getVariable<unsigned int>("j")]
     [FLAMEGPU->getVariable<unsigned int>("k")][FLAMEGPU->getVariable<unsigned int>("w")]
         .exchange(FLAMEGPU->getVariable<unsigned int>("a"));
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(mp_agent_read4, MessageNone, MessageNone) {
    auto t = FLAMEGPU->environment.getMacroProperty<unsigned int, 2, 3, 4, 5>("int4");
    const unsigned int v = t[FLAMEGPU->getVariable<unsigned int>("i")][FLAMEGPU->getVariable<unsigned int>("j")]
                            [FLAMEGPU->getVariable<unsigned int>("k")][FLAMEGPU->getVariable<unsigned int>("w")];
    FLAMEGPU->setVariable<unsigned int>("a", 2 + v == FLAMEGPU->getVariable<unsigned int>("a") + 1 ? 12u : 0u);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(mp_agent_read_zero4, MessageNone, MessageNone) {
    auto t = FLAMEGPU->environment.getMacroProperty<unsigned int, 2, 3, 4, 5>("int4");
    const unsigned int v = t[FLAMEGPU->getVariable<unsigned int>("i")][FLAMEGPU->getVariable<unsigned int>("j")]
                            [FLAMEGPU->getVariable<unsigned int>("k")][FLAMEGPU->getVariable<unsigned int>("w")];
    FLAMEGPU->setVariable<unsigned int>("a", v == 0 ? 1u : 0u);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(mp_contend, MessageNone, MessageNone) {
    const int id = FLAMEGPU->getVariable<int>("id");
    MP(unsigned int)("count") += 1u;
    MP(double)("total") += static_cast<double>(id);
    MP(int)("lo").min(id);
    MP(int)("hi").max(id);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(mp_contend_read, MessageNone, MessageNone) {
    FLAMEGPU->setVariable<unsigned int>("a", MP(unsigned int)("count"));
    FLAMEGPU->setVariable<double>("cd", MP(double)("total"));
    FLAMEGPU->setVariable<unsigned int>("b", static_cast<unsigned int>(static_cast<int>(MP(int)("lo"))));
    FLAMEGPU->setVariable<unsigned int>("c", static_cast<unsigned int>(static_cast<int>(MP(int)("hi"))));
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(mp_write_read, MessageNone, MessageNone) {
    UINT_MP += FLAMEGPU->getVariable<unsigned int>("a");
    FLAMEGPU->setVariable<unsigned int>("b", UINT_MP);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(mp_read_write, MessageNone, MessageNone) {
    const unsigned int t = UINT_MP;
    UINT_MP += FLAMEGPU->getVariable<unsigned int>("a");
    FLAMEGPU->setVariable<unsigned int>("b", t);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(mp_bad_index, MessageNone, MessageNone) {
    auto t = FLAMEGPU->environment.getMacroProperty<unsigned int, 2, 3, 4, 5>("int4");
    t[2][0][0][0].exchange(1u);
    return flamegpu::ALIVE;
}

FLAMEGPU_HOST_FUNCTION(mp_host_read) {
    std::lock_guard<std::mutex> lock(g_mu);
    auto t = FLAMEGPU->environment.getMacroProperty<unsigned int, 2, 3, 4, 5>("int4");
    unsigned int a = 0;
    for (unsigned int i = 0; i < 2; ++i)
        for (unsigned int j = 0; j < 3; ++j)
            for (unsigned int k = 0; k < 4; ++k)
                for (unsigned int w = 0; w < 5; ++w) fail_if(t[i][j][k][w] != a++);
}
FLAMEGPU_HOST_FUNCTION(mp_host_write) {
    auto t = FLAMEGPU->environment.getMacroProperty<unsigned int, 2, 3, 4, 5>("int4");
    unsigned int a = 0;
    for (unsigned int i = 0; i < 2; ++i)
        for (unsigned int j = 0; j < 3; ++j)
            for (unsigned int k = 0; k < 4; ++k)
                for (unsigned int w = 0; w < 5; ++w) t[i][j][k][w] = 1 + a++;
}
FLAMEGPU_HOST_FUNCTION(mp_host_zero) {
    auto t = FLAMEGPU->environment.getMacroProperty<unsigned int, 2, 3, 4, 5>("int4");
    t.zero();
}
FLAMEGPU_HOST_FUNCTION(mp_host_arith_init) {
    FLAMEGPU->environment.getMacroProperty<int>("a_int") = 10;
    FLAMEGPU->environment.getMacroProperty<unsigned int>("a_uint") = 10u;
    FLAMEGPU->environment.getMacroProperty<int8_t>("a_int8") = 10;
    FLAMEGPU->environment.getMacroProperty<uint8_t>("a_uint8") = 10u;
    FLAMEGPU->environment.getMacroProperty<int64_t>("a_int64") = 10;
    FLAMEGPU->environment.getMacroProperty<uint64_t>("a_uint64") = 10u;
    FLAMEGPU->environment.getMacroProperty<flamegpu::id_t>("a_id") = 10u;
    FLAMEGPU->environment.getMacroProperty<float>("a_float") = 10.0f;
    FLAMEGPU->environment.getMacroProperty<double>("a_double") = 10.0;
}
// The arithmetic checks of test_host_macro_property.cu:228-463 for one type.
template <typename T, bool INTEGRAL>
void arith(flamegpu::HostAPI* api, const char* name) {
    auto t = api->environment.getMacroProperty<T>(name);
    fail_if(t++ != static_cast<T>(10));
    fail_if(++t != static_cast<T>(12));
    fail_if(t-- != static_cast<T>(12));
    fail_if(--t != static_cast<T>(10));
    fail_if(t / 5 != static_cast<T>(10) / 5);
    fail_if(t / 3 != static_cast<T>(10) / 3);
    fail_if(t + 5 != static_cast<T>(10) + 5);
    fail_if(t - 3 != static_cast<T>(10) - 3);
    fail_if(t * 5 != static_cast<T>(10) * 5);
    if constexpr (INTEGRAL) {
        fail_if(t / 3.0 != static_cast<T>(10) / 3.0);
        fail_if(t + 3.0 != static_cast<T>(10) + 3.0);
        fail_if(t - 3.0 != static_cast<T>(10) - 3.0);
        fail_if(t * 3.0 != static_cast<T>(10) * 3.0);
        fail_if(t % 5 != static_cast<T>(10) % 5);
        fail_if(t % 3 != static_cast<T>(10) % 3);
    }
    fail_if(t != static_cast<T>(10));
    t += 10;
    fail_if(t != static_cast<T>(20));
    t -= 10;
    fail_if(t != static_cast<T>(10));
    t *= 2;
    fail_if(t != static_cast<T>(20));
    t /= 2;
    fail_if(t != static_cast<T>(10));
}
FLAMEGPU_HOST_FUNCTION(mp_host_arith) {
    std::lock_guard<std::mutex> lock(g_mu);
    arith<int, true>(FLAMEGPU, "a_int");
    arith<unsigned int, true>(FLAMEGPU, "a_uint");
    arith<int8_t, true>(FLAMEGPU, "a_int8");
    arith<uint8_t, true>(FLAMEGPU, "a_uint8");
    arith<int64_t, true>(FLAMEGPU, "a_int64");
    arith<uint64_t, true>(FLAMEGPU, "a_uint64");
    arith<flamegpu::id_t, true>(FLAMEGPU, "a_id");
    arith<float, false>(FLAMEGPU, "a_float");
    arith<double, false>(FLAMEGPU, "a_double");
}

namespace {

void layer(flamegpu::ModelDescription* m, flamegpu::AgentFunctionDescription f) { m->newLayer().addAgentFunction(f); }

void* make_macro_properties(const double* p, int32_t np) {
    const int variant = np > 0 ? static_cast<int>(p[0]) : 0;
    auto* m = new flamegpu::ModelDescription("device_env_test");
    flamegpu::EnvironmentDescription env = m->Environment();
    env.newMacroProperty<unsigned int>("int");
    env.newMacroProperty<double>("double");
    env.newMacroProperty<unsigned int, 2, 3, 4, 5>("int4");
    flamegpu::AgentDescription a = m->newAgent("agent");
    for (const char* v : {"a", "b", "c", "i", "j", "k", "w"}) a.newVariable<unsigned int>(v, 0u);
    a.newVariable<double>("cd", 0.0);
    a.newVariable<int>("id", 0);
    a.newVariable<int64_t>("x_i64", 0);
    a.newVariable<uint64_t>("x_u64", 0);
    a.newVariable<int32_t>("x_i32", 0);
    a.newVariable<uint32_t>("x_u32", 0);
    a.newVariable<double>("x_f64", 0);
    a.newVariable<float>("x_f32", 0);
    switch (variant) {
        case 0: layer(m, a.newFunction("init", mp_init1)); layer(m, a.newFunction("write", mp_add));
                layer(m, a.newFunction("read", mp_read_add)); break;
        case 1: layer(m, a.newFunction("init", mp_init1)); layer(m, a.newFunction("write", mp_add2));
                layer(m, a.newFunction("check", mp_read_c)); break;
        case 2: layer(m, a.newFunction("init", mp_init1)); layer(m, a.newFunction("write", mp_add3));
                layer(m, a.newFunction("check", mp_read_c)); break;
        case 3: layer(m, a.newFunction("init", mp_init25)); layer(m, a.newFunction("write", mp_sub));
                layer(m, a.newFunction("read", mp_read_b)); break;
        case 4: layer(m, a.newFunction("init", mp_init25)); layer(m, a.newFunction("write", mp_sub2));
                layer(m, a.newFunction("check", mp_read_c)); break;
        case 5: layer(m, a.newFunction("init", mp_init25)); layer(m, a.newFunction("write", mp_sub3));
                layer(m, a.newFunction("check", mp_read_c)); break;
        case 6: layer(m, a.newFunction("init", mp_init1)); layer(m, a.newFunction("write", mp_postinc));
                layer(m, a.newFunction("read", mp_read_c)); break;
        case 7: layer(m, a.newFunction("init", mp_init1)); layer(m, a.newFunction("write", mp_preinc));
                layer(m, a.newFunction("read", mp_read_c)); break;
        case 8: layer(m, a.newFunction("init", mp_init1)); layer(m, a.newFunction("write", mp_postdec));
                layer(m, a.newFunction("read", mp_read_c)); break;
        case 9: layer(m, a.newFunction("init", mp_init1)); layer(m, a.newFunction("write", mp_predec));
                layer(m, a.newFunction("read", mp_read_c)); break;
        case 10: layer(m, a.newFunction("init", mp_init25)); layer(m, a.newFunction("write", mp_min));
                 layer(m, a.newFunction("read", mp_read_c)); break;
        case 11: layer(m, a.newFunction("init", mp_init25)); layer(m, a.newFunction("write", mp_max));
                 layer(m, a.newFunction("read", mp_read_c)); break;
        case 12: layer(m, a.newFunction("init", mp_init25)); layer(m, a.newFunction("write", mp_cas));
                 layer(m, a.newFunction("read", mp_read_c)); break;
        case 13:
            env.newMacroProperty<int64_t>("i64");
            env.newMacroProperty<uint64_t>("u64");
            env.newMacroProperty<int32_t>("i32");
            env.newMacroProperty<uint32_t>("u32");
            env.newMacroProperty<double>("f64");
            env.newMacroProperty<float>("f32");
            layer(m, a.newFunction("init", mp_exchange_init));
            layer(m, a.newFunction("read", mp_exchange_read));
            break;
        case 14: layer(m, a.newFunction("agentwrite", mp_agent_write4)); m->newLayer().addHostFunction(mp_host_read); break;
        case 15: m->newLayer().addHostFunction(mp_host_write); layer(m, a.newFunction("agentread", mp_agent_read4)); break;
        case 16:
            m->newLayer().addHostFunction(mp_host_write);
            m->newLayer().addHostFunction(mp_host_zero);
            layer(m, a.newFunction("agentread", mp_agent_read_zero4));
            break;
        case 17:
            env.newMacroProperty<int>("a_int");
            env.newMacroProperty<unsigned int>("a_uint");
            env.newMacroProperty<int8_t>("a_int8");
            env.newMacroProperty<uint8_t>("a_uint8");
            env.newMacroProperty<int64_t>("a_int64");
            env.newMacroProperty<uint64_t>("a_uint64");
            env.newMacroProperty<flamegpu::id_t>("a_id");
            env.newMacroProperty<float>("a_float");
            env.newMacroProperty<double>("a_double");
            m->newLayer().addHostFunction(mp_host_arith_init);
            m->newLayer().addHostFunction(mp_host_arith);
            break;
        case 18:
            env.newMacroProperty<unsigned int>("count");
            env.newMacroProperty<double>("total");
            env.newMacroProperty<int>("lo");
            env.newMacroProperty<int>("hi");
            layer(m, a.newFunction("contend", mp_contend));
            layer(m, a.newFunction("read", mp_contend_read));
            break;
        case 20: layer(m, a.newFunction("write_read", mp_write_read)); break;
        case 21: layer(m, a.newFunction("read_write", mp_read_write)); break;
        default: layer(m, a.newFunction("bad", mp_bad_index)); break;
    }
    return m;
}

struct Register {
    Register() { fgs_register_model("macro_properties", &make_macro_properties); }
} reg;

}  // namespace

extern "C" unsigned int fg_test_macro_errors(int reset) {
    std::lock_guard<std::mutex> lock(g_mu);
    const unsigned int e = g_errors;
    if (reset) g_errors = 0;
    return e;
}
