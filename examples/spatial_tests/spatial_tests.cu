// Models of the reference's messaging and death tests, written against the
// FLAME GPU 2 API, so that the parity tests run the same agent functions:
//   tests/test_cases/runtime/messaging/test_spatial_3d.cu:16-66 (out_mandatory3D,
//   out_optional3D, in3D), :855-900 (inWrapped3D), :1090-1110 (in_bounds_not_factor);
//   tests/test_cases/runtime/messaging/test_spatial_2d.cu (2D equivalents);
//   tests/test_cases/runtime/messaging/test_brute_force.cu (brute-force count);
//   tests/test_cases/simulation/test_cuda_simulation.cu:31-37 (DeathTestFunc).
// Registered models:
//   "spatial_count"  params: dims, minx, miny, minz, maxx, maxy, maxz, radius, wrap, optional
//   "bruteforce_count" params: optional
//   "agent_death"
#include "flamegpu/flamegpu.h"
#include "flamegpu_gb300/fg_sim.h"

FLAMEGPU_AGENT_FUNCTION(out_mandatory3D, flamegpu::MessageNone, flamegpu::MessageSpatial3D) {
    FLAMEGPU->message_out.setVariable<flamegpu::id_t>("id", FLAMEGPU->getID());
    FLAMEGPU->message_out.setLocation(FLAMEGPU->getVariable<float>("x"), FLAMEGPU->getVariable<float>("y"),
                                      FLAMEGPU->getVariable<float>("z"));
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(out_optional3D, flamegpu::MessageNone, flamegpu::MessageSpatial3D) {
    if (FLAMEGPU->getVariable<int>("do_output")) {
        FLAMEGPU->message_out.setVariable<flamegpu::id_t>("id", FLAMEGPU->getID());
        FLAMEGPU->message_out.setLocation(FLAMEGPU->getVariable<float>("x"), FLAMEGPU->getVariable<float>("y"),
                                          FLAMEGPU->getVariable<float>("z"));
    }
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(in3D, flamegpu::MessageSpatial3D, flamegpu::MessageNone) {
    const float x1 = FLAMEGPU->getVariable<float>("x");
    const float y1 = FLAMEGPU->getVariable<float>("y");
    const float z1 = FLAMEGPU->getVariable<float>("z");
    unsigned int count = 0;
    unsigned int badCount = 0;
    const int myBin[3] = {static_cast<int>(x1), static_cast<int>(y1), static_cast<int>(z1)};
    for (const auto& message : FLAMEGPU->message_in(x1, y1, z1)) {
        const int messageBin[3] = {static_cast<int>(message.getVariable<float>("x")),
                                   static_cast<int>(message.getVariable<float>("y")),
                                   static_cast<int>(message.getVariable<float>("z"))};
        bool isBad = false;
        for (unsigned int i = 0; i < 3; ++i) {
            const int binDiff = myBin[i] - messageBin[i];
            if (binDiff > 1 || binDiff < -1) isBad = true;
        }
        count++;
        badCount = isBad ? badCount + 1 : badCount;
    }
    FLAMEGPU->setVariable<unsigned int>("count", count);
    FLAMEGPU->setVariable<unsigned int>("badCount", badCount);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(inWrapped3D, flamegpu::MessageSpatial3D, flamegpu::MessageNone) {
    const float x1 = FLAMEGPU->getVariable<float>("x");
    const float y1 = FLAMEGPU->getVariable<float>("y");
    const float z1 = FLAMEGPU->getVariable<float>("z");
    const flamegpu::id_t ID = FLAMEGPU->getID();
    unsigned int count = 0;
    unsigned int badCount = 0;
    float xSum = 0, ySum = 0, zSum = 0;
    for (const auto& message : FLAMEGPU->message_in.wrap(x1, y1, z1)) {
        const float x2 = message.getVirtualX(x1);
        const float y2 = message.getVirtualY(y1);
        const float z2 = message.getVirtualZ(z1);
        const float x21 = x2 - x1;
        const float y21 = y2 - y1;
        const float z21 = z2 - z1;
        const float distance = sqrtf(x21 * x21 + y21 * y21 + z21 * z21);
        if (distance > FLAMEGPU->message_in.radius() || (fabsf(x21) != 2.0f && x2 != x1) ||
            (fabsf(y21) != 2.0f && y2 != y1) || (fabsf(z21) != 2.0f && z2 != z1)) {
            badCount++;
        } else {
            count++;
            if (message.getVariable<flamegpu::id_t>("id") != ID) {
                xSum += x21;
                ySum += y21;
                zSum += z21;
            }
        }
    }
    FLAMEGPU->setVariable<unsigned int>("count", count);
    FLAMEGPU->setVariable<unsigned int>("badCount", badCount);
    FLAMEGPU->setVariable<float>("result_x", xSum);
    FLAMEGPU->setVariable<float>("result_y", ySum);
    FLAMEGPU->setVariable<float>("result_z", zSum);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(out_mandatory2D, flamegpu::MessageNone, flamegpu::MessageSpatial2D) {
    FLAMEGPU->message_out.setVariable<flamegpu::id_t>("id", FLAMEGPU->getID());
    FLAMEGPU->message_out.setLocation(FLAMEGPU->getVariable<float>("x"), FLAMEGPU->getVariable<float>("y"));
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(out_optional2D, flamegpu::MessageNone, flamegpu::MessageSpatial2D) {
    if (FLAMEGPU->getVariable<int>("do_output")) {
        FLAMEGPU->message_out.setVariable<flamegpu::id_t>("id", FLAMEGPU->getID());
        FLAMEGPU->message_out.setLocation(FLAMEGPU->getVariable<float>("x"), FLAMEGPU->getVariable<float>("y"));
    }
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(in2D, flamegpu::MessageSpatial2D, flamegpu::MessageNone) {
    const float x1 = FLAMEGPU->getVariable<float>("x");
    const float y1 = FLAMEGPU->getVariable<float>("y");
    unsigned int count = 0;
    unsigned int badCount = 0;
    const int myBin[2] = {static_cast<int>(x1), static_cast<int>(y1)};
    for (const auto& message : FLAMEGPU->message_in(x1, y1)) {
        const int messageBin[2] = {static_cast<int>(message.getVariable<float>("x")),
                                   static_cast<int>(message.getVariable<float>("y"))};
        bool isBad = false;
        for (unsigned int i = 0; i < 2; ++i) {
            const int binDiff = myBin[i] - messageBin[i];
            if (binDiff > 1 || binDiff < -1) isBad = true;
        }
        count++;
        badCount = isBad ? badCount + 1 : badCount;
    }
    FLAMEGPU->setVariable<unsigned int>("count", count);
    FLAMEGPU->setVariable<unsigned int>("badCount", badCount);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(inWrapped2D, flamegpu::MessageSpatial2D, flamegpu::MessageNone) {
    const float x1 = FLAMEGPU->getVariable<float>("x");
    const float y1 = FLAMEGPU->getVariable<float>("y");
    const flamegpu::id_t ID = FLAMEGPU->getID();
    unsigned int count = 0;
    unsigned int badCount = 0;
    float xSum = 0, ySum = 0;
    for (const auto& message : FLAMEGPU->message_in.wrap(x1, y1)) {
        const float x2 = message.getVirtualX(x1);
        const float y2 = message.getVirtualY(y1);
        const float x21 = x2 - x1;
        const float y21 = y2 - y1;
        const float distance = sqrtf(x21 * x21 + y21 * y21);
        if (distance > FLAMEGPU->message_in.radius() || (fabsf(x21) != 2.0f && x2 != x1) ||
            (fabsf(y21) != 2.0f && y2 != y1)) {
            badCount++;
        } else {
            count++;
            if (message.getVariable<flamegpu::id_t>("id") != ID) {
                xSum += x21;
                ySum += y21;
            }
        }
    }
    FLAMEGPU->setVariable<unsigned int>("count", count);
    FLAMEGPU->setVariable<unsigned int>("badCount", badCount);
    FLAMEGPU->setVariable<float>("result_x", xSum);
    FLAMEGPU->setVariable<float>("result_y", ySum);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(out_bruteforce, flamegpu::MessageNone, flamegpu::MessageBruteForce) {
    if (FLAMEGPU->getVariable<int>("do_output")) FLAMEGPU->message_out.setVariable<int>("x", FLAMEGPU->getVariable<int>("x"));
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(in_bruteforce, flamegpu::MessageBruteForce, flamegpu::MessageNone) {
    int sum = 0;
    unsigned int count = 0;
    for (const auto& message : FLAMEGPU->message_in) {
        sum += message.getVariable<int>("x");
        ++count;
    }
    FLAMEGPU->setVariable<int>("sum", sum);
    FLAMEGPU->setVariable<unsigned int>("count", count);
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(DeathTestFunc, flamegpu::MessageNone, flamegpu::MessageNone) {
    const unsigned int x = FLAMEGPU->getVariable<unsigned int>("x");
    if (x % 2 == 0) return flamegpu::DEAD;
    return flamegpu::ALIVE;
}

namespace {

void* make_spatial_count(const double* p, int32_t np) {
    auto P = [&](int i, double d) { return i < np ? p[i] : d; };
    const int dims = static_cast<int>(P(0, 3));
    const float mn[3] = {static_cast<float>(P(1, 0)), static_cast<float>(P(2, 0)), static_cast<float>(P(3, 0))};
    const float mx[3] = {static_cast<float>(P(4, 5)), static_cast<float>(P(5, 5)), static_cast<float>(P(6, 5))};
    const float r = static_cast<float>(P(7, 1));
    const bool wrap = P(8, 0) != 0, optional = P(9, 0) != 0;
    auto* model = new flamegpu::ModelDescription("SpatialCount");
    flamegpu::AgentDescription agent = model->newAgent("agent");
    agent.newVariable<float>("x");
    agent.newVariable<float>("y");
    agent.newVariable<float>("z");
    agent.newVariable<int>("do_output", 1);
    agent.newVariable<unsigned int>("count");
    agent.newVariable<unsigned int>("badCount");
    agent.newVariable<float>("result_x");
    agent.newVariable<float>("result_y");
    agent.newVariable<float>("result_z");
    if (dims == 3) {
        auto m = model->newMessage<flamegpu::MessageSpatial3D>("location");
        m.setMin(mn[0], mn[1], mn[2]);
        m.setMax(mx[0], mx[1], mx[2]);
        m.setRadius(r);
        m.newVariable<flamegpu::id_t>("id");
        auto fo = optional ? agent.newFunction("out", out_optional3D) : agent.newFunction("out", out_mandatory3D);
        fo.setMessageOutput("location");
        fo.setMessageOutputOptional(optional);
        auto fi = wrap ? agent.newFunction("in", inWrapped3D) : agent.newFunction("in", in3D);
        fi.setMessageInput("location");
        model->newLayer().addAgentFunction(fo);
        model->newLayer().addAgentFunction(fi);
    } else {
        auto m = model->newMessage<flamegpu::MessageSpatial2D>("location");
        m.setMin(mn[0], mn[1]);
        m.setMax(mx[0], mx[1]);
        m.setRadius(r);
        m.newVariable<flamegpu::id_t>("id");
        auto fo = optional ? agent.newFunction("out", out_optional2D) : agent.newFunction("out", out_mandatory2D);
        fo.setMessageOutput("location");
        fo.setMessageOutputOptional(optional);
        auto fi = wrap ? agent.newFunction("in", inWrapped2D) : agent.newFunction("in", in2D);
        fi.setMessageInput("location");
        model->newLayer().addAgentFunction(fo);
        model->newLayer().addAgentFunction(fi);
    }
    return model;
}

void* make_bruteforce_count(const double* p, int32_t np) {
    const bool optional = np > 0 && p[0] != 0;
    auto* model = new flamegpu::ModelDescription("BruteForceCount");
    auto m = model->newMessage<flamegpu::MessageBruteForce>("msg");
    m.newVariable<int>("x");
    flamegpu::AgentDescription agent = model->newAgent("agent");
    agent.newVariable<int>("x");
    agent.newVariable<int>("do_output", 1);
    agent.newVariable<int>("sum");
    agent.newVariable<unsigned int>("count");
    auto fo = agent.newFunction("out", out_bruteforce);
    fo.setMessageOutput("msg");
    fo.setMessageOutputOptional(optional);
    auto fi = agent.newFunction("in", in_bruteforce);
    fi.setMessageInput("msg");
    model->newLayer().addAgentFunction(fo);
    model->newLayer().addAgentFunction(fi);
    return model;
}

void* make_agent_death(const double*, int32_t) {
    auto* model = new flamegpu::ModelDescription("AgentDeath");
    flamegpu::AgentDescription a = model->newAgent("agent");
    a.newVariable<unsigned int>("x");
    a.newFunction("DeathFunc", DeathTestFunc).setAllowAgentDeath(true);
    model->newLayer().addAgentFunction(DeathTestFunc);
    return model;
}

struct Register {
    Register() {
        fgs_register_model("spatial_count", &make_spatial_count);
        fgs_register_model("bruteforce_count", &make_bruteforce_count);
        fgs_register_model("agent_death", &make_agent_death);
    }
} reg;

}  // namespace
