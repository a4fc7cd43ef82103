// Boids on MessageSpatial3D, written against the FLAME GPU 2 API.
//
// The model follows the reference's example (examples/cpp/boids_spatial3D/src/main.cu:134-309,
// clamped bounds and wall steering) and its wrapped variant
// (examples/python_native/boids_spatial3D_wrapped/boids_spatial3D.py:95-255, wrapped
// iterator with virtual positions and wrapped bounds; wing animation omitted).
// Registered as "boids_spatial3d"; parameters (all optional, in order):
//   min_pos, max_pos, interaction_radius, separation_radius, time_scale,
//   global_scale, steer_scale, collision_scale, match_scale, wrap (0/1), sort_period
#include <cmath>

// Benchmark model: built with seatbelts off, as the reference builds its
// benchmarks (FLAMEGPU_SEATBELTS=OFF, src/CMakeLists.txt:78). The test models
// keep the device checks on.
#ifndef FLAMEGPU_SEATBELTS
#define FLAMEGPU_SEATBELTS 0
#endif
#include "flamegpu/flamegpu.h"
#include "flamegpu_gb300/fg_sim.h"

namespace {

FLAMEGPU_HOST_DEVICE_FUNCTION float vec3Length(const float x, const float y, const float z) {
    return sqrtf(x * x + y * y + z * z);
}
FLAMEGPU_HOST_DEVICE_FUNCTION void vec3Mult(float& x, float& y, float& z, const float m) {
    x *= m;
    y *= m;
    z *= m;
}
FLAMEGPU_HOST_DEVICE_FUNCTION void vec3Div(float& x, float& y, float& z, const float d) {
    x /= d;
    y /= d;
    z /= d;
}

}  // namespace

FLAMEGPU_AGENT_FUNCTION(outputdata, flamegpu::MessageNone, flamegpu::MessageSpatial3D) {
    FLAMEGPU->message_out.setVariable<flamegpu::id_t>("id", FLAMEGPU->getID());
    FLAMEGPU->message_out.setVariable<float>("x", FLAMEGPU->getVariable<float>("x"));
    FLAMEGPU->message_out.setVariable<float>("y", FLAMEGPU->getVariable<float>("y"));
    FLAMEGPU->message_out.setVariable<float>("z", FLAMEGPU->getVariable<float>("z"));
    FLAMEGPU->message_out.setVariable<float>("fx", FLAMEGPU->getVariable<float>("fx"));
    FLAMEGPU->message_out.setVariable<float>("fy", FLAMEGPU->getVariable<float>("fy"));
    FLAMEGPU->message_out.setVariable<float>("fz", FLAMEGPU->getVariable<float>("fz"));
    return flamegpu::ALIVE;
}

// Shared body of inputdata; WRAP selects the wrapped iterator and bounds.
template <bool WRAP, typename API>
__device__ __forceinline__ flamegpu::AGENT_STATUS boids_inputdata(API* FLAMEGPU) {
    const flamegpu::id_t id = FLAMEGPU->getID();
    float agent_x = FLAMEGPU->template getVariable<float>("x");
    float agent_y = FLAMEGPU->template getVariable<float>("y");
    float agent_z = FLAMEGPU->template getVariable<float>("z");
    float agent_fx = FLAMEGPU->template getVariable<float>("fx");
    float agent_fy = FLAMEGPU->template getVariable<float>("fy");
    float agent_fz = FLAMEGPU->template getVariable<float>("fz");
    float perceived_centre_x = 0.0f, perceived_centre_y = 0.0f, perceived_centre_z = 0.0f;
    int perceived_count = 0;
    float global_velocity_x = 0.0f, global_velocity_y = 0.0f, global_velocity_z = 0.0f;
    float velocity_change_x = 0.f, velocity_change_y = 0.f, velocity_change_z = 0.f;
    const float INTERACTION_RADIUS = FLAMEGPU->environment.template getProperty<float>("INTERACTION_RADIUS");
    const float SEPARATION_RADIUS = FLAMEGPU->environment.template getProperty<float>("SEPARATION_RADIUS");
    const float collisionScale = FLAMEGPU->environment.template getProperty<float>("COLLISION_SCALE");
    auto visit = [&](const auto& message, float message_x, float message_y, float message_z) {
        const float separation = vec3Length(agent_x - message_x, agent_y - message_y, agent_z - message_z);
        if (separation < INTERACTION_RADIUS) {
            perceived_centre_x += message_x;
            perceived_centre_y += message_y;
            perceived_centre_z += message_z;
            perceived_count++;
            const float message_fx = message.template getVariable<float>("fx");
            const float message_fy = message.template getVariable<float>("fy");
            const float message_fz = message.template getVariable<float>("fz");
            global_velocity_x += message_fx;
            global_velocity_y += message_fy;
            global_velocity_z += message_fz;
            if (separation < (SEPARATION_RADIUS)) {
                const float normalizedSeparation = (separation / SEPARATION_RADIUS);
                const float invNormSep = (1.0f - normalizedSeparation);
                const float invSqSep = invNormSep * invNormSep;
                velocity_change_x += collisionScale * (agent_x - message_x) * invSqSep;
                velocity_change_y += collisionScale * (agent_y - message_y) * invSqSep;
                velocity_change_z += collisionScale * (agent_z - message_z) * invSqSep;
            }
        }
    };
    if constexpr (WRAP) {
        for (const auto& message : FLAMEGPU->message_in.wrap(agent_x, agent_y, agent_z)) {
            if (message.template getVariable<flamegpu::id_t>("id") != id) {
                visit(message, message.getVirtualX(), message.getVirtualY(), message.getVirtualZ());
            }
        }
    } else {
        for (const auto& message : FLAMEGPU->message_in(agent_x, agent_y, agent_z)) {
            if (message.template getVariable<flamegpu::id_t>("id") != id) {
                visit(message, message.template getVariable<float>("x"), message.template getVariable<float>("y"),
                      message.template getVariable<float>("z"));
            }
        }
    }
    if (perceived_count) {
        vec3Div(perceived_centre_x, perceived_centre_y, perceived_centre_z, perceived_count);
        vec3Div(global_velocity_x, global_velocity_y, global_velocity_z, perceived_count);
        const float STEER_SCALE = FLAMEGPU->environment.template getProperty<float>("STEER_SCALE");
        const float steer_velocity_x = (perceived_centre_x - agent_x) * STEER_SCALE;
        const float steer_velocity_y = (perceived_centre_y - agent_y) * STEER_SCALE;
        const float steer_velocity_z = (perceived_centre_z - agent_z) * STEER_SCALE;
        velocity_change_x += steer_velocity_x;
        velocity_change_y += steer_velocity_y;
        velocity_change_z += steer_velocity_z;
        const float MATCH_SCALE = FLAMEGPU->environment.template getProperty<float>("MATCH_SCALE");
        const float match_velocity_x = global_velocity_x * MATCH_SCALE;
        const float match_velocity_y = global_velocity_y * MATCH_SCALE;
        const float match_velocity_z = global_velocity_z * MATCH_SCALE;
        velocity_change_x += match_velocity_x - agent_fx;
        velocity_change_y += match_velocity_y - agent_fy;
        velocity_change_z += match_velocity_z - agent_fz;
    }
    vec3Mult(velocity_change_x, velocity_change_y, velocity_change_z,
             FLAMEGPU->environment.template getProperty<float>("GLOBAL_SCALE"));
    agent_fx += velocity_change_x;
    agent_fy += velocity_change_y;
    agent_fz += velocity_change_z;
    const float agent_fscale = vec3Length(agent_fx, agent_fy, agent_fz);
    if (agent_fscale > 1) vec3Div(agent_fx, agent_fy, agent_fz, agent_fscale);
    const float minSpeed = 0.5f;
    if (agent_fscale < minSpeed) {
        vec3Div(agent_fx, agent_fy, agent_fz, agent_fscale);
        vec3Mult(agent_fx, agent_fy, agent_fz, minSpeed);
    }
    const float minPosition = FLAMEGPU->environment.template getProperty<float>("MIN_POSITION");
    const float maxPosition = FLAMEGPU->environment.template getProperty<float>("MAX_POSITION");
    if constexpr (!WRAP) {
        const float wallInteractionDistance = 0.10f;
        const float wallSteerStrength = 0.05f;
        if (agent_x - minPosition < wallInteractionDistance) agent_fx += wallSteerStrength;
        if (agent_y - minPosition < wallInteractionDistance) agent_fy += wallSteerStrength;
        if (agent_z - minPosition < wallInteractionDistance) agent_fz += wallSteerStrength;
        if (maxPosition - agent_x < wallInteractionDistance) agent_fx -= wallSteerStrength;
        if (maxPosition - agent_y < wallInteractionDistance) agent_fy -= wallSteerStrength;
        if (maxPosition - agent_z < wallInteractionDistance) agent_fz -= wallSteerStrength;
    }
    const float TIME_SCALE = FLAMEGPU->environment.template getProperty<float>("TIME_SCALE");
    agent_x += agent_fx * TIME_SCALE;
    agent_y += agent_fy * TIME_SCALE;
    agent_z += agent_fz * TIME_SCALE;
    if constexpr (WRAP) {
        const float width = maxPosition - minPosition;
        if (agent_x < minPosition) agent_x += width;
        if (agent_y < minPosition) agent_y += width;
        if (agent_z < minPosition) agent_z += width;
        if (agent_x > maxPosition) agent_x -= width;
        if (agent_y > maxPosition) agent_y -= width;
        if (agent_z > maxPosition) agent_z -= width;
    } else {
        agent_x = (agent_x < minPosition) ? minPosition : agent_x;
        agent_x = (agent_x > maxPosition) ? maxPosition : agent_x;
        agent_y = (agent_y < minPosition) ? minPosition : agent_y;
        agent_y = (agent_y > maxPosition) ? maxPosition : agent_y;
        agent_z = (agent_z < minPosition) ? minPosition : agent_z;
        agent_z = (agent_z > maxPosition) ? maxPosition : agent_z;
    }
    FLAMEGPU->template setVariable<float>("x", agent_x);
    FLAMEGPU->template setVariable<float>("y", agent_y);
    FLAMEGPU->template setVariable<float>("z", agent_z);
    FLAMEGPU->template setVariable<float>("fx", agent_fx);
    FLAMEGPU->template setVariable<float>("fy", agent_fy);
    FLAMEGPU->template setVariable<float>("fz", agent_fz);
    return flamegpu::ALIVE;
}

FLAMEGPU_AGENT_FUNCTION(inputdata, flamegpu::MessageSpatial3D, flamegpu::MessageNone) {
    return boids_inputdata<false>(FLAMEGPU);
}
FLAMEGPU_AGENT_FUNCTION(inputdata_wrapped, flamegpu::MessageSpatial3D, flamegpu::MessageNone) {
    return boids_inputdata<true>(FLAMEGPU);
}

namespace {

void* make_boids(const double* p, int32_t np) {
    auto P = [&](int i, double d) { return i < np ? p[i] : d; };
    const float min_pos = static_cast<float>(P(0, -0.5)), max_pos = static_cast<float>(P(1, 0.5));
    const float radius = static_cast<float>(P(2, 0.05));
    const bool wrap = P(9, 0.0) != 0.0;
    auto* model = new flamegpu::ModelDescription("Boids Spatial3D");
    {
        flamegpu::EnvironmentDescription env = model->Environment();
        env.newProperty("MIN_POSITION", min_pos);
        env.newProperty("MAX_POSITION", max_pos);
        env.newProperty("INTERACTION_RADIUS", radius);
        env.newProperty("SEPARATION_RADIUS", static_cast<float>(P(3, 0.01)));
        env.newProperty("TIME_SCALE", static_cast<float>(P(4, 0.0005)));
        env.newProperty("GLOBAL_SCALE", static_cast<float>(P(5, 0.15)));
        env.newProperty("STEER_SCALE", static_cast<float>(P(6, 0.055)));
        env.newProperty("COLLISION_SCALE", static_cast<float>(P(7, 10.0)));
        env.newProperty("MATCH_SCALE", static_cast<float>(P(8, 0.015)));
    }
    {
        flamegpu::MessageSpatial3D::Description message = model->newMessage<flamegpu::MessageSpatial3D>("location");
        message.setRadius(radius);
        message.setMin(min_pos, min_pos, min_pos);
        message.setMax(max_pos, max_pos, max_pos);
        message.newVariable<flamegpu::id_t>("id");
        message.newVariable<float>("fx");
        message.newVariable<float>("fy");
        message.newVariable<float>("fz");
    }
    flamegpu::AgentDescription agent = model->newAgent("Boid");
    agent.newVariable<float>("x");
    agent.newVariable<float>("y");
    agent.newVariable<float>("z");
    agent.newVariable<float>("fx");
    agent.newVariable<float>("fy");
    agent.newVariable<float>("fz");
    agent.setSortPeriod(static_cast<unsigned int>(P(10, 1.0)));
    flamegpu::AgentFunctionDescription out = agent.newFunction("outputdata", outputdata);
    out.setMessageOutput("location");
    flamegpu::AgentFunctionDescription in = wrap ? agent.newFunction("inputdata", inputdata_wrapped)
                                                 : agent.newFunction("inputdata", inputdata);
    in.setMessageInput("location");
    in.dependsOn(out);
    model->addExecutionRoot(out);
    model->generateLayers();
    return model;
}

struct Register {
    Register() { fgs_register_model("boids_spatial3d", &make_boids); }
} reg;

}  // namespace
