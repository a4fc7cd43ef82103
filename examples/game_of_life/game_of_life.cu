// Conway's Game of Life on a wrapped MessageArray2D, written against the FLAME
// GPU 2 API as the reference's example (examples/cpp/game_of_life/src/main.cu:3-31):
// each cell outputs whether it is alive to its index of the array, then counts
// the living cells of its wrapped Moore neighbourhood and applies the rules.
// Registered as "game_of_life"; parameter: the grid's side (default 1000).
#include <cstdint>

#include "flamegpu/flamegpu.h"
#include "flamegpu_gb300/fg_sim.h"

FLAMEGPU_AGENT_FUNCTION(gol_output, flamegpu::MessageNone, flamegpu::MessageArray2D) {
    FLAMEGPU->message_out.setVariable<char>("is_alive", static_cast<char>(FLAMEGPU->getVariable<unsigned int>("is_alive")));
    FLAMEGPU->message_out.setIndex(FLAMEGPU->getVariable<unsigned int, 2>("pos", 0), FLAMEGPU->getVariable<unsigned int, 2>("pos", 1));
    return flamegpu::ALIVE;
}
FLAMEGPU_AGENT_FUNCTION(gol_update, flamegpu::MessageArray2D, flamegpu::MessageNone) {
    const unsigned int my_x = FLAMEGPU->getVariable<unsigned int, 2>("pos", 0);
    const unsigned int my_y = FLAMEGPU->getVariable<unsigned int, 2>("pos", 1);
    unsigned int living = 0;
    for (const auto& message : FLAMEGPU->message_in.wrap(my_x, my_y)) living += message.getVariable<char>("is_alive") ? 1 : 0;
    unsigned int is_alive = FLAMEGPU->getVariable<unsigned int>("is_alive");
    if (is_alive)
        is_alive = (living == 2 || living == 3) ? 1u : 0u;
    else
        is_alive = living == 3 ? 1u : 0u;
    FLAMEGPU->setVariable<unsigned int>("is_alive", is_alive);
    return flamegpu::ALIVE;
}

namespace {

void* make_game_of_life(const double* p, int32_t np) {
    const unsigned int side = np > 0 ? static_cast<unsigned int>(p[0]) : 1000u;
    auto* model = new flamegpu::ModelDescription("Game of Life");
    flamegpu::MessageArray2D::Description message = model->newMessage<flamegpu::MessageArray2D>("is_alive_message");
    message.newVariable<char>("is_alive");
    message.setDimensions(side, side);
    flamegpu::AgentDescription agent = model->newAgent("cell");
    agent.newVariable<unsigned int, 2>("pos");
    agent.newVariable<unsigned int>("is_alive");
    agent.newFunction("output", gol_output).setMessageOutput("is_alive_message");
    agent.newFunction("update", gol_update).setMessageInput("is_alive_message");
    model->newLayer().addAgentFunction(gol_output);
    model->newLayer().addAgentFunction(gol_update);
    return model;
}

struct Register {
    Register() { fgs_register_model("game_of_life", &make_game_of_life); }
} reg;

}  // namespace
