#ifndef INCLUDE_FLAMEGPU_SIMULATION_SIMULATIONSERVER_H_
#define INCLUDE_FLAMEGPU_SIMULATION_SIMULATIONSERVER_H_
// A request loop over CUDASimulation (GB300 extension; FLAME GPU 2 has no
// server): simulation runs of any registered model arrive as requests, are
// admitted while a slot and the device-memory budget allow, keep their agent
// and message state resident in HBM, and advance together — every poll issues
// the next step of every admitted run on that run's own stream, so their
// kernels overlap on the device, and runs that arrive meanwhile join at the
// next poll (continuous batching). Each run keeps a bounded number of steps
// queued on the device (about work_in_flight agent-steps, at least
// steps_in_flight), so a long run cannot bury a short one under its backlog
// while a small run still advances many steps per poll; runs with the least
// remaining work are issued first, and their streams get a higher priority. A finished run is read back and its memory
// returned without waiting for the others; a run that fails is completed with
// its error and the others carry on.
#include <chrono>
#include <cstdint>
#include <deque>
#include <map>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "flamegpu/model/ModelDescription.h"
#include "flamegpu/simulation/AgentVector.h"

namespace flamegpu {

class CUDASimulation;

class SimulationServer {
 public:
    struct Config {
        size_t memory_budget = 150ull << 30;  // bytes of device memory runs may reserve
        unsigned int max_active = 64;         // runs on the device at once
        unsigned int steps_per_poll = 1;      // steps issued per run per poll
        unsigned int steps_in_flight = 2;     // steps of one run queued on the device at once (at least)
        // ... and up to work_in_flight / (the run's initial agents) steps, at most 64:
        // small runs keep enough steps queued to advance between two polls
        double work_in_flight = 4.0e6;
        // agent-steps queued on the device over all runs: steps are issued in
        // order of least remaining work until this is reached, so the smallest
        // runs go first and the largest wait for what is left (shortest
        // remaining work first, approximately); a step larger than the budget
        // is issued only when nothing else is queued
        double total_work_in_flight = 6.0e6;
        int device = 0;
        bool use_graphs = true;
    };
    struct Result {
        uint64_t id = 0;
        double arrival_s = 0, admitted_s = 0, completed_s = 0;  // seconds since the server started
        unsigned int steps = 0;
        unsigned long long agent_steps = 0;  // agents summed over the steps run (CUDASimulation::getAgentStepCount)
        bool failed = false;
        std::string error;
        size_t reserved_bytes = 0;
        std::map<std::pair<std::string, std::string>, std::shared_ptr<AgentVector>> populations;
    };

    SimulationServer();
    explicit SimulationServer(const Config& cfg);
    ~SimulationServer();
    SimulationServer(const SimulationServer&) = delete;
    SimulationServer& operator=(const SimulationServer&) = delete;

    /** Queues a run of `model` from the given initial populations (agent name,
     *  population in the agent's initial state); returns its id. */
    uint64_t submit(std::shared_ptr<ModelDescription> model,
                    std::vector<std::pair<std::string, AgentVector>> populations, unsigned int steps, uint64_t seed);
    /** One scheduling round: retire finished runs, admit queued ones, issue
     *  the next steps of the active ones. Returns runs still queued or active. */
    size_t poll();
    /** Polls until every submitted run has completed. */
    void runUntilIdle();
    /** Completed runs since the last call (their populations included). */
    std::vector<Result> takeCompleted();
    size_t queued() const;
    size_t active() const;
    size_t reservedBytes() const;
    /** Scheduling counters: polls, host seconds spent inside poll(), steps issued. */
    struct Counters {
        uint64_t polls = 0;
        double poll_seconds = 0.0;
        uint64_t steps_issued = 0;
    };
    Counters counters() const;
    /** Changes the in-flight limits of Config (values <= 0 keep the current one). */
    void setScheduling(double work_in_flight, double total_work_in_flight);
    double now() const;
    /** Device bytes a run is budgeted at: agent columns (twice, with head room
     *  for births), message columns and records, spatial indexes, scratch. */
    static size_t estimateBytes(const ModelDescription& model,
                                const std::vector<std::pair<std::string, AgentVector>>& populations);

 private:
    struct Job;
    void retire(Job& j, bool failed, const std::string& error);
    int priority_for(double work) const;
    Config cfg;
    std::chrono::steady_clock::time_point t0;
    uint64_t next_id = 1;
    std::deque<std::unique_ptr<Job>> queue;
    std::vector<std::unique_ptr<Job>> admitting;  // set-up in progress on their own threads
    std::vector<std::unique_ptr<Job>> running;
    std::vector<Result> completed;
    size_t reserved = 0;
    Counters stats_;
};

}  // namespace flamegpu

#endif  // INCLUDE_FLAMEGPU_SIMULATION_SIMULATIONSERVER_H_
