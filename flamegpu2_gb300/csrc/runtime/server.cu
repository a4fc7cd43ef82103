// SimulationServer: continuous batching of simulation runs over CUDASimulation.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <future>
#include <thread>

#include "flamegpu/simulation/CUDASimulation.h"
#include "flamegpu/simulation/SimulationServer.h"

namespace flamegpu {

struct SimulationServer::Job {
    uint64_t id = 0;
    std::shared_ptr<ModelDescription> model;
    std::vector<std::pair<std::string, AgentVector>> populations;
    unsigned int steps = 0;
    uint64_t seed = 0;
    double arrival = 0, admitted = 0;
    unsigned int issued = 0;     // steps enqueued on the run's stream
    unsigned int completed = 0;  // steps known to have finished on the device
    size_t agents = 0;           // initial agents, all types
    size_t bytes = 0;
    std::unique_ptr<CUDASimulation> sim;
    std::vector<cudaEvent_t> ring;  // event of step k in ring[k % size]
    std::future<void> setup;        // admission work running on its own thread
    bool births = false;            // the model has agent output (birth)
    ~Job() {
        for (cudaEvent_t e : ring) cudaEventDestroy(e);
    }
    // advance `completed` over the steps whose events have fired
    void reap() {
        while (completed < issued && cudaEventQuery(ring[completed % ring.size()]) == cudaSuccess) ++completed;
    }
    double remaining_work() const { return static_cast<double>(steps - completed) * static_cast<double>(agents); }
};

SimulationServer::SimulationServer() : SimulationServer(Config()) {}

SimulationServer::SimulationServer(const Config& c) : cfg(c), t0(std::chrono::steady_clock::now()) {}

SimulationServer::~SimulationServer() {
    // let admissions and in-flight work finish before the simulations free their buffers
    for (auto& j : admitting)
        if (j->setup.valid()) j->setup.wait();
    for (auto* list : {&admitting, &running})
        for (auto& j : *list)
            if (j->sim) cudaStreamSynchronize(j->sim->getStream());
}

double SimulationServer::now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

size_t SimulationServer::queued() const { return queue.size(); }
size_t SimulationServer::active() const { return running.size() + admitting.size(); }
size_t SimulationServer::reservedBytes() const { return reserved; }

size_t SimulationServer::estimateBytes(const ModelDescription& model,
                                       const std::vector<std::pair<std::string, AgentVector>>& pops) {
    const auto& m = *model.getData();
    size_t total = 32ull << 20, max_pop = 1024;
    for (const auto& a : m.agents) {
        size_t n = 1024;
        for (const auto& p : pops)
            if (p.first == a->name) n = std::max<size_t>(n, p.second.size());
        bool births = false;
        for (const auto& f : a->functions) births = births || !f->agent_output.empty();
        size_t row = 0;
        for (const auto& v : a->variables) row += v.bytes();
        // ping-pong columns, sort/compaction scratch; births may grow the list fourfold
        total += n * (2 * row + 24) * (births ? 4 : 1);
        max_pop = std::max(max_pop, n * (births ? 4 : 1));
    }
    for (const auto& msg : m.messages) {
        size_t row = 0;
        for (const auto& v : msg->variables) row += (v.bytes() + 3) & ~size_t(3);
        total += max_pop * (2 * row + 32);  // columns, sorted records, build scratch
        if (msg->kind == detail::MessageKind::Bucket) {
            total += max_pop * (row + 24) +
                     (static_cast<size_t>(static_cast<int64_t>(msg->bucket_upper) - msg->bucket_lower) + 2) * 8;
        } else if (detail::array_dims(msg->kind)) {
            total += static_cast<size_t>(msg->dims[0]) * std::max(1u, msg->dims[1]) * std::max(1u, msg->dims[2]) *
                     (row + 4);  // the array and its claim words
        } else if (msg->kind != detail::MessageKind::BruteForce) {
            double bins = 1.0;
            const int dims = msg->kind == detail::MessageKind::Spatial3D ? 3 : 2;
            for (int d = 0; d < dims; ++d) bins *= std::ceil((msg->max[d] - msg->min[d]) / msg->radius);
            total += static_cast<size_t>(bins) * 16;  // histogram, PBM, scan
        }
    }
    return total;
}

uint64_t SimulationServer::submit(std::shared_ptr<ModelDescription> model,
                                  std::vector<std::pair<std::string, AgentVector>> pops, unsigned int steps,
                                  uint64_t seed) {
    auto j = std::make_unique<Job>();
    j->id = next_id++;
    j->model = std::move(model);
    j->populations = std::move(pops);
    j->steps = steps;
    j->seed = seed;
    j->arrival = now();
    j->bytes = estimateBytes(*j->model, j->populations);
    for (const auto& p : j->populations) j->agents += p.second.size();
    for (const auto& a : j->model->getData()->agents)
        for (const auto& f : a->functions) j->births = j->births || !f->agent_output.empty();
    const uint64_t id = j->id;
    queue.push_back(std::move(j));
    return id;
}

void SimulationServer::retire(Job& j, bool failed, const std::string& error) {
    Result r;
    r.id = j.id;
    r.arrival_s = j.arrival;
    r.admitted_s = j.admitted;
    r.steps = j.steps;
    r.reserved_bytes = j.bytes;
    r.failed = failed;
    r.error = error;
    if (!failed && j.sim) {
        try {
            r.agent_steps = j.sim->getAgentStepCount();
            for (const auto& a : j.model->getData()->agents)
                for (const auto& st : a->states) {
                    auto pop = std::make_shared<AgentVector>(AgentDescription(j.model->getData(), a.get()));
                    j.sim->getPopulationData(*pop, st);
                    r.populations[{a->name, st}] = pop;
                }
        } catch (const exception::FLAMEGPUException& e) {
            r.failed = true;
            r.error = std::string(e.exception_type()) + ": " + e.what();
        }
    }
    r.completed_s = now();
    j.sim.reset();
    reserved -= j.bytes;
    completed.push_back(std::move(r));
}

SimulationServer::Counters SimulationServer::counters() const { return stats_; }

void SimulationServer::setScheduling(double work_in_flight, double total_work_in_flight) {
    if (work_in_flight > 0.0) cfg.work_in_flight = work_in_flight;
    if (total_work_in_flight > 0.0) cfg.total_work_in_flight = total_work_in_flight;
}

size_t SimulationServer::poll() {
    const auto t_poll = std::chrono::steady_clock::now();
    ++stats_.polls;
    // 1. retire runs whose last step has completed (non-blocking test)
    for (size_t k = 0; k < running.size();) {
        Job& j = *running[k];
        j.reap();
        if (j.completed >= j.steps) {
            retire(j, false, "");
            running.erase(running.begin() + static_cast<long>(k));
        } else {
            ++k;
        }
    }
    // 2. runs whose set-up has finished join the active ones
    for (size_t k = 0; k < admitting.size();) {
        Job& j = *admitting[k];
        if (j.setup.wait_for(std::chrono::seconds(0)) != std::future_status::ready) {
            ++k;
            continue;
        }
        try {
            j.setup.get();
            running.push_back(std::move(admitting[k]));
        } catch (const exception::FLAMEGPUException& e) {
            retire(j, true, std::string(e.exception_type()) + ": " + e.what());
        } catch (const std::exception& e) {
            retire(j, true, e.what());
        }
        admitting.erase(admitting.begin() + static_cast<long>(k));
    }
    // 3. admit queued runs in arrival order while a slot and the budget allow;
    //    each builds its simulation and uploads its populations on a thread of
    //    its own, so a large upload does not hold up the steps of the others
    while (!queue.empty() && running.size() + admitting.size() < cfg.max_active &&
           (reserved + queue.front()->bytes <= cfg.memory_budget || (running.empty() && admitting.empty()))) {
        std::unique_ptr<Job> j = std::move(queue.front());
        queue.pop_front();
        j->admitted = now();
        reserved += j->bytes;
        Job* jp = j.get();
        const Config c = cfg;
        const int prio = priority_for(static_cast<double>(j->steps) * static_cast<double>(j->agents));
        jp->setup = std::async(std::launch::async, [jp, c, prio] {
            jp->sim = std::make_unique<CUDASimulation>(*jp->model);
            jp->sim->CUDAConfig().device_id = c.device;
            jp->sim->CUDAConfig().use_graphs = c.use_graphs;
            jp->sim->CUDAConfig().stream_priority = prio;
            jp->sim->SimulationConfig().random_seed = jp->seed;
            jp->sim->SimulationConfig().steps = jp->steps;
            // births may grow a population to four times its start (as budgeted), no further
            size_t largest = 1024;
            for (const auto& p : jp->populations) largest = std::max<size_t>(largest, p.second.size());
            jp->sim->CUDAConfig().max_agents = static_cast<unsigned int>(std::min<size_t>(4 * largest, (1u << 31) - 1));
            for (auto& p : jp->populations) jp->sim->setPopulationData(p.second);
            jp->populations.clear();
            // runs with births need a population count from the device to size
            // the next step's output, so they keep few steps queued
            const double by_work = c.work_in_flight / static_cast<double>(std::max<size_t>(jp->agents, 1));
            const double depth = jp->births ? 1.0 : by_work;
            const unsigned int ring = static_cast<unsigned int>(
                std::min(64.0, std::max(static_cast<double>(std::max(1u, c.steps_in_flight)), depth)));
            jp->ring.assign(ring, nullptr);
            for (cudaEvent_t& e : jp->ring)
                if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
                    throw exception::CUDAError("cudaEventCreate failed");
            if (cudaStreamSynchronize(jp->sim->getStream()) != cudaSuccess)
                throw exception::CUDAError("population upload failed");
        });
        admitting.push_back(std::move(j));
    }
    // 4. issue the next steps, least remaining work first, keeping at most
    //    steps_in_flight steps of a run queued on the device
    std::vector<Job*> order;
    order.reserve(running.size());
    for (auto& j : running) order.push_back(j.get());
    std::stable_sort(order.begin(), order.end(),
                     [](const Job* a, const Job* b) { return a->remaining_work() < b->remaining_work(); });
    std::vector<Job*> failed;
    double inflight = 0.0;
    for (Job* jp : order) {
        jp->reap();
        inflight += static_cast<double>(jp->issued - jp->completed) * static_cast<double>(jp->agents);
    }
    for (Job* jp : order) {
        Job& j = *jp;
        try {
            const double per_step = static_cast<double>(std::max<size_t>(j.agents, 1));
            const unsigned int per_poll = std::max<unsigned int>(cfg.steps_per_poll, static_cast<unsigned int>(j.ring.size()));
            for (unsigned int s = 0; s < per_poll && j.issued < j.steps && j.issued - j.completed < j.ring.size(); ++s) {
                if (inflight > 0.0 && inflight + per_step > cfg.total_work_in_flight) break;
                j.sim->step();
                if (cudaEventRecord(j.ring[j.issued % j.ring.size()], j.sim->getStream()) != cudaSuccess)
                    throw exception::CUDAError("cudaEventRecord failed");
                ++j.issued;
                ++stats_.steps_issued;
                inflight += per_step;
            }
        } catch (const exception::FLAMEGPUException& e) {
            // failure isolation: this run completes with its error, the others go on
            retire(j, true, std::string(e.exception_type()) + ": " + e.what());
            failed.push_back(jp);
        }
    }
    if (!failed.empty())
        running.erase(std::remove_if(running.begin(), running.end(),
                                     [&](const std::unique_ptr<Job>& j) {
                                         return std::find(failed.begin(), failed.end(), j.get()) != failed.end();
                                     }),
                      running.end());
    stats_.poll_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t_poll).count();
    return queue.size() + admitting.size() + running.size();
}

int SimulationServer::priority_for(double work) const {
    // the device's priority range split by decades of work (agent-steps):
    // under 1e7 gets the highest priority, each further decade one level less
    int least = 0, greatest = 0;
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess || least == greatest) return 0;
    const int levels = least - greatest;  // greatest is the numerically lower
    int decade = work < 1e7 ? 0 : static_cast<int>(std::floor(std::log10(work))) - 6;
    return greatest + std::min(std::max(decade, 0), levels);
}

void SimulationServer::runUntilIdle() {
    while (poll()) {
        if (running.empty()) std::this_thread::yield();  // only admissions in progress
    }
}

std::vector<SimulationServer::Result> SimulationServer::takeCompleted() {
    std::vector<Result> out;
    out.swap(completed);
    return out;
}

}  // namespace flamegpu
