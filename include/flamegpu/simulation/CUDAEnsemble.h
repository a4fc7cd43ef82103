#ifndef INCLUDE_FLAMEGPU_SIMULATION_CUDAENSEMBLE_H_
#define INCLUDE_FLAMEGPU_SIMULATION_CUDAENSEMBLE_H_
// RunPlan / RunPlanVector / CUDAEnsemble with the reference's names
// (include/flamegpu/simulation/RunPlan.h, RunPlanVector.h:43-49,
// CUDAEnsemble.h:28-129).
//
// The reference runs an ensemble as `concurrent_runs` host threads, each
// building a fresh CUDASimulation per plan (src/flamegpu/simulation/detail/
// AbstractSimRunner.cu:82-117). Here, when the model allows it (one agent type
// in one state, no agent birth/death, spatial or no message input), every plan
// of the ensemble becomes one instance of a single batched simulation: the
// instances are concatenated into segments of the agent and message buffers,
// each with its own spatial grid, PBM slice, environment, seed and step count,
// and one captured graph per step sorts, builds and iterates all of them with
// segmented kernels. Other models fall back to running the plans one after
// another through CUDASimulation.
#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <typeindex>
#include <vector>

#include "flamegpu/model/ModelDescription.h"
#include "flamegpu/simulation/AgentVector.h"

namespace flamegpu {

class RunPlan {
 public:
    explicit RunPlan(const ModelDescription& model);
    void setRandomSimulationSeed(uint64_t seed) { seed_ = seed; }
    void setSteps(unsigned int steps) { steps_ = steps; }
    template <typename T>
    void setProperty(const std::string& name, T value) {
        set_property(name, std::type_index(typeid(T)), sizeof(T), &value);
    }
    uint64_t getRandomSimulationSeed() const { return seed_; }
    unsigned int getSteps() const { return steps_; }

    // ---- GB300 extensions ----
    /** Initial population of an agent (state) for this run. */
    void setPopulation(const AgentVector& population, const std::string& state = "default");
    /** The same, taking the vector's storage instead of copying it. */
    void setPopulation(AgentVector&& population, const std::string& state = "default");
    /** Per-run bounds and radius of a spatial message list (the model's are the default). */
    void setSpatialMessageBounds(const std::string& message, const std::vector<float>& min,
                                 const std::vector<float>& max, float radius);

    // read by the ensemble
    struct SpatialOverride {
        std::vector<float> min, max;
        float radius = 0.0f;
    };
    const std::shared_ptr<detail::ModelData>& model() const { return model_; }
    const std::map<std::string, std::vector<char>>& properties() const { return properties_; }
    const std::map<std::pair<std::string, std::string>, std::shared_ptr<AgentVector>>& populations() const {
        return populations_;
    }
    const std::map<std::string, SpatialOverride>& spatial() const { return spatial_; }

 private:
    void set_property(const std::string& name, std::type_index t, size_t size, const void* v);
    std::shared_ptr<detail::ModelData> model_;
    uint64_t seed_ = 0;
    unsigned int steps_ = 1;
    std::map<std::string, std::vector<char>> properties_;
    std::map<std::pair<std::string, std::string>, std::shared_ptr<AgentVector>> populations_;
    std::map<std::string, SpatialOverride> spatial_;
};

class RunPlanVector : public std::vector<RunPlan> {
 public:
    RunPlanVector(const ModelDescription& model, unsigned int initial_length);
    void setSteps(unsigned int steps);
    /** Seeds initial_seed, initial_seed + step, ... (RunPlanVector.h:49). */
    void setRandomSimulationSeed(uint64_t initial_seed, unsigned int step = 1);
    template <typename T>
    void setProperty(const std::string& name, T value) {
        for (auto& p : *this) p.setProperty<T>(name, value);
    }
};

namespace detail {
struct EnsembleImpl;
}

class CUDAEnsemble {
 public:
    /** CUDAEnsemble::EnsembleConfig (CUDAEnsemble.h:28-101) plus the GB300 switches. */
    struct EnsembleConfig {
        unsigned int concurrent_runs = 4;
        int device = 0;
        bool batched = true;            // one batched simulation when the model allows it
        bool use_graphs = true;
        unsigned int message_stage_bytes = 96u * 1024u;
        bool timing = false;
        // Launch shapes of the batched step (threads per agent block, blocks
        // per SM, staging bytes, the scans' wide-tile threshold): 0 the fixed
        // defaults; 1 the entry of tuning_cache for this GPU, model and size
        // class (defaults if it has none); 2 measured now, every candidate
        // timed by CUDA events on the batch's own step graph, the fastest
        // kept and written to tuning_cache. The reference picks one block size
        // per launch by occupancy (CUDASimulation.cu:988). GB300 extension.
        int tuning = 0;
        std::string tuning_cache;
    };
    explicit CUDAEnsemble(const ModelDescription& model, int argc = 0, const char** argv = nullptr);
    ~CUDAEnsemble();
    EnsembleConfig& Config();
    /** Runs every plan; returns the number of failed runs (CUDAEnsemble::simulate). */
    unsigned int simulate(const RunPlanVector& plans);
    /** Seconds of the last simulate() (getEnsembleElapsedTime). */
    double getEnsembleElapsedTime() const;
    /** Device seconds of the last simulate()'s steps, by CUDA events: from the
     *  first step to the last of the batched simulation, or summed over the
     *  runs on the sequential path (GB300 extension). */
    double getEnsembleStepTime() const;
    /** True if the last simulate() ran as one batched simulation. */
    bool lastRunBatched() const;
    /** The launch shape the last batched simulate() used and where it came
     *  from, as JSON ({"tuned", "source", "key", "shape", ...}). */
    const std::string& getTuning() const;
    /** Final population of one run (GB300 extension; the reference reports through logs). */
    void getPopulationData(unsigned int run, AgentVector& population, const std::string& state = "default") const;
    /** The same population without a copy (valid until the next simulate()). */
    std::shared_ptr<const AgentVector> getPopulationView(unsigned int run, const std::string& agent,
                                                          const std::string& state = "default") const;
    /** Kernel launches per batched step and graph replays of the last simulate(). */
    unsigned int getKernelsPerStep() const;
    unsigned long long getGraphLaunches() const;

 private:
    std::unique_ptr<detail::EnsembleImpl> impl;
};

}  // namespace flamegpu

#endif  // INCLUDE_FLAMEGPU_SIMULATION_CUDAENSEMBLE_H_
