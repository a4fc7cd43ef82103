/*
 * fg_sim.h — C ABI over the C++ simulation runtime (libflamegpu2_gb300.so).
 *
 * Lets a non-C++ caller drive CUDASimulation / CUDAEnsemble-style runs of a
 * registered model: the role pyflamegpu's SWIG layer plays for the reference
 * (swig/python/flamegpu.i wraps ModelDescription, CUDASimulation::{setPopulationData,
 * getPopulationData, step, simulate} and CUDAEnsemble::simulate). Models are
 * C++ translation units that register a factory under a name
 * (fgs_register_model); the bundled ones live in libfg_models.so.
 *
 * Every function returns 0 on success or -1 with a message in fgs_last_error().
 */
#ifndef FLAMEGPU_GB300_FG_SIM_H_
#define FLAMEGPU_GB300_FG_SIM_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fgs_sim fgs_sim;

/* A model factory: builds a flamegpu::ModelDescription (returned as void*,
 * owned by the caller of the factory) from numeric parameters. */
typedef void* (*fgs_model_factory)(const double* params, int32_t nparams);

int fgs_register_model(const char* name, fgs_model_factory factory);
/* Comma-separated names of the registered models. */
int fgs_list_models(char* buf, size_t len);
const char* fgs_last_error(void);

/* new CUDASimulation(model) (include/flamegpu/simulation/CUDASimulation.h:177). */
fgs_sim* fgs_create(const char* model, const double* params, int32_t nparams, int32_t device);
void fgs_destroy(fgs_sim* sim);
/* SimulationConfig().steps / random_seed and the GB300 switches. */
int fgs_configure(fgs_sim* sim, uint32_t steps, uint64_t seed, int32_t use_graphs, int32_t check_each_step);
/* setPopulationData: n agents; the named host columns (struct of arrays, each
 * n * sizeof(variable) bytes) are copied, other variables take their defaults.
 * "_id" may be given; unset (0) ids are assigned. */
int fgs_set_population(fgs_sim* sim, const char* agent, const char* state, uint32_t n, int32_t nvars,
                       const char* const* names, const void* const* host_cols);
/* Same, from device columns (no host copy of the data). */
int fgs_set_population_device(fgs_sim* sim, const char* agent, const char* state, uint32_t n, int32_t nvars,
                              const char* const* names, const void* const* device_cols);
/* Replace a population from device columns without a host copy: every
 * variable (including "_id") must be given; next_id is the agent type's next id. */
int fgs_reset_population_device(fgs_sim* sim, const char* agent, const char* state, uint32_t n, int32_t nvars,
                                const char* const* names, const void* const* device_cols, uint32_t next_id);
int fgs_get_count(fgs_sim* sim, const char* agent, const char* state, uint32_t* n);
/* getPopulationData for one variable: copies count * sizeof(variable) bytes. */
int fgs_get_variable(fgs_sim* sim, const char* agent, const char* state, const char* var, void* out, size_t bytes);
/* getPopulationData for several variables at once: out[k] receives *n *
 * sizeof(variable k) bytes (caller buffers of at least cap agents). */
int fgs_get_population(fgs_sim* sim, const char* agent, const char* state, int32_t nvars, const char* const* names,
                       void* const* out, uint32_t cap, uint32_t* n);
/* Copy one variable's current device column into a device buffer (no host hop). */
int fgs_get_variable_device(fgs_sim* sim, const char* agent, const char* state, const char* var, void* dst,
                            size_t bytes);
int fgs_step(fgs_sim* sim, uint32_t steps);
int fgs_simulate(fgs_sim* sim);
/* Agents summed over the steps run so far (each step counted with the
 * populations that entered it; CUDASimulation::getAgentStepCount). Waits for
 * the steps issued. */
int fgs_agent_steps(fgs_sim* sim, uint64_t* agent_steps);
/* Waits for the simulation stream and reports recorded device errors. */
int fgs_synchronize(fgs_sim* sim);
int fgs_set_environment(fgs_sim* sim, const char* name, const void* value, size_t bytes);
int fgs_get_environment(fgs_sim* sim, const char* name, void* value, size_t bytes);
int fgs_stream(fgs_sim* sim, void** stream);
int fgs_stats(fgs_sim* sim, uint64_t* graph_launches, uint32_t* kernels_per_step, uint32_t* step_counter);
/* Shared memory per block used to stage spatial neighbour windows
 * (CUDASimulation::Config::message_stage_bytes; 0 disables staging). */
int fgs_set_stage_bytes(fgs_sim* sim, uint32_t bytes);
/* Enable/disable per-operation CUDA-event timing (steps then run eagerly, not as graphs). */
int fgs_profile_ops(fgs_sim* sim, int32_t enable);
/* Per-operation totals since the last call as "label,total_ms,count;..." (see
 * CUDASimulation::takeOperationProfile). */
int fgs_take_profile(fgs_sim* sim, char* buf, size_t len);
/* Enable/disable timing events captured into the step graphs around every
 * operation (CUDASimulation::Config::time_ops_in_graphs; rebuilds the graphs). */
int fgs_time_ops_in_graphs(fgs_sim* sim, int32_t enable);
/* Adds the operation times of the last replay of each graph replayed since the
 * previous call to the profile read by fgs_take_profile (waits for the stream). */
/* One operation's launches timed by CUDA events inside the step graphs while
 * steps stay replayed several per graph (CUDAConfig::time_op_label; NULL or ""
 * turns it off); read with fgs_harvest_profile / fgs_take_profile. */
int fgs_time_op_in_graphs(fgs_sim* sim, const char* label);
int fgs_harvest_profile(fgs_sim* sim);
/* CUDASimulation::exportData / loadState: JSON state files in the reference's
 * layout (config, stats.step_count, environment, agents -> state -> rows). */
int fgs_export(fgs_sim* sim, const char* path);
int fgs_load_state(fgs_sim* sim, const char* path);
/* SimulationConfig() / CUDAConfig() items by name as text (input_file,
 * step_log_file, exit_log_file, common_log_file, truncate_log_files,
 * random_seed, steps, verbosity, timing, device_id, inLayerConcurrency): the
 * settings a state file records. */
int fgs_set_config(fgs_sim* sim, const char* key, const char* value);
int fgs_get_config(fgs_sim* sim, const char* key, char* out, size_t len);
/* Step (exit == 0) or exit (exit != 0) log configuration
 * (CUDASimulation::setStepLog / setExitLog). spec lists entries separated by
 * ';': "count:agent:state", "mean|sd|min|max|sum:agent:state:variable" (the
 * variable's own type), "env:property". frequency applies to the step log. */
int fgs_set_log(fgs_sim* sim, int32_t exit, const char* spec, uint32_t frequency);
/* The run log as JSON (CUDASimulation::runLogJSON); *needed receives its size + 1. */
int fgs_run_log(fgs_sim* sim, char* buf, size_t len, size_t* needed);
/* getElapsedTimeSteps (seconds) for up to cap steps; returns the count in *n. */
int fgs_step_times(fgs_sim* sim, double* out, uint32_t cap, uint32_t* n);

/* ------------------------------------------------------------ ensembles
 * CUDAEnsemble::simulate(RunPlanVector) (include/flamegpu/simulation/CUDAEnsemble.h:129)
 * of a registered model; runs are added one by one. */
typedef struct fge_ensemble fge_ensemble;
fge_ensemble* fge_create(const char* model, const double* params, int32_t nparams, int32_t device);
void fge_destroy(fge_ensemble* e);
/* EnsembleConfig: batched (one batched simulation when the model allows it), graphs, staging bytes. */
int fge_configure(fge_ensemble* e, int32_t batched, int32_t use_graphs, uint32_t stage_bytes);
/* Adds a RunPlan: steps, seed, initial population of `agent` (named host columns,
 * n rows) and, if message != NULL, that spatial message's bounds and radius for the run. */
int fge_add_run(fge_ensemble* e, uint32_t steps, uint64_t seed, const char* agent, uint32_t n, int32_t nvars,
                const char* const* names, const void* const* host_cols, const char* message, const float* min,
                const float* max, float radius);
int fge_set_run_property(fge_ensemble* e, uint32_t run, const char* name, const void* value, size_t bytes);
/* Runs every plan; *failures receives the number of failed runs. */
int fge_simulate(fge_ensemble* e, uint32_t* failures);
int fge_get_count(fge_ensemble* e, uint32_t run, const char* agent, uint32_t* n);
int fge_get_variable(fge_ensemble* e, uint32_t run, const char* agent, const char* var, void* out, size_t bytes);
int fge_stats(fge_ensemble* e, double* elapsed_s, int32_t* batched, uint32_t* kernels_per_step,
              uint64_t* graph_launches);
/* Device seconds of the last simulate()'s steps (CUDAEnsemble::getEnsembleStepTime). */
int fge_step_time(fge_ensemble* e, double* seconds);
/* Launch-shape tuning of batched steps (CUDAEnsemble::EnsembleConfig::tuning):
 * 0 fixed defaults, 1 read cache_path, 2 measure and write cache_path. */
int fge_set_tuning(fge_ensemble* e, int32_t mode, const char* cache_path);
/* The shape the last simulate() used, as JSON (CUDAEnsemble::getTuning). */
int fge_tuning(fge_ensemble* e, char* json, size_t len);

/* --------------------------------------------------------------- server
 * flamegpu::SimulationServer (include/flamegpu/simulation/SimulationServer.h;
 * no counterpart in the reference): runs of registered models are submitted as
 * requests and advance together, each on its own stream, admitted against a
 * device-memory budget and a slot limit. */
typedef struct fgv_server fgv_server;
fgv_server* fgv_create(int32_t device, uint64_t memory_budget, uint32_t max_active, uint32_t steps_per_poll,
                       int32_t use_graphs);
void fgv_destroy(fgv_server* v);
/* Queues a run of model `model` (factory parameters `params`) for `steps` steps
 * with seed `seed`. Its initial populations: `npops` agents; population k is
 * agents[k] with counts[k] rows and nvars[k] named host columns, taken in order
 * from the flattened `names` / `host_cols` arrays. *id receives the run's id. */
int fgv_submit(fgv_server* v, const char* model, const double* params, int32_t nparams, uint32_t steps, uint64_t seed,
               int32_t npops, const char* const* agents, const uint32_t* counts, const int32_t* nvars,
               const char* const* names, const void* const* host_cols, uint64_t* id);
/* One scheduling round; *remaining receives the runs still queued or active. */
int fgv_poll(fgv_server* v, uint32_t* remaining);
int fgv_run_until_idle(fgv_server* v);
/* Ids of runs completed since the last call (at most cap; *n receives the count). */
int fgv_take_completed(fgv_server* v, uint64_t* ids, uint32_t cap, uint32_t* n);
/* Times (seconds since the server started: arrival, admitted, completed) and
 * status of a completed run; the error text goes to err (len bytes) if failed. */
int fgv_result_info(fgv_server* v, uint64_t id, double* times3, int32_t* failed, char* err, size_t len);
/* Agents summed over the steps a completed run ran (CUDASimulation::getAgentStepCount). */
int fgv_result_agent_steps(fgv_server* v, uint64_t id, uint64_t* agent_steps);
int fgv_result_count(fgv_server* v, uint64_t id, const char* agent, const char* state, uint32_t* n);
int fgv_result_variable(fgv_server* v, uint64_t id, const char* agent, const char* state, const char* var, void* out,
                        size_t bytes);
/* Drops a completed run's results. */
int fgv_release(fgv_server* v, uint64_t id);
int fgv_stats(fgv_server* v, uint32_t* queued, uint32_t* active, uint64_t* reserved_bytes);
/* In-flight limits (SimulationServer::Config::work_in_flight, total_work_in_flight;
 * values <= 0 keep the current one). */
int fgv_set_scheduling(fgv_server* v, double work_in_flight, double total_work_in_flight);
/* Scheduling counters: polls, host seconds inside poll, steps issued. */
int fgv_counters(fgv_server* v, uint64_t* polls, double* poll_seconds, uint64_t* steps_issued);

#ifdef __cplusplus
}
#endif

#endif /* FLAMEGPU_GB300_FG_SIM_H_ */
