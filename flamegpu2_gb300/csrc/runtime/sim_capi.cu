// C ABI over CUDASimulation (include/flamegpu_gb300/fg_sim.h) and the model registry.
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "flamegpu/flamegpu.h"
#include "flamegpu_gb300/fg_sim.h"

namespace {

std::mutex g_reg_mu;
std::map<std::string, fgs_model_factory>& registry() {
    static std::map<std::string, fgs_model_factory> r;
    return r;
}
thread_local std::string g_err;

template <typename F>
int guarded(F&& f) {
    try {
        f();
        return 0;
    } catch (const flamegpu::exception::FLAMEGPUException& e) {
        g_err = std::string(e.exception_type()) + ": " + e.what();
    } catch (const std::exception& e) {
        g_err = e.what();
    } catch (...) {
        g_err = "unknown exception";
    }
    return -1;
}

}  // namespace

struct fgs_sim {
    std::unique_ptr<flamegpu::ModelDescription> model;
    std::unique_ptr<flamegpu::CUDASimulation> sim;
};

namespace {

const flamegpu::detail::EnvProperty* find_env(fgs_sim* s, const char* name) {
    for (const auto& p : s->model->getData()->environment)
        if (p.name == name) return &p;
    throw flamegpu::exception::InvalidEnvProperty(std::string("no environment property ") + name);
}

}  // namespace

extern "C" int fgs_register_model(const char* name, fgs_model_factory f) {
    std::lock_guard<std::mutex> lk(g_reg_mu);
    registry()[name] = f;
    return 0;
}

extern "C" int fgs_list_models(char* buf, size_t len) {
    std::lock_guard<std::mutex> lk(g_reg_mu);
    std::string s;
    for (const auto& kv : registry()) s += (s.empty() ? "" : ",") + kv.first;
    if (len) {
        std::strncpy(buf, s.c_str(), len - 1);
        buf[len - 1] = 0;
    }
    return 0;
}

extern "C" const char* fgs_last_error(void) { return g_err.c_str(); }

extern "C" fgs_sim* fgs_create(const char* model, const double* params, int32_t nparams, int32_t device) {
    fgs_sim* out = nullptr;
    guarded([&] {
        fgs_model_factory f = nullptr;
        {
            std::lock_guard<std::mutex> lk(g_reg_mu);
            auto it = registry().find(model);
            if (it == registry().end()) throw flamegpu::exception::InvalidArgument(std::string("unknown model ") + model);
            f = it->second;
        }
        auto s = std::make_unique<fgs_sim>();
        s->model.reset(static_cast<flamegpu::ModelDescription*>(f(params, nparams)));
        if (device != 0) {
            // the device is chosen before the simulation allocates
            cudaSetDevice(device);
        }
        s->sim = std::make_unique<flamegpu::CUDASimulation>(*s->model);
        out = s.release();
    });
    return out;
}

extern "C" void fgs_destroy(fgs_sim* s) { delete s; }

extern "C" int fgs_configure(fgs_sim* s, uint32_t steps, uint64_t seed, int32_t graphs, int32_t check) {
    return guarded([&] {
        s->sim->SimulationConfig().steps = steps;
        s->sim->SimulationConfig().random_seed = seed;
        s->sim->CUDAConfig().use_graphs = graphs != 0;
        s->sim->CUDAConfig().check_each_step = check != 0;
        s->sim->applyConfig();
    });
}

extern "C" int fgs_set_population(fgs_sim* s, const char* agent, const char* state, uint32_t n, int32_t nvars,
                                  const char* const* names, const void* const* cols) {
    return guarded([&] {
        // every variable given: straight to the device, where the transfer
        // also checks that every id is set; a population with ids to assign
        // goes through AgentVector (the list is left empty by the failed try)
        const auto* ad = s->model->Agent(agent).getData();
        bool all = static_cast<size_t>(nvars) == ad->variables.size();
        std::vector<std::pair<std::string, const void*>> direct;
        for (int32_t k = 0; k < nvars && all; ++k) {
            all = ad->find(names[k]) != nullptr;
            direct.emplace_back(names[k], cols[k]);
        }
        if (all) {
            try {
                s->sim->setPopulationColumns(agent, state ? state : "default", n, direct);
                return;
            } catch (const flamegpu::exception::InvalidArgument& e) {
                if (!std::strstr(e.what(), "every _id must be set")) throw;
            }
        }
        flamegpu::AgentVector pop(s->model->Agent(agent), n);
        for (int32_t k = 0; k < nvars; ++k) {
            const size_t c = pop.columnIndex(names[k]);
            std::memcpy(pop.columns()[c].data(), cols[k], pop.columns()[c].size());
        }
        s->sim->setPopulationData(pop, state);
    });
}

extern "C" int fgs_set_population_device(fgs_sim* s, const char* agent, const char* state, uint32_t n, int32_t nvars,
                                         const char* const* names, const void* const* dcols) {
    return guarded([&] {
        // size the lists and assign ids through the host path (defaults only), then
        // overwrite the given columns device-to-device
        flamegpu::AgentVector pop(s->model->Agent(agent), n);
        s->sim->setPopulationData(pop, state);
        const auto* ad = pop.getAgentData();
        for (int32_t k = 0; k < nvars; ++k) {
            const flamegpu::detail::Variable* v = ad->find(names[k]);
            if (!v) throw flamegpu::exception::InvalidAgentVar(std::string("no variable ") + names[k]);
            void* dst = s->sim->getDeviceVariable(agent, names[k], state);
            if (cudaMemcpyAsync(dst, dcols[k], static_cast<size_t>(v->bytes()) * n, cudaMemcpyDeviceToDevice,
                                s->sim->getStream()) != cudaSuccess)
                throw flamegpu::exception::CUDAError("device population copy failed");
        }
        cudaStreamSynchronize(s->sim->getStream());
    });
}

extern "C" int fgs_reset_population_device(fgs_sim* s, const char* agent, const char* state, uint32_t n, int32_t nvars,
                                           const char* const* names, const void* const* dcols, uint32_t next_id) {
    return guarded([&] {
        std::vector<std::pair<std::string, const void*>> cols;
        for (int32_t k = 0; k < nvars; ++k) cols.emplace_back(names[k], dcols[k]);
        s->sim->setPopulationDevice(agent, state, n, cols, next_id);
    });
}

extern "C" int fgs_get_count(fgs_sim* s, const char* agent, const char* state, uint32_t* n) {
    return guarded([&] { *n = s->sim->getAgentCount(agent, state); });
}

extern "C" int fgs_get_variable(fgs_sim* s, const char* agent, const char* state, const char* var, void* out,
                                size_t bytes) {
    return guarded([&] {
        flamegpu::AgentVector pop(s->model->Agent(agent));
        s->sim->getPopulationData(pop, state);
        const size_t c = pop.columnIndex(var);
        const auto& col = pop.columns()[c];
        if (bytes < col.size()) throw flamegpu::exception::InvalidArgument("output buffer too small");
        std::memcpy(out, col.data(), col.size());
    });
}

extern "C" int fgs_get_population(fgs_sim* s, const char* agent, const char* state, int32_t nvars,
                                  const char* const* names, void* const* out, uint32_t cap, uint32_t* n) {
    return guarded([&] {
        std::vector<std::pair<std::string, void*>> cols;
        for (int32_t k = 0; k < nvars; ++k) cols.emplace_back(names[k], out[k]);
        *n = s->sim->getPopulationColumns(agent, state ? state : "default", cols, cap);
    });
}

extern "C" int fgs_get_variable_device(fgs_sim* s, const char* agent, const char* state, const char* var, void* dst,
                                       size_t bytes) {
    return guarded([&] {
        void* src = s->sim->getDeviceVariable(agent, var, state);
        if (cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, s->sim->getStream()) != cudaSuccess)
            throw flamegpu::exception::CUDAError("device copy failed");
    });
}

extern "C" int fgs_agent_steps(fgs_sim* s, uint64_t* agent_steps) {
    return guarded([&] { *agent_steps = s->sim->getAgentStepCount(); });
}

extern "C" int fgs_step(fgs_sim* s, uint32_t steps) {
    return guarded([&] {
        s->sim->step(static_cast<unsigned int>(steps));
    });
}

extern "C" int fgs_simulate(fgs_sim* s) { return guarded([&] { s->sim->simulate(); }); }

extern "C" int fgs_synchronize(fgs_sim* s) { return guarded([&] { s->sim->synchronize(); }); }

extern "C" int fgs_set_environment(fgs_sim* s, const char* name, const void* value, size_t bytes) {
    return guarded([&] {
        const auto* p = find_env(s, name);
        if (bytes != p->value.size()) throw flamegpu::exception::InvalidEnvPropertyType("size mismatch");
        // the property's bytes, whatever its type (the size was checked)
        flamegpu::HostAPI::Environment e(s->sim->getImpl());
        e.setRaw(name, value, bytes);
    });
}

extern "C" int fgs_get_environment(fgs_sim* s, const char* name, void* value, size_t bytes) {
    return guarded([&] {
        const auto* p = find_env(s, name);
        if (bytes != p->value.size()) throw flamegpu::exception::InvalidEnvPropertyType("size mismatch");
        s->sim->getEnvironmentRaw(name, value, bytes);
    });
}

extern "C" int fgs_stream(fgs_sim* s, void** stream) {
    return guarded([&] { *stream = s->sim->getStream(); });
}

extern "C" int fgs_stats(fgs_sim* s, uint64_t* gl, uint32_t* kps, uint32_t* sc) {
    return guarded([&] {
        if (gl) *gl = s->sim->getGraphLaunches();
        if (kps) *kps = s->sim->getKernelsPerStep();
        if (sc) *sc = s->sim->getStepCounter();
    });
}

extern "C" int fgs_step_times(fgs_sim* s, double* out, uint32_t cap, uint32_t* n) {
    return guarded([&] {
        s->sim->synchronize();
        const auto t = s->sim->getElapsedTimeSteps();
        const uint32_t m = static_cast<uint32_t>(std::min<size_t>(cap, t.size()));
        for (uint32_t i = 0; i < m; ++i) out[i] = t[i];
        *n = m;
    });
}

extern "C" int fgs_profile_ops(fgs_sim* s, int32_t enable) {
    return guarded([&] { s->sim->CUDAConfig().profile_ops = enable != 0; });
}

extern "C" int fgs_time_ops_in_graphs(fgs_sim* s, int32_t enable) {
    return guarded([&] {
        s->sim->CUDAConfig().time_ops_in_graphs = enable != 0;
        s->sim->applyConfig();
    });
}

extern "C" int fgs_time_op_in_graphs(fgs_sim* s, const char* label) {
    return guarded([&] {
        s->sim->CUDAConfig().time_op_label = label ? label : "";
        s->sim->applyConfig();
    });
}

extern "C" int fgs_harvest_profile(fgs_sim* s) { return guarded([&] { s->sim->harvestOperationTimes(); }); }

extern "C" int fgs_export(fgs_sim* s, const char* path) { return guarded([&] { s->sim->exportData(path); }); }

namespace {

template <typename T>
void add_reduction(flamegpu::LoggingConfig::AgentLoggingConfig& a, const std::string& op, const std::string& var) {
    if (op == "mean") a.logMean<T>(var);
    else if (op == "sd") a.logStandardDev<T>(var);
    else if (op == "min") a.logMin<T>(var);
    else if (op == "max") a.logMax<T>(var);
    else if (op == "sum") a.logSum<T>(var);
    else throw flamegpu::exception::InvalidArgument("unknown log reduction " + op);
}

void apply_log_spec(flamegpu::LoggingConfig& cfg, const flamegpu::ModelDescription& model, const std::string& spec) {
    size_t b = 0;
    while (b <= spec.size()) {
        size_t e = spec.find(';', b);
        if (e == std::string::npos) e = spec.size();
        const std::string item = spec.substr(b, e - b);
        b = e + 1;
        if (item.empty()) continue;
        std::vector<std::string> f;
        size_t p = 0;
        while (true) {
            const size_t q = item.find(':', p);
            f.push_back(item.substr(p, q == std::string::npos ? std::string::npos : q - p));
            if (q == std::string::npos) break;
            p = q + 1;
        }
        if (f[0] == "env" && f.size() == 2) {
            cfg.logEnvironment(f[1]);
        } else if (f[0] == "count" && f.size() == 3) {
            cfg.agent(f[1], f[2]).logCount();
        } else if (f.size() == 4) {
            auto a = cfg.agent(f[1], f[2]);
            const flamegpu::detail::Variable* v = model.getData()->agent(f[1])->find(f[3]);
            if (!v) throw flamegpu::exception::InvalidAgentVar("no variable " + f[3]);
            const std::type_index t = v->type;
            if (t == std::type_index(typeid(float))) add_reduction<float>(a, f[0], f[3]);
            else if (t == std::type_index(typeid(double))) add_reduction<double>(a, f[0], f[3]);
            else if (t == std::type_index(typeid(int32_t))) add_reduction<int32_t>(a, f[0], f[3]);
            else if (t == std::type_index(typeid(uint32_t))) add_reduction<uint32_t>(a, f[0], f[3]);
            else if (t == std::type_index(typeid(int64_t))) add_reduction<int64_t>(a, f[0], f[3]);
            else if (t == std::type_index(typeid(uint64_t))) add_reduction<uint64_t>(a, f[0], f[3]);
            else throw flamegpu::exception::InvalidVarType("unsupported variable type for the C ABI log");
        } else {
            throw flamegpu::exception::InvalidArgument("bad log entry '" + item + "'");
        }
    }
}

}  // namespace

extern "C" int fgs_set_log(fgs_sim* s, int32_t exit, const char* spec, uint32_t frequency) {
    return guarded([&] {
        if (exit) {
            flamegpu::LoggingConfig cfg(*s->model);
            apply_log_spec(cfg, *s->model, spec ? spec : "");
            s->sim->setExitLog(cfg);
        } else {
            flamegpu::StepLoggingConfig cfg(*s->model);
            apply_log_spec(cfg, *s->model, spec ? spec : "");
            cfg.setFrequency(frequency);
            s->sim->setStepLog(cfg);
        }
    });
}

extern "C" int fgs_run_log(fgs_sim* s, char* buf, size_t len, size_t* needed) {
    return guarded([&] {
        const std::string j = s->sim->runLogJSON();
        if (needed) *needed = j.size() + 1;
        if (buf && len) {
            std::strncpy(buf, j.c_str(), len - 1);
            buf[len - 1] = 0;
        }
    });
}

extern "C" int fgs_load_state(fgs_sim* s, const char* path) { return guarded([&] { s->sim->loadState(path); }); }

// SimulationConfig() / CUDAConfig() items by name, as text (the settings a state
// file carries: the reference's Simulation::Config and CUDASimulation::Config)
extern "C" int fgs_set_config(fgs_sim* s, const char* key, const char* value) {
    return guarded([&] {
        auto& c = s->sim->SimulationConfig();
        auto& g = s->sim->CUDAConfig();
        const std::string k = key, v = value ? value : "";
        auto flag = [&] { return v == "1" || v == "true"; };
        if (k == "input_file") c.input_file = v;
        else if (k == "step_log_file") c.step_log_file = v;
        else if (k == "exit_log_file") c.exit_log_file = v;
        else if (k == "common_log_file") c.common_log_file = v;
        else if (k == "truncate_log_files") c.truncate_log_files = flag();
        else if (k == "random_seed") c.random_seed = std::strtoull(v.c_str(), nullptr, 10);
        else if (k == "steps") c.steps = static_cast<unsigned int>(std::strtoul(v.c_str(), nullptr, 10));
        else if (k == "verbosity") c.verbosity = static_cast<unsigned int>(std::strtoul(v.c_str(), nullptr, 10));
        else if (k == "timing") c.timing = flag();
        else if (k == "device_id") g.device_id = std::atoi(v.c_str());
        else if (k == "inLayerConcurrency") g.inLayerConcurrency = flag();
        else THROW flamegpu::exception::InvalidArgument(flamegpu::exception::format("No config item '%s'", key));
    });
}

extern "C" int fgs_get_config(fgs_sim* s, const char* key, char* out, size_t len) {
    return guarded([&] {
        const auto& c = s->sim->SimulationConfig();
        const auto& g = s->sim->CUDAConfig();
        const std::string k = key;
        std::string v;
        if (k == "input_file") v = c.input_file;
        else if (k == "step_log_file") v = c.step_log_file;
        else if (k == "exit_log_file") v = c.exit_log_file;
        else if (k == "common_log_file") v = c.common_log_file;
        else if (k == "truncate_log_files") v = c.truncate_log_files ? "true" : "false";
        else if (k == "random_seed") v = std::to_string(c.random_seed);
        else if (k == "steps") v = std::to_string(c.steps);
        else if (k == "verbosity") v = std::to_string(c.verbosity);
        else if (k == "timing") v = c.timing ? "true" : "false";
        else if (k == "device_id") v = std::to_string(g.device_id);
        else if (k == "inLayerConcurrency") v = g.inLayerConcurrency ? "true" : "false";
        else THROW flamegpu::exception::InvalidArgument(flamegpu::exception::format("No config item '%s'", key));
        if (out && len) {
            std::strncpy(out, v.c_str(), len - 1);
            out[len - 1] = 0;
        }
    });
}

extern "C" int fgs_take_profile(fgs_sim* s, char* buf, size_t len) {
    return guarded([&] {
        std::string out;
        for (const auto& t : s->sim->takeOperationProfile()) {
            char tmp[512];
            std::snprintf(tmp, sizeof(tmp), "%s,%.6f,%llu;", std::get<0>(t).c_str(), std::get<1>(t), std::get<2>(t));
            out += tmp;
        }
        if (len) {
            std::strncpy(buf, out.c_str(), len - 1);
            buf[len - 1] = 0;
        }
    });
}

extern "C" int fgs_set_stage_bytes(fgs_sim* s, uint32_t bytes) {
    return guarded([&] {
        s->sim->CUDAConfig().message_stage_bytes = bytes;
        s->sim->applyConfig();
    });
}

// ---------------------------------------------------------------- ensembles

struct fge_ensemble {
    std::unique_ptr<flamegpu::ModelDescription> model;
    std::unique_ptr<flamegpu::CUDAEnsemble> ens;
    std::unique_ptr<flamegpu::RunPlanVector> plans;
};

extern "C" fge_ensemble* fge_create(const char* model, const double* params, int32_t nparams, int32_t device) {
    fge_ensemble* out = nullptr;
    guarded([&] {
        fgs_model_factory f = nullptr;
        {
            std::lock_guard<std::mutex> lk(g_reg_mu);
            auto it = registry().find(model);
            if (it == registry().end()) throw flamegpu::exception::InvalidArgument(std::string("unknown model ") + model);
            f = it->second;
        }
        auto e = std::make_unique<fge_ensemble>();
        e->model.reset(static_cast<flamegpu::ModelDescription*>(f(params, nparams)));
        e->ens = std::make_unique<flamegpu::CUDAEnsemble>(*e->model);
        e->ens->Config().device = device;
        e->plans = std::make_unique<flamegpu::RunPlanVector>(*e->model, 0);
        out = e.release();
    });
    return out;
}

extern "C" void fge_destroy(fge_ensemble* e) { delete e; }

extern "C" int fge_configure(fge_ensemble* e, int32_t batched, int32_t graphs, uint32_t stage) {
    return guarded([&] {
        e->ens->Config().batched = batched != 0;
        e->ens->Config().use_graphs = graphs != 0;
        e->ens->Config().message_stage_bytes = stage;
    });
}

extern "C" int fge_add_run(fge_ensemble* e, uint32_t steps, uint64_t seed, const char* agent, uint32_t n, int32_t nvars,
                           const char* const* names, const void* const* cols, const char* message, const float* mn,
                           const float* mx, float radius) {
    return guarded([&] {
        flamegpu::RunPlan plan(*e->model);
        plan.setSteps(steps);
        plan.setRandomSimulationSeed(seed);
        if (agent) {
            flamegpu::AgentVector pop(e->model->Agent(agent), n);
            for (int32_t k = 0; k < nvars; ++k) {
                const size_t c = pop.columnIndex(names[k]);
                std::memcpy(pop.columns()[c].data(), cols[k], pop.columns()[c].size());
            }
            plan.setPopulation(std::move(pop));
        }
        if (message) plan.setSpatialMessageBounds(message, {mn[0], mn[1], mn[2]}, {mx[0], mx[1], mx[2]}, radius);
        e->plans->push_back(plan);
    });
}

extern "C" int fge_set_run_property(fge_ensemble* e, uint32_t run, const char* name, const void* value, size_t bytes) {
    return guarded([&] {
        if (run >= e->plans->size()) throw flamegpu::exception::OutOfBoundsException("run out of range");
        flamegpu::RunPlan& p = (*e->plans)[run];
        const flamegpu::detail::EnvProperty* prop = e->model->getData()->property(name);
        if (!prop || prop->value.size() != bytes) throw flamegpu::exception::InvalidEnvProperty(name);
        if (prop->type == std::type_index(typeid(float))) p.setProperty<float>(name, *static_cast<const float*>(value));
        else if (prop->type == std::type_index(typeid(double))) p.setProperty<double>(name, *static_cast<const double*>(value));
        else if (prop->type == std::type_index(typeid(int32_t))) p.setProperty<int32_t>(name, *static_cast<const int32_t*>(value));
        else if (prop->type == std::type_index(typeid(uint32_t))) p.setProperty<uint32_t>(name, *static_cast<const uint32_t*>(value));
        else if (prop->type == std::type_index(typeid(uint64_t))) p.setProperty<uint64_t>(name, *static_cast<const uint64_t*>(value));
        else throw flamegpu::exception::InvalidEnvPropertyType("unsupported property type for the C ABI");
    });
}

extern "C" int fge_simulate(fge_ensemble* e, uint32_t* failures) {
    return guarded([&] {
        const unsigned int f = e->ens->simulate(*e->plans);
        if (failures) *failures = f;
    });
}

extern "C" int fge_get_count(fge_ensemble* e, uint32_t run, const char* agent, uint32_t* n) {
    return guarded([&] { *n = e->ens->getPopulationView(run, agent)->size(); });
}

extern "C" int fge_get_variable(fge_ensemble* e, uint32_t run, const char* agent, const char* var, void* out,
                                size_t bytes) {
    return guarded([&] {
        const auto pop = e->ens->getPopulationView(run, agent);
        const auto& col = pop->columns()[pop->columnIndex(var)];
        if (bytes < col.size()) throw flamegpu::exception::InvalidArgument("output buffer too small");
        std::memcpy(out, col.data(), col.size());
    });
}

extern "C" int fge_stats(fge_ensemble* e, double* el, int32_t* batched, uint32_t* kps, uint64_t* gl) {
    return guarded([&] {
        if (el) *el = e->ens->getEnsembleElapsedTime();
        if (batched) *batched = e->ens->lastRunBatched() ? 1 : 0;
        if (kps) *kps = e->ens->getKernelsPerStep();
        if (gl) *gl = e->ens->getGraphLaunches();
    });
}

extern "C" int fge_set_tuning(fge_ensemble* e, int32_t mode, const char* cache_path) {
    return guarded([&] {
        if (mode < 0 || mode > 2) THROW flamegpu::exception::InvalidArgument("tuning mode must be 0, 1 or 2");
        e->ens->Config().tuning = mode;
        e->ens->Config().tuning_cache = cache_path ? cache_path : "";
    });
}

extern "C" int fge_tuning(fge_ensemble* e, char* json, size_t len) {
    return guarded([&] {
        const std::string& t = e->ens->getTuning();
        if (json && len) {
            std::strncpy(json, t.c_str(), len - 1);
            json[len - 1] = 0;
        }
    });
}

extern "C" int fge_step_time(fge_ensemble* e, double* seconds) {
    return guarded([&] { *seconds = e->ens->getEnsembleStepTime(); });
}

// ------------------------------------------------------------------- server

struct fgv_server {
    std::unique_ptr<flamegpu::SimulationServer> server;
    // model descriptions shared by the runs that asked for the same (model, params)
    std::map<std::pair<std::string, std::vector<double>>, std::shared_ptr<flamegpu::ModelDescription>> models;
    std::map<uint64_t, flamegpu::SimulationServer::Result> results;
    std::vector<uint64_t> pending;  // completed ids not yet handed out
};

namespace {

const flamegpu::SimulationServer::Result& result_of(fgv_server* v, uint64_t id) {
    auto it = v->results.find(id);
    if (it == v->results.end()) throw flamegpu::exception::InvalidArgument("no completed run with id " + std::to_string(id));
    return it->second;
}

const flamegpu::AgentVector& result_population(fgv_server* v, uint64_t id, const char* agent, const char* state) {
    const auto& r = result_of(v, id);
    if (r.failed) throw flamegpu::exception::InvalidArgument("run " + std::to_string(id) + " failed: " + r.error);
    auto it = r.populations.find({agent, state ? state : "default"});
    if (it == r.populations.end()) throw flamegpu::exception::InvalidAgentName(std::string("no population ") + agent);
    return *it->second;
}

}  // namespace

extern "C" fgv_server* fgv_create(int32_t device, uint64_t budget, uint32_t max_active, uint32_t steps_per_poll,
                                  int32_t graphs) {
    fgv_server* out = nullptr;
    guarded([&] {
        flamegpu::SimulationServer::Config c;
        c.device = device;
        if (budget) c.memory_budget = budget;
        if (max_active) c.max_active = max_active;
        if (steps_per_poll) c.steps_per_poll = steps_per_poll;
        c.use_graphs = graphs != 0;
        auto v = std::make_unique<fgv_server>();
        v->server = std::make_unique<flamegpu::SimulationServer>(c);
        out = v.release();
    });
    return out;
}

extern "C" void fgv_destroy(fgv_server* v) { delete v; }

extern "C" int fgv_submit(fgv_server* v, const char* model, const double* params, int32_t nparams, uint32_t steps,
                          uint64_t seed, int32_t npops, const char* const* agents, const uint32_t* counts,
                          const int32_t* nvars, const char* const* names, const void* const* cols, uint64_t* id) {
    return guarded([&] {
        const auto key = std::make_pair(std::string(model), std::vector<double>(params, params + std::max(nparams, 0)));
        auto& m = v->models[key];
        if (!m) {
            fgs_model_factory f = nullptr;
            {
                std::lock_guard<std::mutex> lk(g_reg_mu);
                auto it = registry().find(model);
                if (it == registry().end())
                    throw flamegpu::exception::InvalidArgument(std::string("unknown model ") + model);
                f = it->second;
            }
            m.reset(static_cast<flamegpu::ModelDescription*>(f(params, nparams)));
        }
        std::vector<std::pair<std::string, flamegpu::AgentVector>> pops;
        int32_t c = 0;
        for (int32_t k = 0; k < npops; ++k) {
            flamegpu::AgentVector pop(m->Agent(agents[k]), counts[k]);
            for (int32_t j = 0; j < nvars[k]; ++j, ++c) {
                const size_t col = pop.columnIndex(names[c]);
                std::memcpy(pop.columns()[col].data(), cols[c], pop.columns()[col].size());
            }
            pops.emplace_back(agents[k], std::move(pop));
        }
        const uint64_t rid = v->server->submit(m, std::move(pops), steps, seed);
        if (id) *id = rid;
    });
}

extern "C" int fgv_poll(fgv_server* v, uint32_t* remaining) {
    return guarded([&] {
        const size_t r = v->server->poll();
        if (remaining) *remaining = static_cast<uint32_t>(r);
    });
}

extern "C" int fgv_run_until_idle(fgv_server* v) { return guarded([&] { v->server->runUntilIdle(); }); }

extern "C" int fgv_take_completed(fgv_server* v, uint64_t* ids, uint32_t cap, uint32_t* n) {
    return guarded([&] {
        auto& pending = v->pending;
        for (auto& r : v->server->takeCompleted()) {
            pending.push_back(r.id);
            v->results.emplace(r.id, std::move(r));
        }
        uint32_t k = 0;
        while (k < cap && k < pending.size()) {
            ids[k] = pending[k];
            ++k;
        }
        pending.erase(pending.begin(), pending.begin() + k);
        if (n) *n = k;
    });
}

extern "C" int fgv_result_agent_steps(fgv_server* v, uint64_t id, uint64_t* agent_steps) {
    return guarded([&] { *agent_steps = result_of(v, id).agent_steps; });
}

extern "C" int fgv_result_info(fgv_server* v, uint64_t id, double* t, int32_t* failed, char* err, size_t len) {
    return guarded([&] {
        const auto& r = result_of(v, id);
        if (t) {
            t[0] = r.arrival_s;
            t[1] = r.admitted_s;
            t[2] = r.completed_s;
        }
        if (failed) *failed = r.failed ? 1 : 0;
        if (err && len) {
            std::strncpy(err, r.error.c_str(), len - 1);
            err[len - 1] = 0;
        }
    });
}

extern "C" int fgv_result_count(fgv_server* v, uint64_t id, const char* agent, const char* state, uint32_t* n) {
    return guarded([&] { *n = result_population(v, id, agent, state).size(); });
}

extern "C" int fgv_result_variable(fgv_server* v, uint64_t id, const char* agent, const char* state, const char* var,
                                   void* out, size_t bytes) {
    return guarded([&] {
        const auto& pop = result_population(v, id, agent, state);
        const auto& col = pop.columns()[pop.columnIndex(var)];
        if (bytes < col.size()) throw flamegpu::exception::InvalidArgument("output buffer too small");
        std::memcpy(out, col.data(), col.size());
    });
}

extern "C" int fgv_release(fgv_server* v, uint64_t id) { return guarded([&] { v->results.erase(id); }); }

extern "C" int fgv_stats(fgv_server* v, uint32_t* q, uint32_t* a, uint64_t* r) {
    return guarded([&] {
        if (q) *q = static_cast<uint32_t>(v->server->queued());
        if (a) *a = static_cast<uint32_t>(v->server->active());
        if (r) *r = v->server->reservedBytes();
    });
}

extern "C" int fgv_counters(fgv_server* v, uint64_t* polls, double* poll_s, uint64_t* steps) {
    return guarded([&] {
        const auto c = v->server->counters();
        if (polls) *polls = c.polls;
        if (poll_s) *poll_s = c.poll_seconds;
        if (steps) *steps = c.steps_issued;
    });
}

extern "C" int fgv_set_scheduling(fgv_server* v, double work, double total) {
    return guarded([&] { v->server->setScheduling(work, total); });
}
