// CUDAEnsemble on GB300: RunPlans become instances of one batched simulation.
//
// Layout. Instance k owns rows [row_begin_k, row_begin_k + cap_k) of every
// agent column and message column (cap_k = its population rounded up to the
// 128-thread agent block, so no block straddles two instances). Each spatial
// message list keeps one concatenated record buffer and one PBM: instance k's
// bins are buckets [bucket_begin_k, bucket_begin_k + binCount_k] (+1 padding
// bucket), so a single segmented counting sort builds every instance's index
// and its PBM is the slice at bucket_begin_k. The automatic agent sort is
// batched the same way over per-instance sort buckets. Agent function kernels
// find their block's instance in a small table (grid, PBM offset, environment
// buffer, seed, step offset) and otherwise run the model code unchanged. One
// CUDA graph per buffer parity replays a whole ensemble step.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "flamegpu/simulation/CUDAEnsemble.h"
#include "flamegpu/detail/launch.cuh"
#include "flamegpu/simulation/CUDASimulation.h"
#include "flamegpu_gb300/fg_capi.h"
#include "runtime/internal.h"
#include "runtime/json.h"

namespace flamegpu {

using exception::format;

#define FG_ECUDA(call)                                                                                     \
    do {                                                                                                   \
        const cudaError_t _e = (call);                                                                     \
        if (_e != cudaSuccess)                                                                             \
            THROW exception::CUDAError(format("%s failed: %s (%s:%d)", #call, cudaGetErrorString(_e), __FILE__, __LINE__)); \
    } while (0)
#define FG_ECAPI(call)                                                                                     \
    do {                                                                                                   \
        const int _r = (call);                                                                             \
        if (_r != FG_OK) THROW exception::CUDAError(format("%s returned %d (%s:%d)", #call, _r, __FILE__, __LINE__)); \
    } while (0)

// ------------------------------------------------------------------ RunPlan

RunPlan::RunPlan(const ModelDescription& model) : model_(model.getData()) {}

void RunPlan::set_property(const std::string& name, std::type_index t, size_t size, const void* v) {
    const detail::EnvProperty* p = model_->property(name);
    if (!p) THROW exception::InvalidEnvProperty(format("Environment has no property '%s'", name.c_str()));
    if (p->type != t || p->type_size != size || p->elements != 1)
        THROW exception::InvalidEnvPropertyType(format("Environment property '%s' has another type", name.c_str()));
    std::vector<char> bytes(size);
    std::memcpy(bytes.data(), v, size);
    properties_[name] = std::move(bytes);
}

void RunPlan::setPopulation(AgentVector&& population, const std::string& state) {
    const std::string name = population.getAgentName();
    populations_[{name, state}] = std::make_shared<AgentVector>(std::move(population));
}

void RunPlan::setPopulation(const AgentVector& population, const std::string& state) {
    populations_[{population.getAgentName(), state}] = std::make_shared<AgentVector>(population);
}

void RunPlan::setSpatialMessageBounds(const std::string& message, const std::vector<float>& mn,
                                      const std::vector<float>& mx, float radius) {
    const detail::MessageData* m = model_->message(message);
    if (!m || (m->kind != detail::MessageKind::Spatial2D && m->kind != detail::MessageKind::Spatial3D))
        THROW exception::InvalidMessageName(format("No spatial message '%s'", message.c_str()));
    spatial_[message] = SpatialOverride{mn, mx, radius};
}

RunPlanVector::RunPlanVector(const ModelDescription& model, unsigned int n) {
    for (unsigned int i = 0; i < n; ++i) emplace_back(model);
}

void RunPlanVector::setSteps(unsigned int steps) {
    for (auto& p : *this) p.setSteps(steps);
}

void RunPlanVector::setRandomSimulationSeed(uint64_t initial_seed, unsigned int step) {
    uint64_t s = initial_seed;
    for (auto& p : *this) {
        p.setRandomSimulationSeed(s);
        s += step;
    }
}

namespace detail {

namespace {

__global__ void k_batch_step_increment(uint32_t* d_step) {
    grid_dependency_enter();
    *d_step += 1;
}

constexpr uint32_t kRowAlign = kAgentBlock;

uint32_t round_rows(uint32_t n) { return std::max(kRowAlign, (n + kRowAlign - 1) / kRowAlign * kRowAlign); }

struct Alloc {
    std::vector<void*> ptrs;
    void* get(size_t bytes) {
        void* p = nullptr;
        FG_ECUDA(cudaMalloc(&p, std::max<size_t>(bytes, 256)));
        FG_ECUDA(cudaMemset(p, 0, std::max<size_t>(bytes, 256)));
        ptrs.push_back(p);
        return p;
    }
    // frees p (null: nothing); the device must be done with it
    void release(void* p) {
        if (!p) return;
        auto it = std::find(ptrs.begin(), ptrs.end(), p);
        if (it != ptrs.end()) {
            cudaFree(p);
            ptrs.erase(it);
        }
    }
    void* release_and_get(void* p, size_t bytes) {
        release(p);
        return get(bytes);
    }
    ~Alloc() {
        for (void* p : ptrs) cudaFree(p);
    }
};

}  // namespace

/** Why a model cannot run as one batched simulation ("" if it can). */
std::string batch_unsupported(const ModelData& m) {
    if (m.agents.size() != 1) return "the model has more than one agent type";
    const AgentData& a = *m.agents[0];
    if (a.states.size() != 1) return "the agent has more than one state";
    if (!m.init_functions.empty() || !m.step_functions.empty() || !m.exit_functions.empty() ||
        !m.exit_conditions.empty())
        return "the model has host functions";
    for (const auto& l : m.layers)
        if (!l->host_functions.empty()) return "the model has host layer functions";
    if (!m.macro_environment.empty()) return "the model has environment macro properties";
    for (const auto& f : a.functions)
        for (const auto& g : a.functions)
            if (f != g && !f->message_output.empty() && f->message_output == g->message_output)
                return "a message list output by more than one function";
    for (const auto& f : a.functions) {
        if (!f->agent_output.empty() && (f->agent_output != a.name || f->agent_output_state != a.states[0]))
            return "agent birth into another agent type or state";
        if (f->condition) return "an agent function condition";
        if (f->message_output_optional) return "optional message output";
        if (!f->message_input.empty() && m.message(f->message_input)->kind == MessageKind::BruteForce)
            return "brute-force message input";
        if ((!f->message_input.empty() && array_dims(m.message(f->message_input)->kind)) ||
            (!f->message_output.empty() && array_dims(m.message(f->message_output)->kind)))
            return "array messages";
        if ((!f->message_input.empty() && m.message(f->message_input)->kind == MessageKind::Bucket) ||
            (!f->message_output.empty() && m.message(f->message_output)->kind == MessageKind::Bucket))
            return "bucket messages";
    }
    return "";
}

/** One ensemble run as a single batched simulation. */
struct BatchedSim {
    std::shared_ptr<ModelData> model;
    AgentData* agent = nullptr;
    const RunPlanVector& plans;
    const CUDAEnsemble::EnsembleConfig& cfg;
    Alloc mem;
    cudaStream_t stream = nullptr, side = nullptr;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    int sms = 132;
    uint32_t ninst = 0, total_rows = 0;
    std::vector<uint32_t> row_begin, cap, count;
    std::vector<std::array<void*, 2>> cols;  // per agent variable
    int parity = 0;
    uint32_t* d_counts = nullptr;
    uint32_t* d_next_ids = nullptr;  // next agent id per instance
    uint32_t* d_misc = nullptr;  // [0] step, [1..4] error record
    std::vector<size_t> env_offset;
    size_t env_stride = 0;
    char* d_env = nullptr;
    int id_col = -1;
    // birth / death: births per step at most double an instance per birth
    // function; bound[k] bounds instance k's population (host)
    int birth_fns = 0;
    bool death_or_birth = false;
    std::vector<uint64_t> bound;
    uint32_t* d_tile_begin = nullptr;  // compaction tiles per instance (ninst + 1)
    uint32_t comp_tiles = 0;
    void* comp_ws = nullptr;
    size_t comp_ws_bytes = 0;
    // population reports copied after steps, for bounds without a wait
    struct Report {
        cudaEvent_t ev = nullptr;
        uint32_t* host = nullptr;
        unsigned int step_after = 0;  // the report holds the counts entering this step
        bool used = false;
    };
    std::vector<Report> reports;
    size_t report_next = 0;
    uint32_t* reports_pinned = nullptr;
    unsigned int relayouts = 0;

    struct BMsg {
        MessageData* msg = nullptr;
        int dims = 0;
        std::vector<uint32_t> slot_bytes, field_word;
        uint32_t record_words = 0;
        uint32_t pay_mult = 0, pay_shift = 0, pay_stride = 0;  // record layout of the non-location fields
        std::vector<void*> cols;
        uint32_t* records = nullptr;
        uint32_t* pbm = nullptr;
        uint32_t total_buckets = 0;
        std::vector<fg_batch_instance> inst;
        fg_batch_instance* d_inst = nullptr;
        void* ws = nullptr;
        size_t ws_bytes = 0;
        bool needs_build = true;
    };
    std::vector<std::unique_ptr<BMsg>> msgs;

    struct BFn {
        AgentFunctionData* fn = nullptr;
        BMsg* in = nullptr;
        BMsg* out = nullptr;
        bool sort = false;
        bool births = false;
        std::vector<fg_batch_instance> sort_inst;
        fg_batch_instance* d_sort_inst = nullptr;
        uint32_t sort_buckets = 0;
        void* sort_ws = nullptr;
        size_t sort_ws_bytes = 0;
        BatchInstanceRT* d_rt = nullptr;
        uint32_t* death_flags = nullptr;
        uint32_t* birth_flags = nullptr;
        std::vector<void*> birth_cols;
        void* birth_defaults = nullptr;
        std::unique_ptr<FunctionTables> tables[2];
    };
    std::vector<BFn> fns;
    unsigned int kernels_per_step = 0;
    unsigned long long graph_launches = 0;
    std::map<std::pair<int, bool>, cudaGraphExec_t> cache;

    // Launch shape of the batched step (the autotuner's knobs): threads per
    // agent-function block, resident blocks per SM of its grid-stride grid,
    // shared memory for staged neighbourhoods, and the scans' wide-tile
    // threshold (fg_tuning; 0: the library's default).
    struct Shape {
        uint32_t block = kAgentBlock;
        uint32_t blocks_per_sm = 16;
        uint32_t stage_bytes = 96u * 1024u;
        uint32_t scan_wide_min = 0;
    };
    Shape shape;
    std::string tuning_json = "{\"tuned\": false}";

    BatchedSim(std::shared_ptr<ModelData> m, const RunPlanVector& p, const CUDAEnsemble::EnsembleConfig& c)
        : model(std::move(m)), plans(p), cfg(c) {}
    ~BatchedSim() {
        drop_graphs();
        for (auto& r : reports)
            if (r.ev) cudaEventDestroy(r.ev);
        if (reports_pinned) cudaFreeHost(reports_pinned);
        if (fork_ev) cudaEventDestroy(fork_ev);
        if (join_ev) cudaEventDestroy(join_ev);
        if (side) cudaStreamDestroy(side);
        if (stream) cudaStreamDestroy(stream);
    }

    void drop_graphs() {
        for (auto& c : cache) cudaGraphExecDestroy(c.second);
        cache.clear();
    }

    BMsg* msg_of(const std::string& name) {
        for (auto& m : msgs)
            if (m->msg->name == name) return m.get();
        return nullptr;
    }

    // Message grid of run k (the plan's override, else the model's bounds).
    fg_spatial_grid grid_of(const MessageData* m, uint32_t k) const {
        const int dims = m->kind == MessageKind::Spatial3D ? 3 : 2;
        std::vector<float> mn(m->min, m->min + 3), mx(m->max, m->max + 3);
        float r = m->radius;
        auto it = plans[k].spatial().find(m->name);
        if (it != plans[k].spatial().end()) {
            mn = it->second.min;
            mx = it->second.max;
            r = it->second.radius;
            mn.resize(3, 0.0f);
            mx.resize(3, 0.0f);
        }
        fg_spatial_grid g{};
        if (fg_spatial_grid_init(&g, dims, mn.data(), mx.data(), r) != FG_OK)
            THROW exception::InvalidArgument(format("Run %u: invalid bounds/radius for message '%s'", k, m->name.c_str()));
        return g;
    }

    // Rows of an instance of n agents: its agents plus room for the births of
    // two steps, rounded up to the agent block.
    uint32_t rows_for(uint64_t n) const {
        const uint64_t grow = birth_fns ? (1ull << std::min(2 * birth_fns, 8)) : 1ull;
        const uint64_t r = std::max<uint64_t>(1, n) * grow;
        if (r >= (1ull << 31)) THROW exception::OutOfMemory("An ensemble run may exceed 2^31 agents");
        return round_rows(static_cast<uint32_t>(r));
    }

    void setup() {
        FG_ECUDA(cudaSetDevice(cfg.device));
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, cfg.device);
        if (sms <= 0) sms = 132;
        FG_ECUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        FG_ECUDA(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
        FG_ECUDA(cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming));
        FG_ECUDA(cudaEventCreateWithFlags(&join_ev, cudaEventDisableTiming));
        agent = model->agents[0].get();
        const std::string state = agent->states[0];
        ninst = static_cast<uint32_t>(plans.size());
        for (size_t v = 0; v < agent->variables.size(); ++v)
            if (agent->variables[v].name == "_id") id_col = static_cast<int>(v);
        for (const auto& f : agent->functions) {
            if (!f->agent_output.empty()) ++birth_fns;
            death_or_birth = death_or_birth || f->has_agent_death || !f->agent_output.empty();
        }
        // ---- row segments
        for (uint32_t k = 0; k < ninst; ++k) {
            auto it = plans[k].populations().find({agent->name, state});
            const uint32_t n = it == plans[k].populations().end() ? 0u : it->second->size();
            count.push_back(n);
            bound.push_back(n);
            cap.push_back(rows_for(n));
        }
        place_rows();
        cols.resize(agent->variables.size());
        for (size_t v = 0; v < cols.size(); ++v) {
            const size_t b = agent->variables[v].bytes();
            cols[v] = {mem.get(b * total_rows), mem.get(b * total_rows)};
        }
        std::vector<id_t> next(ninst, 1);
        for (uint32_t k = 0; k < ninst; ++k) {
            auto it = plans[k].populations().find({agent->name, state});
            if (it == plans[k].populations().end() || count[k] == 0) continue;
            // ids are per run: unset ones are filled (CUDAFatAgent.cu:311-319), in
            // a copy of the id column only
            const AgentVector& pop = *it->second;
            const size_t idc = pop.columnIndex("_id");
            const id_t* ids = reinterpret_cast<const id_t*>(pop.columns()[idc].data());
            std::vector<id_t> filled;
            for (uint32_t i = 0; i < count[k]; ++i) next[k] = std::max<id_t>(next[k], ids[i] + 1);
            for (uint32_t i = 0; i < count[k]; ++i) {
                if (ids[i] != ID_NOT_SET) continue;
                if (filled.empty()) filled.assign(ids, ids + count[k]);
                filled[i] = next[k]++;
            }
            for (size_t v = 0; v < cols.size(); ++v) {
                const size_t b = agent->variables[v].bytes();
                const void* src = (v == idc && !filled.empty()) ? static_cast<const void*>(filled.data())
                                                                 : static_cast<const void*>(pop.columns()[v].data());
                FG_ECUDA(cudaMemcpy(static_cast<char*>(cols[v][0]) + b * row_begin[k], src, b * count[k],
                                    cudaMemcpyHostToDevice));
            }
        }
        d_counts = static_cast<uint32_t*>(mem.get(sizeof(uint32_t) * ninst));
        FG_ECUDA(cudaMemcpy(d_counts, count.data(), sizeof(uint32_t) * ninst, cudaMemcpyHostToDevice));
        d_next_ids = static_cast<uint32_t*>(mem.get(sizeof(uint32_t) * ninst));
        FG_ECUDA(cudaMemcpy(d_next_ids, next.data(), sizeof(uint32_t) * ninst, cudaMemcpyHostToDevice));
        d_misc = static_cast<uint32_t*>(mem.get(64));
        // ---- environments: the model's values with each plan's overrides
        size_t off = 0;
        for (const auto& p : model->environment) {
            env_offset.push_back(off);
            off += (p.value.size() + 7) & ~size_t(7);
        }
        env_stride = std::max<size_t>(256, (off + 255) & ~size_t(255));
        std::vector<char> envs(env_stride * ninst, 0);
        for (uint32_t k = 0; k < ninst; ++k)
            for (size_t i = 0; i < model->environment.size(); ++i) {
                const auto& p = model->environment[i];
                auto ov = plans[k].properties().find(p.name);
                const std::vector<char>& val = ov == plans[k].properties().end() ? p.value : ov->second;
                std::memcpy(envs.data() + env_stride * k + env_offset[i], val.data(), val.size());
            }
        d_env = static_cast<char*>(mem.get(envs.size()));
        FG_ECUDA(cudaMemcpy(d_env, envs.data(), envs.size(), cudaMemcpyHostToDevice));
        // ---- message lists (row-independent part)
        for (const auto& m : model->messages) {
            auto bm = std::make_unique<BMsg>();
            bm->msg = m.get();
            bm->dims = m->kind == MessageKind::Spatial3D ? 3 : (m->kind == MessageKind::Spatial2D ? 2 : 0);
            std::vector<std::pair<uint32_t, uint32_t>> vars;
            for (const auto& v : m->variables) {
                const uint32_t sb = (v.bytes() + 3u) & ~3u;
                bm->slot_bytes.push_back(sb);
                vars.emplace_back(fnv1a32(v.name), sb);
            }
            if (bm->dims) {
                const SpatialRecordLayout L = spatial_record_layout(vars, bm->dims, m->name.c_str());
                bm->field_word = L.field_word;
                bm->record_words = L.record_words;
                bm->pay_mult = L.pay_mult;
                bm->pay_shift = L.pay_shift;
                bm->pay_stride = L.pay_stride;
            }
            msgs.push_back(std::move(bm));
        }
        // ---- agent functions (row-independent part)
        for (const auto& f : agent->functions) {
            BFn b;
            b.fn = f.get();
            b.in = f->message_input.empty() ? nullptr : msg_of(f->message_input);
            b.out = f->message_output.empty() ? nullptr : msg_of(f->message_output);
            b.births = !f->agent_output.empty();
            if (b.in && b.in->dims) {
                bool ok = true;
                const char* ax[3] = {"x", "y", "z"};
                for (int d = 0; d < b.in->dims; ++d) {
                    const Variable* v = agent->find(ax[d]);
                    ok = ok && v && v->type == std::type_index(typeid(float)) && v->elements == 1;
                }
                b.sort = ok;
            }
            if (b.births) {
                std::vector<char> defaults;
                for (const auto& var : agent->variables) {
                    defaults.insert(defaults.end(), var.default_value.begin(), var.default_value.end());
                    defaults.resize((defaults.size() + 7) & ~size_t(7));
                }
                b.birth_defaults = mem.get(defaults.size());
                FG_ECUDA(cudaMemcpy(b.birth_defaults, defaults.data(), defaults.size(), cudaMemcpyHostToDevice));
            }
            fns.push_back(std::move(b));
        }
        layout_rows();
        if (death_or_birth) {
            FG_ECUDA(cudaMallocHost(&reports_pinned, sizeof(uint32_t) * ninst * 4));
            reports.resize(4);
            for (size_t r = 0; r < reports.size(); ++r) {
                FG_ECUDA(cudaEventCreateWithFlags(&reports[r].ev, cudaEventDisableTiming));
                reports[r].host = reports_pinned + r * ninst;
            }
        }
    }

    // row_begin from cap; total_rows
    void place_rows() {
        row_begin.assign(ninst, 0);
        uint64_t row = 0;
        for (uint32_t k = 0; k < ninst; ++k) {
            row_begin[k] = static_cast<uint32_t>(row);
            row += cap[k];
            if (row >= (1ull << 31)) THROW exception::OutOfMemory("Ensemble exceeds 2^31 agent rows");
        }
        total_rows = static_cast<uint32_t>(row);
    }

    // Every buffer and table that depends on the row segments (columns excepted):
    // message columns and records, the instance tables of the builds, sorts and
    // agent launches, flags and birth staging, workspaces, function tables.
    void layout_rows() {
        for (auto& mp : msgs) {
            BMsg& bm = *mp;
            for (void* p : bm.cols) mem.release(p);
            bm.cols.clear();
            for (uint32_t sb : bm.slot_bytes) bm.cols.push_back(mem.get(static_cast<size_t>(sb) * total_rows));
            if (!bm.dims) continue;
            mem.release(bm.records);
            bm.records = static_cast<uint32_t*>(mem.get(sizeof(uint32_t) * bm.record_words * static_cast<size_t>(total_rows)));
            bm.inst.clear();
            uint32_t bucket = 0;
            for (uint32_t k = 0; k < ninst; ++k) {
                fg_batch_instance bi{};
                const fg_spatial_grid g = grid_of(bm.msg, k);
                uint32_t nb = 0;
                FG_ECAPI(fg_batch_instance_init(&bi, &g, row_begin[k], cap[k], bucket, 0, &nb));
                bm.inst.push_back(bi);
                bucket += (nb + 3u) & ~3u;  // 16-byte aligned PBM slices (staging copies)
            }
            if (!bm.pbm) {
                bm.total_buckets = bucket;
                bm.pbm = static_cast<uint32_t*>(mem.get(sizeof(uint32_t) * (static_cast<size_t>(bucket) + 8)));
            }
            if (!bm.d_inst) bm.d_inst = static_cast<fg_batch_instance*>(mem.get(sizeof(fg_batch_instance) * ninst));
            FG_ECUDA(cudaMemcpy(bm.d_inst, bm.inst.data(), sizeof(fg_batch_instance) * ninst, cudaMemcpyHostToDevice));
            mem.release(bm.ws);
            bm.ws_bytes = fg_batched_workspace_size(total_rows, bm.total_buckets);
            bm.ws = mem.get(bm.ws_bytes);
        }
        for (auto& b : fns) {
            if (b.sort) {
                b.sort_inst.clear();
                uint32_t bucket = 0;
                for (uint32_t k = 0; k < ninst; ++k) {
                    fg_batch_instance bi{};
                    const fg_spatial_grid g = grid_of(b.in->msg, k);
                    uint32_t nb = 0;
                    FG_ECAPI(fg_batch_instance_init(&bi, &g, row_begin[k], cap[k], bucket, 1, &nb));
                    b.sort_inst.push_back(bi);
                    bucket += nb;
                }
                b.sort_buckets = bucket;
                if (!b.d_sort_inst) b.d_sort_inst = static_cast<fg_batch_instance*>(mem.get(sizeof(fg_batch_instance) * ninst));
                FG_ECUDA(cudaMemcpy(b.d_sort_inst, b.sort_inst.data(), sizeof(fg_batch_instance) * ninst, cudaMemcpyHostToDevice));
                mem.release(b.sort_ws);
                b.sort_ws_bytes = fg_batched_workspace_size(total_rows, bucket);
                b.sort_ws = mem.get(b.sort_ws_bytes);
            }
            std::vector<BatchInstanceRT> rt(ninst);
            for (uint32_t k = 0; k < ninst; ++k) {
                rt[k].row_begin = row_begin[k];
                rt[k].row_capacity = cap[k];
                rt[k].step_offset = 0;
                rt[k].env = d_env + env_stride * k;
                rt[k].seed = plans[k].getRandomSimulationSeed();
                if (b.in && b.in->dims) {
                    rt[k].in_grid = b.in->inst[k].grid;
                    rt[k].in_bucket_begin = b.in->inst[k].bucket_begin;
                }
            }
            if (!b.d_rt) b.d_rt = static_cast<BatchInstanceRT*>(mem.get(sizeof(BatchInstanceRT) * ninst));
            FG_ECUDA(cudaMemcpy(b.d_rt, rt.data(), sizeof(BatchInstanceRT) * ninst, cudaMemcpyHostToDevice));
            if (b.fn->has_agent_death) {
                mem.release(b.death_flags);
                b.death_flags = static_cast<uint32_t*>(mem.get(sizeof(uint32_t) * total_rows));
            }
            if (b.births) {
                mem.release(b.birth_flags);
                b.birth_flags = static_cast<uint32_t*>(mem.get(sizeof(uint32_t) * total_rows));
                for (void* p : b.birth_cols) mem.release(p);
                b.birth_cols.clear();
                for (const auto& v : agent->variables) b.birth_cols.push_back(mem.get(static_cast<size_t>(v.bytes()) * total_rows));
            }
            build_tables(b);
        }
        if (death_or_birth) {
            std::vector<fg_batch_instance> ci(ninst);
            for (uint32_t k = 0; k < ninst; ++k) {
                ci[k] = fg_batch_instance{};
                ci[k].row_begin = row_begin[k];
                ci[k].row_capacity = cap[k];
            }
            std::vector<uint32_t> tb(ninst + 1);
            comp_tiles = fg_batch_compact_tiles(ci.data(), ninst, tb.data());
            mem.release(d_tile_begin);
            d_tile_begin = static_cast<uint32_t*>(mem.get(sizeof(uint32_t) * (ninst + 1)));
            FG_ECUDA(cudaMemcpy(d_tile_begin, tb.data(), sizeof(uint32_t) * (ninst + 1), cudaMemcpyHostToDevice));
            comp_inst = static_cast<fg_batch_instance*>(mem.release_and_get(comp_inst, sizeof(fg_batch_instance) * ninst));
            FG_ECUDA(cudaMemcpy(comp_inst, ci.data(), sizeof(fg_batch_instance) * ninst, cudaMemcpyHostToDevice));
            mem.release(comp_ws);
            comp_ws_bytes = fg_compact_batched_workspace_size(comp_tiles, ninst);
            comp_ws = mem.get(comp_ws_bytes);
        }
        drop_graphs();
    }
    fg_batch_instance* comp_inst = nullptr;  // row segments, for the segmented compaction

    void build_tables(BFn& b) {
        for (int par = 0; par < 2; ++par) {
            auto T = std::make_unique<FunctionTables>();
            std::memset(T.get(), 0, sizeof(FunctionTables));
            std::vector<TableEntry> e;
            for (size_t v = 0; v < agent->variables.size(); ++v) {
                const Variable& var = agent->variables[v];
                e.push_back({fnv1a32(var.name), static_cast<char*>(cols[v][par]), var.bytes(), var.type_size, var.elements});
            }
            T->agent = make_table(e, "agent");
            if (b.out) {
                e.clear();
                for (size_t v = 0; v < b.out->msg->variables.size(); ++v) {
                    const Variable& var = b.out->msg->variables[v];
                    e.push_back({fnv1a32(var.name), static_cast<char*>(b.out->cols[v]), b.out->slot_bytes[v], var.type_size, var.elements});
                }
                T->msg_out = make_table(e, "message");
            }
            if (b.in) {
                e.clear();
                for (size_t v = 0; v < b.in->msg->variables.size(); ++v) {
                    const Variable& var = b.in->msg->variables[v];
                    e.push_back({fnv1a32(var.name), reinterpret_cast<char*>(b.in->records + b.in->field_word[v]),
                                 b.in->record_words * 4, var.type_size, var.elements});
                }
                T->msg_in = make_table(e, "message");
            }
            if (b.births) {
                e.clear();
                std::vector<TableEntry> d;
                size_t doff = 0;
                for (size_t v = 0; v < agent->variables.size(); ++v) {
                    const Variable& var = agent->variables[v];
                    e.push_back({fnv1a32(var.name), static_cast<char*>(b.birth_cols[v]), var.bytes(), var.type_size, var.elements});
                    d.push_back({fnv1a32(var.name), static_cast<char*>(b.birth_defaults) + doff, var.bytes(), var.type_size,
                                 var.elements});
                    doff = (doff + var.default_value.size() + 7) & ~size_t(7);
                }
                T->birth = make_table(e, "agent");
                T->birth_def = make_table(d, "agent");
            }
            e.clear();
            for (size_t i = 0; i < model->environment.size(); ++i) {
                const EnvProperty& p = model->environment[i];
                e.push_back({fnv1a32(p.name), reinterpret_cast<char*>(env_offset[i]), 0, p.type_size, p.elements});
            }
            T->env = make_table(e, "environment");
            b.tables[par] = std::move(T);
        }
    }

    // Grow the row segments to new_cap (device idle; count holds the exact counts).
    void relayout(const std::vector<uint32_t>& new_cap) {
        const std::vector<uint32_t> old_begin = row_begin;
        cap = new_cap;
        place_rows();
        for (size_t v = 0; v < cols.size(); ++v) {
            const size_t b = agent->variables[v].bytes();
            void* n0 = mem.get(b * total_rows);
            void* n1 = mem.get(b * total_rows);
            for (uint32_t k = 0; k < ninst; ++k)
                if (count[k])
                    FG_ECUDA(cudaMemcpyAsync(static_cast<char*>(n0) + b * row_begin[k],
                                             static_cast<const char*>(cols[v][parity]) + b * old_begin[k], b * count[k],
                                             cudaMemcpyDeviceToDevice, stream));
            FG_ECUDA(cudaStreamSynchronize(stream));
            mem.release(cols[v][0]);
            mem.release(cols[v][1]);
            cols[v] = {n0, n1};
        }
        parity = 0;
        layout_rows();
        ++relayouts;
    }

    // Before a step: every instance's population bound after it (its bound
    // entering the step, doubled per birth function) must fit its segment.
    // Bounds entering the step come from the newest population report that has
    // arrived (doubled per birth function and step since); if that is not
    // enough, wait for the exact counts, and grow the segments that still need it.
    void prepare_capacity(unsigned int step) {
        if (!birth_fns) return;
        const Report* known = nullptr;
        for (const auto& r : reports)
            if (r.used && r.step_after <= step && (!known || r.step_after > known->step_after) &&
                cudaEventQuery(r.ev) == cudaSuccess)
                known = &r;
        bool over = false;
        for (uint32_t k = 0; k < ninst; ++k) {
            uint64_t b = bound[k];
            if (known) {
                const int doublings = birth_fns * static_cast<int>(step - known->step_after);
                b = std::min<uint64_t>(b, static_cast<uint64_t>(known->host[k]) << std::min(doublings, 31));
            }
            bound[k] = b;
            over = over || (b << birth_fns) > cap[k];
        }
        if (!over) return;
        FG_ECUDA(cudaStreamSynchronize(stream));
        FG_ECUDA(cudaMemcpy(count.data(), d_counts, sizeof(uint32_t) * ninst, cudaMemcpyDeviceToHost));
        std::vector<uint32_t> want = cap;
        bool grow = false;
        for (uint32_t k = 0; k < ninst; ++k) {
            bound[k] = count[k];
            if ((bound[k] << birth_fns) > cap[k]) {
                want[k] = rows_for(count[k]);
                grow = true;
            }
        }
        if (grow) relayout(want);
    }

    // After a step: bounds advance by the births it may have had; the counts
    // are copied out for later bounds.
    void after_step(unsigned int step) {
        if (!death_or_birth) return;
        for (uint32_t k = 0; k < ninst; ++k) bound[k] = std::min<uint64_t>(bound[k], cap[k]);
        Report& r = reports[report_next];
        report_next = (report_next + 1) % reports.size();
        if (r.used) FG_ECUDA(cudaEventSynchronize(r.ev));
        FG_ECUDA(cudaMemcpyAsync(r.host, d_counts, sizeof(uint32_t) * ninst, cudaMemcpyDeviceToHost, stream));
        FG_ECUDA(cudaEventRecord(r.ev, stream));
        r.step_after = step + 1;
        r.used = true;
    }

    void enqueue_sort(BFn& b) {
        std::vector<fg_column> c(cols.size());
        for (size_t v = 0; v < cols.size(); ++v)
            c[v] = fg_column{cols[v][parity], cols[v][parity ^ 1], agent->variables[v].bytes()};
        auto col_of = [&](const char* n) -> const float* {
            for (size_t v = 0; v < agent->variables.size(); ++v)
                if (agent->variables[v].name == n) return static_cast<const float*>(cols[v][parity]);
            return nullptr;
        };
        FG_ECAPI(fg_spatial_sort_agents_batched(b.d_sort_inst, d_counts, ninst, total_rows, b.sort_buckets, col_of("x"),
                                                col_of("y"), b.in->dims == 3 ? col_of("z") : nullptr, b.in->dims,
                                                c.data(), static_cast<uint32_t>(c.size()), b.sort_ws, b.sort_ws_bytes,
                                                stream));
        parity ^= 1;
        kernels_per_step += 5;
    }

    void enqueue_build(BMsg& m, cudaStream_t st) {
        fg_record_desc rec;
        std::memset(&rec, 0, sizeof(rec));
        rec.words = m.record_words;
        for (size_t v = 0; v < m.cols.size(); ++v) {
            const uint32_t words = m.slot_bytes[v] / 4;
            for (uint32_t k = 0; k < words; ++k) {
                const uint32_t w = m.field_word[v] + k;
                rec.src[w] = static_cast<const uint32_t*>(m.cols[v]);
                rec.src_stride[w] = words;
                rec.src_word[w] = k;
            }
        }
        FG_ECAPI(fg_spatial_build_batched(m.d_inst, d_counts, ninst, total_rows, m.total_buckets,
                                          static_cast<const float*>(m.cols[0]), static_cast<const float*>(m.cols[1]),
                                          m.dims == 3 ? static_cast<const float*>(m.cols[2]) : nullptr, m.dims, nullptr,
                                          &rec, m.records, m.pbm, m.ws, m.ws_bytes, st));
        m.needs_build = false;
        kernels_per_step += 5;
    }

    // Stage neighbourhood windows when the instances holding most of the agents
    // have windows that fit the staging buffer.
    bool stage_pays(const BMsg& m) const {
        double fit = 0.0, all = 0.0;
        for (uint32_t k = 0; k < ninst && k < m.inst.size(); ++k) {
            const fg_spatial_grid& g = m.inst[k].grid;
            const double per_bin = static_cast<double>(count[k]) / std::max<uint32_t>(g.binCount, 1u);
            all += count[k];
            if (detail::stage_window_fits(g, per_bin, m.record_words, shape.block, shape.stage_bytes)) fit += count[k];
        }
        return all > 0.0 && fit >= 0.5 * all;
    }

    void launch_fn(BFn& b) {
        LaunchParams P;
        std::memset(&P, 0, sizeof(P));
        P.T = *b.tables[parity];
        P.max_n = total_rows;
        P.msg_out_enabled = b.out ? 1 : 0;
        unsigned int smem = 0;
        if (b.in && b.in->dims) {
            P.in_pbm = b.in->pbm;
            P.in_records = reinterpret_cast<const char*>(b.in->records);
            P.in_record_bytes = b.in->record_words * 4u;
            P.in_pay_mult = b.in->pay_mult;
            P.in_pay_shift = b.in->pay_shift;
            P.in_pay_stride = b.in->pay_stride;
            if (b.sort && shape.stage_bytes >= 1024u && stage_pays(*b.in)) {
                P.stage_bytes = (shape.stage_bytes + 15u) & ~15u;
                smem = P.stage_bytes + static_cast<unsigned int>(sizeof(StageHeader));
            }
        }
        P.death_flags = b.fn->has_agent_death ? b.death_flags : nullptr;
        P.birth_flags = b.births ? b.birth_flags : nullptr;
        P.birth_next_id = b.births ? d_next_ids : nullptr;
        P.d_step = d_misc;
        P.fn_uid = b.fn->uid;
        P.agent_hash = detail::fnv1a32(agent->name);
        P.state_hash = detail::fnv1a32(b.fn->initial_state);
        P.error = d_misc + 1;
        P.batch = b.d_rt;
        P.batch_counts = d_counts;
        P.batch_n = ninst;
        const uint32_t grid = std::min(total_rows / shape.block, static_cast<uint32_t>(sms) * shape.blocks_per_sm);
        const cudaError_t e = b.fn->launcher(P, std::max(1u, grid), shape.block, smem, stream, detail::pdl_enabled());
        if (e != cudaSuccess)
            THROW exception::CUDAError(format("Launch of agent function '%s' failed: %s", b.fn->name.c_str(), cudaGetErrorString(e)));
        kernels_per_step += 1;
        if (b.fn->has_agent_death || b.births) {
            // CUDAFatAgent::processDeath + CUDAAgentStateList::scatterNew of every
            // run at once, each in its own row segment
            std::vector<fg_column> c(cols.size()), bc(cols.size());
            for (size_t v = 0; v < cols.size(); ++v) {
                const uint32_t vb = agent->variables[v].bytes();
                c[v] = fg_column{cols[v][parity], cols[v][parity ^ 1], vb};
                bc[v] = fg_column{b.births ? b.birth_cols[v] : cols[v][parity], cols[v][parity ^ 1], vb};
            }
            FG_ECAPI(fg_compact_agents_batched(comp_inst, d_tile_begin, ninst, comp_tiles, total_rows, d_counts,
                                               b.fn->has_agent_death ? b.death_flags : nullptr,
                                               b.births ? b.birth_flags : nullptr, c.data(), bc.data(),
                                               static_cast<uint32_t>(c.size()), b.births ? id_col : -1, d_next_ids,
                                               comp_ws, comp_ws_bytes, stream));
            parity ^= 1;
            kernels_per_step += 2;
            for (uint32_t k = 0; b.births && k < ninst; ++k) bound[k] = std::min<uint64_t>(bound[k] * 2, 1ull << 33);
        }
    }

    bool sorts_at(unsigned int step) const {
        return agent->sort_period != 0 && step % agent->sort_period == 0;
    }

    void enqueue_step(unsigned int step) {
        kernels_per_step = 0;
        for (auto& m : msgs) m->needs_build = true;
        for (const auto& layer : model->layers)
            for (auto* fd : layer->functions)
                for (auto& b : fns) {
                    if (b.fn != fd) continue;
                    const bool do_sort = b.sort && sorts_at(step);
                    const bool do_build = b.in && b.in->dims && b.in->needs_build;
                    if (do_sort && do_build) {
                        FG_ECUDA(cudaEventRecord(fork_ev, stream));
                        FG_ECUDA(cudaStreamWaitEvent(side, fork_ev, 0));
                        enqueue_build(*b.in, side);
                        enqueue_sort(b);
                        FG_ECUDA(cudaEventRecord(join_ev, side));
                        FG_ECUDA(cudaStreamWaitEvent(stream, join_ev, 0));
                    } else {
                        if (do_sort) enqueue_sort(b);
                        if (do_build) enqueue_build(*b.in, stream);
                    }
                    launch_fn(b);
                    if (b.out) b.out->needs_build = true;
                }
        launch_kernel(pdl_enabled(), k_batch_step_increment, 1, 1, 0, stream, d_misc);
        kernels_per_step += 1;
    }

    // buffer flips of one step (sorts and compactions), replayed on the host for a cached graph
    int flips_at(unsigned int step) const {
        int f = 0;
        for (const auto& b : fns) {
            if (b.sort && sorts_at(step)) ++f;
            if (b.fn->has_agent_death || b.births) ++f;
        }
        return f;
    }

    double step_seconds = 0.0;  // device time from the first step's start to the last step's end

    AgentVector read_instance(uint32_t k) {
        AgentVector pop(AgentDescription(model, agent), 0);
        pop.setCountRaw(count[k]);
        for (size_t v = 0; v < cols.size(); ++v) {
            const size_t b = agent->variables[v].bytes();
            if (count[k])
                FG_ECUDA(cudaMemcpy(pop.columns()[v].data(), static_cast<char*>(cols[v][parity]) + b * row_begin[k],
                                    b * count[k], cudaMemcpyDeviceToHost));
        }
        return pop;
    }

    // One step: captured (or replayed) as a graph per buffer parity and sort decision.
    void issue_step(unsigned int s) {
        prepare_capacity(s);
        fg_tuning t{};
        t.scan_wide_min = shape.scan_wide_min;
        FG_ECAPI(fg_set_thread_tuning(&t));
        if (cfg.use_graphs) {
            const auto key = std::make_pair(parity, sorts_at(s));
            auto it = cache.find(key);
            if (it == cache.end()) {
                cudaGraph_t g;
                FG_ECUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
                try {
                    enqueue_step(s);
                } catch (...) {
                    cudaStreamEndCapture(stream, &g);
                    fg_set_thread_tuning(nullptr);
                    throw;
                }
                FG_ECUDA(cudaStreamEndCapture(stream, &g));
                cudaGraphExec_t ge;
                FG_ECUDA(cudaGraphInstantiate(&ge, g, 0));
                cudaGraphDestroy(g);
                it = cache.emplace(key, ge).first;
            } else {
                if (flips_at(s) & 1) parity ^= 1;
                for (const auto& b : fns)
                    if (b.births)
                        for (uint32_t k = 0; k < ninst; ++k) bound[k] = std::min<uint64_t>(bound[k] * 2, 1ull << 33);
            }
            FG_ECUDA(cudaGraphLaunch(it->second, stream));
            ++graph_launches;
        } else {
            enqueue_step(s);
        }
        fg_set_thread_tuning(nullptr);
        after_step(s);
    }

    // ---- autotuner
    // The size class of this batch: GPU, model, and powers of two of the
    // total agents, the runs and the agents per run.
    std::string size_class() const {
        cudaDeviceProp prop{};
        cudaGetDeviceProperties(&prop, cfg.device);
        uint64_t total = 0;
        for (uint32_t k = 0; k < ninst; ++k) total += count[k];
        auto lg = [](double v) { return static_cast<int>(std::lround(std::log2(std::max(v, 1.0)))); };
        return format("%s|%s|agents 2^%d|runs 2^%d|per run 2^%d", prop.name, model->name.c_str(), lg(double(total)),
                      lg(double(ninst)), lg(double(total) / std::max(1u, ninst)));
    }
    static std::string shape_json(const Shape& h) {
        return format("{\"block\": %u, \"blocks_per_sm\": %u, \"stage_bytes\": %u, \"scan_wide_min\": %u}", h.block,
                      h.blocks_per_sm, h.stage_bytes, h.scan_wide_min);
    }
    // The state every tuning trial starts from (agent columns, counts, ids, step).
    struct Snapshot {
        std::vector<void*> cols;
        int parity = 0;
        std::vector<uint32_t> counts, next_ids, misc;
    };
    Snapshot snapshot() {
        Snapshot sn;
        FG_ECUDA(cudaStreamSynchronize(stream));
        sn.parity = parity;
        for (size_t v = 0; v < cols.size(); ++v) {
            const size_t b = agent->variables[v].bytes() * static_cast<size_t>(total_rows);
            void* p = mem.get(b);
            FG_ECUDA(cudaMemcpy(p, cols[v][parity], b, cudaMemcpyDeviceToDevice));
            sn.cols.push_back(p);
        }
        sn.counts.resize(ninst);
        sn.next_ids.resize(ninst);
        sn.misc.resize(16);
        FG_ECUDA(cudaMemcpy(sn.counts.data(), d_counts, sizeof(uint32_t) * ninst, cudaMemcpyDeviceToHost));
        FG_ECUDA(cudaMemcpy(sn.next_ids.data(), d_next_ids, sizeof(uint32_t) * ninst, cudaMemcpyDeviceToHost));
        FG_ECUDA(cudaMemcpy(sn.misc.data(), d_misc, sizeof(uint32_t) * 16, cudaMemcpyDeviceToHost));
        return sn;
    }
    void restore(const Snapshot& sn) {
        FG_ECUDA(cudaStreamSynchronize(stream));
        parity = sn.parity;
        for (size_t v = 0; v < cols.size(); ++v)
            FG_ECUDA(cudaMemcpy(cols[v][parity], sn.cols[v], agent->variables[v].bytes() * static_cast<size_t>(total_rows),
                                cudaMemcpyDeviceToDevice));
        FG_ECUDA(cudaMemcpy(d_counts, sn.counts.data(), sizeof(uint32_t) * ninst, cudaMemcpyHostToDevice));
        FG_ECUDA(cudaMemcpy(d_next_ids, sn.next_ids.data(), sizeof(uint32_t) * ninst, cudaMemcpyHostToDevice));
        FG_ECUDA(cudaMemcpy(d_misc, sn.misc.data(), sizeof(uint32_t) * 16, cudaMemcpyHostToDevice));
        count = sn.counts;
    }
    // Device milliseconds per step of a shape: one step to capture, then
    // `steps` replays timed with CUDA events on the step's stream.
    double time_shape(const Shape& h, const Snapshot& sn, unsigned int steps) {
        restore(sn);
        shape = h;
        drop_graphs();
        issue_step(0);
        cudaEvent_t a, b;
        FG_ECUDA(cudaEventCreate(&a));
        FG_ECUDA(cudaEventCreate(&b));
        FG_ECUDA(cudaEventRecord(a, stream));
        for (unsigned int s = 1; s <= steps; ++s) issue_step(s);
        FG_ECUDA(cudaEventRecord(b, stream));
        FG_ECUDA(cudaEventSynchronize(b));
        float ms = 0.0f;
        FG_ECUDA(cudaEventElapsedTime(&ms, a, b));
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        return ms / steps;
    }
    // mode 1: the cache's shape for this size class (defaults if none);
    // mode 2: every candidate timed on this batch, the fastest kept and stored.
    void autotune(int mode, const std::string& path) {
        const std::string key = size_class();
        Shape def;
        def.stage_bytes = cfg.message_stage_bytes;
        shape = def;
        json::Value doc;
        bool have_doc = false;
        if (!path.empty()) {
            if (std::FILE* f = std::fopen(path.c_str(), "rb")) {
                std::string text;
                char buf[4096];
                size_t r;
                while ((r = std::fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, r);
                std::fclose(f);
                try {
                    doc = json::Parser(text).parse();
                    have_doc = doc.kind == json::Value::Object;
                } catch (const std::exception&) {
                    have_doc = false;
                }
            }
        }
        const json::Value* entries = have_doc ? doc.find("entries") : nullptr;
        const json::Value* hit = entries ? entries->find(key) : nullptr;
        if (mode == 1) {
            if (hit) {
                auto u = [&](const char* n, uint32_t d) {
                    const json::Value* v = hit->find(n);
                    return v ? static_cast<uint32_t>(v->uinteger()) : d;
                };
                shape.block = u("block", def.block);
                shape.blocks_per_sm = u("blocks_per_sm", def.blocks_per_sm);
                shape.stage_bytes = u("stage_bytes", def.stage_bytes);
                shape.scan_wide_min = u("scan_wide_min", def.scan_wide_min);
                if (shape.block != 32 && shape.block != 64 && shape.block != 128) shape.block = def.block;
                if (!shape.blocks_per_sm) shape.blocks_per_sm = def.blocks_per_sm;
            }
            tuning_json = format("{\"tuned\": %s, \"source\": \"%s\", \"key\": \"%s\", \"shape\": %s}",
                                 hit ? "true" : "false", hit ? "cache" : "default (no cache entry)", key.c_str(),
                                 shape_json(shape).c_str());
            return;
        }
        // measure
        if (death_or_birth) {  // trials would move populations: keep the defaults
            tuning_json = format("{\"tuned\": false, \"source\": \"default (birth/death model)\", \"key\": \"%s\", \"shape\": %s}",
                                 key.c_str(), shape_json(shape).c_str());
            return;
        }
        const Snapshot sn = snapshot();
        std::vector<Shape> cand;
        for (uint32_t block : {64u, 128u})
            for (uint32_t bps : {4u, 8u, 16u, 32u})
                for (uint32_t stage : {0u, def.stage_bytes})
                    for (uint32_t wide : {0u, 1u << 30}) {
                        Shape h;
                        h.block = block;
                        h.blocks_per_sm = bps;
                        h.stage_bytes = stage;
                        h.scan_wide_min = wide;
                        cand.push_back(h);
                    }
        const double def_ms = time_shape(def, sn, 3);
        double best_ms = def_ms;
        Shape best = def;
        std::string trials;
        for (const Shape& h : cand) {
            const double ms = time_shape(h, sn, 3);
            trials += format("%s[%u, %u, %u, %u, %.4f]", trials.empty() ? "" : ", ", h.block, h.blocks_per_sm,
                             h.stage_bytes, h.scan_wide_min, ms);
            if (ms < best_ms) {
                best_ms = ms;
                best = h;
            }
        }
        // the winner again, against the defaults, to confirm it (noise)
        const double again = time_shape(best, sn, 3);
        const double def_again = time_shape(def, sn, 3);
        if (again > def_again) {
            best = def;
            best_ms = def_again;
        } else {
            best_ms = again;
        }
        restore(sn);
        for (void* p : sn.cols) mem.release(p);
        drop_graphs();
        shape = best;
        tuning_json = format("{\"tuned\": true, \"source\": \"measured\", \"key\": \"%s\", \"shape\": %s, "
                             "\"step_ms\": %.4f, \"default_step_ms\": %.4f, \"trials\": "
                             "\"[block, blocks_per_sm, stage_bytes, scan_wide_min, ms]: %s\"}",
                             key.c_str(), shape_json(best).c_str(), best_ms, def_again, trials.c_str());
        if (path.empty()) return;
        // store: the file's other entries kept, this size class replaced
        std::vector<std::pair<std::string, std::string>> keep;
        if (entries)
            for (const auto& e : entries->fields) {
                if (e.first == key) continue;
                std::string body;
                for (const auto& f : e.second.fields)
                    body += format("%s\"%s\": %s", body.empty() ? "" : ", ", f.first.c_str(),
                                   f.second.kind == json::Value::String ? ("\"" + f.second.text + "\"").c_str()
                                                                        : f.second.text.c_str());
                keep.emplace_back(e.first, "{" + body + "}");
            }
        keep.emplace_back(key, format("{\"block\": %u, \"blocks_per_sm\": %u, \"stage_bytes\": %u, "
                                      "\"scan_wide_min\": %u, \"step_ms\": %.4f, \"default_step_ms\": %.4f}",
                                      best.block, best.blocks_per_sm, best.stage_bytes, best.scan_wide_min, best_ms,
                                      def_again));
        if (std::FILE* f = std::fopen(path.c_str(), "wb")) {
            std::fprintf(f, "{\n  \"about\": \"launch shapes of batched ensemble steps, measured by CUDAEnsemble's "
                            "autotuner (tuning = 2) per GPU, model and size class\",\n  \"entries\": {\n");
            for (size_t i = 0; i < keep.size(); ++i)
                std::fprintf(f, "    \"%s\": %s%s\n", keep[i].first.c_str(), keep[i].second.c_str(),
                             i + 1 < keep.size() ? "," : "");
            std::fprintf(f, "  }\n}\n");
            std::fclose(f);
        }
    }

    // Runs every plan to its step count; fills results[k].
    void run(std::vector<std::shared_ptr<AgentVector>>& results) {
        unsigned int max_steps = 0;
        for (const auto& p : plans) max_steps = std::max(max_steps, p.getSteps());
        results.assign(ninst, nullptr);
        cudaEvent_t t_begin = nullptr, t_end = nullptr;
        FG_ECUDA(cudaEventCreate(&t_begin));
        FG_ECUDA(cudaEventCreate(&t_end));
        FG_ECUDA(cudaEventRecord(t_begin, stream));
        for (unsigned int s = 0; s < max_steps; ++s) {
            issue_step(s);
            // runs that end here: read them back and drop them from later steps
            bool any = false;
            for (uint32_t k = 0; k < ninst; ++k) any = any || (plans[k].getSteps() == s + 1 && s + 1 < max_steps);
            if (any) {
                FG_ECUDA(cudaStreamSynchronize(stream));
                if (death_or_birth) FG_ECUDA(cudaMemcpy(count.data(), d_counts, sizeof(uint32_t) * ninst, cudaMemcpyDeviceToHost));
                for (uint32_t k = 0; k < ninst; ++k) {
                    if (plans[k].getSteps() != s + 1 || s + 1 >= max_steps) continue;
                    results[k] = std::make_shared<AgentVector>(read_instance(k));
                    count[k] = 0;
                    bound[k] = 0;
                    FG_ECUDA(cudaMemcpy(d_counts + k, &count[k], sizeof(uint32_t), cudaMemcpyHostToDevice));
                }
            }
        }
        FG_ECUDA(cudaEventRecord(t_end, stream));
        FG_ECUDA(cudaStreamSynchronize(stream));
        float ms = 0.0f;
        FG_ECUDA(cudaEventElapsedTime(&ms, t_begin, t_end));
        step_seconds = ms / 1000.0;
        cudaEventDestroy(t_begin);
        cudaEventDestroy(t_end);
        drop_graphs();
        uint32_t err[4];
        FG_ECUDA(cudaMemcpy(err, d_misc + 1, sizeof(err), cudaMemcpyDeviceToHost));
        if (err[0]) THROW exception::DeviceError(format("Device error %u in a batched ensemble step (name hash 0x%08x, row %u)", err[0], err[1], err[2]));
        if (death_or_birth) {
            uint32_t st = 0;
            FG_ECUDA(cudaMemcpy(&st, comp_ws, sizeof(st), cudaMemcpyDeviceToHost));
            if (st) THROW exception::DeviceError(format("Batched compaction reported status %d", static_cast<int>(st)));
            FG_ECUDA(cudaMemcpy(count.data(), d_counts, sizeof(uint32_t) * ninst, cudaMemcpyDeviceToHost));
        }
        for (uint32_t k = 0; k < ninst; ++k)
            if (!results[k]) results[k] = std::make_shared<AgentVector>(read_instance(k));
    }
};

struct EnsembleImpl {
    ModelDescription desc;
    CUDAEnsemble::EnsembleConfig cfg;
    std::vector<std::map<std::pair<std::string, std::string>, std::shared_ptr<AgentVector>>> results;
    double elapsed = 0.0;
    double step_seconds = 0.0;
    bool batched = false;
    unsigned int kernels_per_step = 0;
    unsigned long long graph_launches = 0;
    std::string tuning = "{\"tuned\": false}";
    explicit EnsembleImpl(const ModelDescription& d) : desc(d) {}
};

}  // namespace detail

CUDAEnsemble::CUDAEnsemble(const ModelDescription& model, int, const char**)
    : impl(std::make_unique<detail::EnsembleImpl>(model)) {}
CUDAEnsemble::~CUDAEnsemble() = default;
CUDAEnsemble::EnsembleConfig& CUDAEnsemble::Config() { return impl->cfg; }
double CUDAEnsemble::getEnsembleElapsedTime() const { return impl->elapsed; }
double CUDAEnsemble::getEnsembleStepTime() const { return impl->step_seconds; }
bool CUDAEnsemble::lastRunBatched() const { return impl->batched; }
const std::string& CUDAEnsemble::getTuning() const { return impl->tuning; }
unsigned int CUDAEnsemble::getKernelsPerStep() const { return impl->kernels_per_step; }
unsigned long long CUDAEnsemble::getGraphLaunches() const { return impl->graph_launches; }

unsigned int CUDAEnsemble::simulate(const RunPlanVector& plans) {
    const auto t0 = std::chrono::steady_clock::now();
    impl->results.assign(plans.size(), {});
    const auto& model = impl->desc.getData();
    for (const auto& p : plans)
        if (p.model() != model) THROW exception::InvalidArgument("RunPlan belongs to another model");
    unsigned int failures = 0;
    impl->step_seconds = 0.0;
    impl->batched = impl->cfg.batched && !plans.empty() && detail::batch_unsupported(*model).empty();
    if (impl->batched) {
        detail::BatchedSim b(model, plans, impl->cfg);
        b.setup();
        if (impl->cfg.tuning == 1 || impl->cfg.tuning == 2) b.autotune(impl->cfg.tuning, impl->cfg.tuning_cache);
        impl->tuning = b.tuning_json;
        std::vector<std::shared_ptr<AgentVector>> res;
        b.run(res);
        const auto key = std::make_pair(model->agents[0]->name, model->agents[0]->states[0]);
        for (size_t k = 0; k < plans.size(); ++k) impl->results[k][key] = res[k];
        impl->kernels_per_step = b.kernels_per_step;
        impl->step_seconds = b.step_seconds;
        impl->graph_launches = b.graph_launches;
    } else {
        // the plain path: one CUDASimulation per plan, one after another
        for (size_t k = 0; k < plans.size(); ++k) {
            const RunPlan& p = plans[k];
            try {
                CUDASimulation sim(impl->desc);
                sim.CUDAConfig().device_id = impl->cfg.device;
                sim.CUDAConfig().use_graphs = impl->cfg.use_graphs;
                sim.CUDAConfig().message_stage_bytes = impl->cfg.message_stage_bytes;
                sim.SimulationConfig().random_seed = p.getRandomSimulationSeed();
                sim.SimulationConfig().steps = p.getSteps();
                for (const auto& sp : p.spatial()) sim.setSpatialMessageBounds(sp.first, sp.second.min, sp.second.max, sp.second.radius);
                HostAPI::Environment env(sim.getImpl());
                for (const auto& pr : p.properties()) env.setRaw(pr.first, pr.second.data(), pr.second.size());
                for (const auto& pop : p.populations()) {
                    AgentVector copy = *pop.second;
                    sim.setPopulationData(copy, pop.first.second);
                }
                sim.simulate();
                for (double t : sim.getElapsedTimeSteps()) impl->step_seconds += t;
                for (const auto& a : model->agents)
                    for (const auto& st : a->states) {
                        auto out = std::make_shared<AgentVector>(AgentDescription(model, a.get()));
                        sim.getPopulationData(*out, st);
                        impl->results[k][{a->name, st}] = out;
                    }
            } catch (const exception::FLAMEGPUException&) {
                ++failures;
            }
        }
    }
    impl->elapsed = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return failures;
}

std::shared_ptr<const AgentVector> CUDAEnsemble::getPopulationView(unsigned int run, const std::string& agent,
                                                                    const std::string& state) const {
    if (run >= impl->results.size()) THROW exception::OutOfBoundsException(format("Run %u out of range", run));
    auto it = impl->results[run].find({agent, state});
    if (it == impl->results[run].end() || !it->second)
        THROW exception::InvalidAgentName(format("Run %u has no population of '%s' in state '%s'", run, agent.c_str(),
                                                  state.c_str()));
    return it->second;
}

void CUDAEnsemble::getPopulationData(unsigned int run, AgentVector& population, const std::string& state) const {
    if (run >= impl->results.size()) THROW exception::OutOfBoundsException(format("Run %u out of range", run));
    auto it = impl->results[run].find({population.getAgentName(), state});
    if (it == impl->results[run].end() || !it->second)
        THROW exception::InvalidAgentName(format("Run %u has no population of '%s' in state '%s'", run,
                                                  population.getAgentName().c_str(), state.c_str()));
    population = *it->second;
}

}  // namespace flamegpu
