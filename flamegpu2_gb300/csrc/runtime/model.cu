// Model description and AgentVector implementations (host only).
#include <algorithm>
#include <map>
#include <set>

#include "flamegpu/model/ModelDescription.h"
#include "flamegpu/simulation/AgentVector.h"

namespace flamegpu {

using exception::format;

// ---------------------------------------------------------------- model

ModelDescription::ModelDescription(const std::string& name) : model(std::make_shared<detail::ModelData>()) {
    model->name = name;
}

AgentDescription ModelDescription::newAgent(const std::string& name) {
    detail::check_name(name, "Agent");
    if (model->agent(name)) THROW exception::InvalidAgentName(format("Model already has agent '%s'", name.c_str()));
    auto a = std::make_shared<detail::AgentData>();
    a->name = name;
    // every agent carries the internal id variable (defines.h:40, ID_VARIABLE_NAME "_id")
    const id_t unset = ID_NOT_SET;
    a->variables.push_back(detail::make_variable<id_t>("_id", &unset, 1));
    model->agents.push_back(a);
    return AgentDescription(model, a.get());
}

AgentDescription ModelDescription::Agent(const std::string& name) const {
    detail::AgentData* a = model->agent(name);
    if (!a) THROW exception::InvalidAgentName(format("Model has no agent '%s'", name.c_str()));
    return AgentDescription(model, a);
}

detail::MessageData* ModelDescription::new_message(const std::string& name, detail::MessageKind kind) {
    detail::check_name(name, "Message");
    if (model->message(name)) THROW exception::InvalidMessageName(format("Model already has message '%s'", name.c_str()));
    auto m = std::make_shared<detail::MessageData>();
    m->name = name;
    m->kind = kind;
    const float zero = 0.0f;
    if (kind == detail::MessageKind::Bucket) {
        // the key each message is output with (MessageBucketDevice.cuh:275-290)
        const int32_t none = 0;
        m->variables.push_back(detail::make_variable<int32_t>("___KEY", &none, 1));
    } else if (detail::array_dims(kind)) {
        // the index each message is output to (MessageArray2D.cu:155-158)
        const uint32_t none = 0;
        m->variables.push_back(detail::make_variable<uint32_t>("___INDEX", &none, 1));
    } else if (kind != detail::MessageKind::BruteForce) {
        m->variables.push_back(detail::make_variable<float>("x", &zero, 1));
        m->variables.push_back(detail::make_variable<float>("y", &zero, 1));
        if (kind == detail::MessageKind::Spatial3D) m->variables.push_back(detail::make_variable<float>("z", &zero, 1));
    }
    model->messages.push_back(m);
    return m.get();
}

LayerDescription ModelDescription::newLayer(const std::string& name) {
    std::string n = name.empty() ? format("_layer%zu", model->layers.size()) : name;
    for (const auto& l : model->layers)
        if (l->name == n) THROW exception::InvalidArgument(format("Model already has layer '%s'", n.c_str()));
    auto l = std::make_shared<detail::LayerData>();
    l->name = n;
    model->layers.push_back(l);
    return LayerDescription(model, l.get());
}

LayerDescription ModelDescription::Layer(flamegpu::size_type index) const {
    if (index >= model->layers.size()) THROW exception::OutOfBoundsException(format("Layer %u out of range", index));
    return LayerDescription(model, model->layers[index].get());
}

LayerDescription ModelDescription::Layer(const std::string& name) const {
    for (const auto& l : model->layers)
        if (l->name == name) return LayerDescription(model, l.get());
    THROW exception::InvalidArgument(format("Model has no layer '%s'", name.c_str()));
}

void ModelDescription::generateLayers() {
    // Dependency graph -> layers (src/flamegpu/model/DependencyGraph.cpp:89-180):
    // a function's layer is one more than the deepest layer of its dependencies;
    // functions in a layer keep the order in which they were reached.
    std::map<detail::AgentFunctionData*, int> depth;
    std::vector<detail::AgentFunctionData*> all;
    for (const auto& a : model->agents)
        for (const auto& f : a->functions) all.push_back(f.get());
    std::set<detail::AgentFunctionData*> reachable;
    std::vector<detail::AgentFunctionData*> stack(model->execution_roots.begin(), model->execution_roots.end());
    // children: functions that depend on f
    std::map<detail::AgentFunctionData*, std::vector<detail::AgentFunctionData*>> children;
    for (auto* f : all)
        for (auto* d : f->dependencies) children[d].push_back(f);
    while (!stack.empty()) {
        auto* f = stack.back();
        stack.pop_back();
        if (!reachable.insert(f).second) continue;
        for (auto* c : children[f]) stack.push_back(c);
    }
    std::function<int(detail::AgentFunctionData*, int)> depth_of = [&](detail::AgentFunctionData* f, int guard) -> int {
        if (guard > 10000) THROW exception::InvalidDependencyGraph("Dependency graph has a cycle");
        auto it = depth.find(f);
        if (it != depth.end()) return it->second;
        int d = 0;
        for (auto* p : f->dependencies) d = std::max(d, depth_of(p, guard + 1) + 1);
        depth[f] = d;
        return d;
    };
    int max_d = -1;
    for (auto* f : all)
        if (reachable.count(f)) max_d = std::max(max_d, depth_of(f, 0));
    model->layers.clear();
    for (int d = 0; d <= max_d; ++d) {
        auto l = std::make_shared<detail::LayerData>();
        l->name = format("_generated%d", d);
        for (auto* f : all)
            if (reachable.count(f) && depth[f] == d) l->functions.push_back(f);
        model->layers.push_back(l);
    }
}

// ---------------------------------------------------------------- agent

void AgentDescription::add_variable(detail::Variable v) {
    detail::check_name(v.name, "Agent variable");
    if (v.name[0] == '_') THROW exception::ReservedName(format("Agent variable '%s' starts with '_'", v.name.c_str()));
    if (agent->find(v.name))
        THROW exception::InvalidAgentVar(format("Agent '%s' already has variable '%s'", agent->name.c_str(), v.name.c_str()));
    agent->variables.push_back(std::move(v));
}

void AgentDescription::newState(const std::string& state) {
    detail::check_name(state, "State");
    if (!agent->explicit_states) {
        agent->states.clear();
        agent->explicit_states = true;
        agent->initial_state = state;
        for (auto& f : agent->functions) {
            f->initial_state = state;
            f->end_state = state;
        }
    }
    if (std::find(agent->states.begin(), agent->states.end(), state) != agent->states.end())
        THROW exception::InvalidAgentState(format("Agent '%s' already has state '%s'", agent->name.c_str(), state.c_str()));
    agent->states.push_back(state);
}

void AgentDescription::setInitialState(const std::string& state) {
    if (std::find(agent->states.begin(), agent->states.end(), state) == agent->states.end())
        THROW exception::InvalidAgentState(format("Agent '%s' has no state '%s'", agent->name.c_str(), state.c_str()));
    agent->initial_state = state;
}

std::type_index AgentDescription::getVariableType(const std::string& name) const {
    const detail::Variable* v = agent->find(name);
    if (!v) THROW exception::InvalidAgentVar(format("Agent '%s' has no variable '%s'", agent->name.c_str(), name.c_str()));
    return v->type;
}

flamegpu::size_type AgentDescription::getVariableLength(const std::string& name) const {
    const detail::Variable* v = agent->find(name);
    if (!v) THROW exception::InvalidAgentVar(format("Agent '%s' has no variable '%s'", agent->name.c_str(), name.c_str()));
    return v->elements;
}

// ---------------------------------------------------------------- function

namespace {
// The device message type a function must name for a message of this kind.
std::type_index message_type_of(detail::MessageKind k) {
    switch (k) {
        case detail::MessageKind::Spatial3D: return std::type_index(typeid(MessageSpatial3D));
        case detail::MessageKind::Spatial2D: return std::type_index(typeid(MessageSpatial2D));
        case detail::MessageKind::Array1D: return std::type_index(typeid(MessageArray));
        case detail::MessageKind::Array2D: return std::type_index(typeid(MessageArray2D));
        case detail::MessageKind::Array3D: return std::type_index(typeid(MessageArray3D));
        case detail::MessageKind::Bucket: return std::type_index(typeid(MessageBucket));
        default: return std::type_index(typeid(MessageBruteForce));
    }
}
}  // namespace

void AgentFunctionDescription::setMessageInput(const std::string& name) {
    detail::MessageData* m = model->message(name);
    if (!m) THROW exception::InvalidMessageName(format("Model has no message '%s'", name.c_str()));
    const std::type_index want = message_type_of(m->kind);
    if (fn->msg_in_type != want)
        THROW exception::InvalidMessageType(format("Function '%s' input message type does not match message '%s'",
                                                   fn->name.c_str(), name.c_str()));
    if (fn->message_output == name)
        THROW exception::InvalidMessageName(format("Function '%s' cannot read and write message '%s'", fn->name.c_str(), name.c_str()));
    fn->message_input = name;
}

void AgentFunctionDescription::setMessageOutput(const std::string& name) {
    detail::MessageData* m = model->message(name);
    if (!m) THROW exception::InvalidMessageName(format("Model has no message '%s'", name.c_str()));
    const std::type_index want = message_type_of(m->kind);
    if (fn->msg_out_type != want)
        THROW exception::InvalidMessageType(format("Function '%s' output message type does not match message '%s'",
                                                   fn->name.c_str(), name.c_str()));
    if (fn->message_input == name)
        THROW exception::InvalidMessageName(format("Function '%s' cannot read and write message '%s'", fn->name.c_str(), name.c_str()));
    fn->message_output = name;
}

void AgentFunctionDescription::setAgentOutput(const std::string& agent_name, const std::string& state) {
    detail::AgentData* a = model->agent(agent_name);
    if (!a) THROW exception::InvalidAgentName(format("Model has no agent '%s'", agent_name.c_str()));
    const std::string st = state.empty() ? a->initial_state : state;
    if (std::find(a->states.begin(), a->states.end(), st) == a->states.end())
        THROW exception::InvalidAgentState(format("Agent '%s' has no state '%s'", agent_name.c_str(), st.c_str()));
    fn->agent_output = agent_name;
    fn->agent_output_state = st;
}

void AgentFunctionDescription::setAgentOutput(const AgentDescription& agent, const std::string& state) {
    setAgentOutput(agent.getName(), state);
}

void AgentFunctionDescription::setInitialState(const std::string& s) {
    const auto& st = fn->parent->states;
    if (std::find(st.begin(), st.end(), s) == st.end())
        THROW exception::InvalidAgentState(format("Agent '%s' has no state '%s'", fn->parent->name.c_str(), s.c_str()));
    fn->initial_state = s;
}

void AgentFunctionDescription::setEndState(const std::string& s) {
    const auto& st = fn->parent->states;
    if (std::find(st.begin(), st.end(), s) == st.end())
        THROW exception::InvalidAgentState(format("Agent '%s' has no state '%s'", fn->parent->name.c_str(), s.c_str()));
    fn->end_state = s;
}

// ---------------------------------------------------------------- layer

void LayerDescription::add(detail::AgentFunctionData* f) {
    for (auto* g : layer->functions) {
        if (g == f) THROW exception::InvalidAgentFunc(format("Layer already contains function '%s'", f->name.c_str()));
        // LayerDescription.h:152-220: two functions of one agent state may not share a layer
        if (g->parent == f->parent && (g->initial_state == f->initial_state || g->end_state == f->end_state))
            THROW exception::InvalidAgentFunc(format("Functions '%s' and '%s' of agent '%s' act on the same state in one layer",
                                                     g->name.c_str(), f->name.c_str(), f->parent->name.c_str()));
    }
    layer->functions.push_back(f);
}

void LayerDescription::addAgentFunction(const std::string& agent_name, const std::string& function_name) {
    detail::AgentData* a = model->agent(agent_name);
    if (!a) THROW exception::InvalidAgentName(format("Model has no agent '%s'", agent_name.c_str()));
    for (const auto& f : a->functions)
        if (f->name == function_name) {
            add(f.get());
            return;
        }
    THROW exception::InvalidAgentFunc(format("Agent '%s' has no function '%s'", agent_name.c_str(), function_name.c_str()));
}

// ---------------------------------------------------------------- environment

void EnvironmentDescription::add(const std::string& name, std::type_index t, uint32_t size, uint32_t n, const void* v,
                                 bool c) {
    detail::check_name(name, "Environment property");
    if (model->property(name) || model->macro_property(name))
        THROW exception::InvalidEnvProperty(format("Environment already has property '%s'", name.c_str()));
    detail::EnvProperty p;
    p.name = name;
    p.type = t;
    p.type_size = size;
    p.elements = n;
    p.value.resize(static_cast<size_t>(size) * n);
    std::memcpy(p.value.data(), v, p.value.size());
    p.is_const = c;
    model->environment.push_back(std::move(p));
}

void EnvironmentDescription::add_macro(const std::string& name, std::type_index t, uint32_t size, const uint32_t (&dims)[4]) {
    detail::check_name(name, "Environment macro property");
    if (model->property(name) || model->macro_property(name))
        THROW exception::InvalidEnvProperty(format("Environment already has property '%s'", name.c_str()));
    uint64_t n = 1;
    for (uint32_t d : dims) n *= d;
    if (n * size > (1ull << 34))
        THROW exception::InvalidEnvProperty(format("Environment macro property '%s' is too large", name.c_str()));
    detail::MacroProperty p;
    p.name = name;
    p.type = t;
    p.type_size = size;
    for (int a = 0; a < 4; ++a) p.dims[a] = dims[a];
    model->macro_environment.push_back(std::move(p));
}

const detail::EnvProperty* EnvironmentDescription::find(const std::string& name, const std::type_info& t,
                                                        size_t size) const {
    const detail::EnvProperty* p = model->property(name);
    if (!p) THROW exception::InvalidEnvProperty(format("Environment has no property '%s'", name.c_str()));
    if (p->type != std::type_index(t) || p->type_size != size)
        THROW exception::InvalidEnvPropertyType(format("Environment property '%s' has another type", name.c_str()));
    return p;
}

// ---------------------------------------------------------------- AgentVector

AgentVector::AgentVector(const AgentDescription& a, flamegpu::size_type n) : model(a.getModel()), agent(a.getData()) {
    cols.resize(agent->variables.size());
    resize(n);
}

AgentVector::Agent AgentVector::at(flamegpu::size_type i) {
    if (i >= count) THROW exception::OutOfBoundsException(format("Agent index %u out of range (%u agents)", i, count));
    return Agent(this, i);
}

void AgentVector::reserve(flamegpu::size_type n) {
    for (size_t v = 0; v < cols.size(); ++v) cols[v].reserve(static_cast<size_t>(n) * agent->variables[v].bytes());
}

void AgentVector::resize(flamegpu::size_type n) {
    for (size_t v = 0; v < cols.size(); ++v) {
        const detail::Variable& var = agent->variables[v];
        const size_t b = var.bytes();
        const size_t old = cols[v].size() / (b ? b : 1);
        cols[v].resize(static_cast<size_t>(n) * b);
        for (size_t i = old; i < n; ++i) std::memcpy(cols[v].data() + i * b, var.default_value.data(), b);
    }
    count = n;
}

void AgentVector::push_back() { resize(count + 1); }

AgentVector AgentVector::row(flamegpu::size_type i) const {
    if (i >= count) THROW exception::OutOfBoundsException(format("Agent index %u out of range (%u agents)", i, count));
    AgentVector r(AgentDescription(model, agent), 0);
    for (size_t v = 0; v < cols.size(); ++v) {
        const size_t b = agent->variables[v].bytes();
        r.cols[v].assign(cols[v].begin() + static_cast<std::ptrdiff_t>(i * b),
                         cols[v].begin() + static_cast<std::ptrdiff_t>((i + 1) * b));
    }
    r.count = 1;
    return r;
}

void AgentVector::insert(flamegpu::size_type pos, flamegpu::size_type n, const AgentInstance& a) {
    const AgentVector& src = a.values();
    if (src.agent != agent)
        THROW exception::InvalidArgument(format("AgentInstance of agent '%s' inserted into a vector of agent '%s'",
                                                src.agent->name.c_str(), agent->name.c_str()));
    if (pos > count) THROW exception::OutOfBoundsException(format("Insert position %u past the %u agents", pos, count));
    for (size_t v = 0; v < cols.size(); ++v) {
        const detail::Variable& var = agent->variables[v];
        const size_t b = var.bytes();
        std::vector<char> one(src.cols[v].begin(), src.cols[v].begin() + static_cast<std::ptrdiff_t>(b));
        if (var.name == "_id") std::memset(one.data(), 0, b);  // ID_NOT_SET: a fresh id when set
        std::vector<char> block;
        block.reserve(static_cast<size_t>(n) * b);
        for (flamegpu::size_type k = 0; k < n; ++k) block.insert(block.end(), one.begin(), one.end());
        cols[v].insert(cols[v].begin() + static_cast<std::ptrdiff_t>(static_cast<size_t>(pos) * b), block.begin(), block.end());
    }
    count += n;
}

void AgentVector::erase(flamegpu::size_type first, flamegpu::size_type last) {
    if (first > last || last > count)
        THROW exception::OutOfBoundsException(
            format("AgentVector::erase: [%u, %u) is not within the %u agents", first, last, count));
    if (first == last) return;
    for (size_t v = 0; v < cols.size(); ++v) {
        const size_t b = agent->variables[v].bytes();
        char* d = cols[v].data();
        std::memmove(d + first * b, d + last * b, (count - last) * b);
        cols[v].resize(static_cast<size_t>(count - (last - first)) * b);
    }
    count -= last - first;
}

void AgentVector::setCountRaw(flamegpu::size_type n) {
    for (size_t v = 0; v < cols.size(); ++v) cols[v].resize(static_cast<size_t>(n) * agent->variables[v].bytes());
    count = n;
}

size_t AgentVector::columnIndex(const std::string& name) const {
    for (size_t v = 0; v < agent->variables.size(); ++v)
        if (agent->variables[v].name == name) return v;
    THROW exception::InvalidAgentVar(format("Agent '%s' has no variable '%s'", agent->name.c_str(), name.c_str()));
}

char* AgentVector::column(const std::string& name) { return cols[columnIndex(name)].data(); }
const char* AgentVector::column(const std::string& name) const { return cols[columnIndex(name)].data(); }

char* AgentVector::ptr(const std::string& name, const std::type_info& t, size_t size, flamegpu::size_type i,
                       flamegpu::size_type element, flamegpu::size_type expect_len) {
    const size_t c = columnIndex(name);
    const detail::Variable& v = agent->variables[c];
    if (v.type != std::type_index(t) || v.type_size != size)
        THROW exception::InvalidVarType(format("Variable '%s' of agent '%s' has another type", name.c_str(), agent->name.c_str()));
    if (expect_len && expect_len != v.elements)
        THROW exception::InvalidVarType(format("Variable '%s' has %u elements, %u requested", name.c_str(), v.elements, expect_len));
    if (element >= v.elements)
        THROW exception::OutOfBoundsException(format("Element %u of variable '%s' out of range", element, name.c_str()));
    if (i >= count) THROW exception::OutOfBoundsException(format("Agent index %u out of range (%u agents)", i, count));
    return cols[c].data() + static_cast<size_t>(i) * v.bytes() + static_cast<size_t>(element) * v.type_size;
}

}  // namespace flamegpu
