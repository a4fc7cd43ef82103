#ifndef INCLUDE_FLAMEGPU_MODEL_MODELDESCRIPTION_H_
#define INCLUDE_FLAMEGPU_MODEL_MODELDESCRIPTION_H_
// Model description API: ModelDescription, AgentDescription,
// AgentFunctionDescription, message descriptions, LayerDescription and
// EnvironmentDescription with the reference's names and signatures
// (include/flamegpu/model/ModelDescription.h:83-273, AgentDescription.h:209-310,
// AgentFunctionDescription.h:190-334, LayerDescription.h:152-220,
// include/flamegpu/runtime/messaging/MessageSpatial3D/MessageSpatial3DHost.h).
// Descriptions are cheap handles onto shared model data, as in the reference.
#include <array>
#include <cmath>
#include <cstring>
#include <functional>
#include <limits>
#include <map>
#include <memory>
#include <set>
#include <string>
#include <type_traits>
#include <typeindex>
#include <vector>

#include "flamegpu/defines.h"
#include "flamegpu/exception/FLAMEGPUException.h"
#include "flamegpu/runtime/AgentFunction.cuh"

namespace flamegpu {

class ModelDescription;
class AgentDescription;
class AgentFunctionDescription;
class LayerDescription;
class EnvironmentDescription;
class HostAPI;

typedef void (*FLAMEGPU_HOST_FUNCTION_POINTER)(HostAPI* api);
/** What an exit condition returns (include/flamegpu/defines.h CONDITION_RESULT). */
enum CONDITION_RESULT { CONTINUE, EXIT };
typedef CONDITION_RESULT (*FLAMEGPU_EXIT_CONDITION_POINTER)(HostAPI* api);

namespace detail {

enum class MessageKind { BruteForce = 1, Spatial2D = 2, Spatial3D = 3, Array1D = 4, Array2D = 5, Array3D = 6, Bucket = 7 };
// the array message kinds' dimension count (0: not an array)
inline int array_dims(MessageKind k) {
    return k == MessageKind::Array1D ? 1 : k == MessageKind::Array2D ? 2 : k == MessageKind::Array3D ? 3 : 0;
}

struct Variable {
    std::string name;
    std::type_index type = std::type_index(typeid(void));
    uint32_t type_size = 0;
    uint32_t elements = 1;
    std::vector<char> default_value;  // type_size * elements bytes
    uint32_t bytes() const { return type_size * elements; }
};

struct AgentData;
struct MessageData;

struct AgentFunctionData {
    std::string name;
    AgentData* parent = nullptr;
    AgentFunctionLauncher launcher = nullptr;
    AgentFunctionLauncher condition = nullptr;  // FLAMEGPU_AGENT_FUNCTION_CONDITION kernel, or null
    std::type_index msg_in_type = std::type_index(typeid(void));
    std::type_index msg_out_type = std::type_index(typeid(void));
    std::string message_input, message_output;
    bool message_output_optional = false;
    std::string agent_output, agent_output_state;
    bool has_agent_death = false;
    std::string initial_state, end_state;
    std::vector<AgentFunctionData*> dependencies;
    uint32_t uid = 0;
};

struct AgentData {
    std::string name;
    std::vector<Variable> variables;  // _id first
    std::vector<std::shared_ptr<AgentFunctionData>> functions;
    std::vector<std::string> states{"default"};
    std::string initial_state = "default";
    bool explicit_states = false;
    unsigned int sort_period = 1;  // AgentData.cpp:17
    const Variable* find(const std::string& n) const {
        for (const auto& v : variables)
            if (v.name == n) return &v;
        return nullptr;
    }
};

struct MessageData {
    std::string name;
    MessageKind kind = MessageKind::BruteForce;
    std::vector<Variable> variables;
    float radius = std::numeric_limits<float>::quiet_NaN();
    float min[3] = {std::numeric_limits<float>::quiet_NaN(), std::numeric_limits<float>::quiet_NaN(),
                    std::numeric_limits<float>::quiet_NaN()};
    float max[3] = {std::numeric_limits<float>::quiet_NaN(), std::numeric_limits<float>::quiet_NaN(),
                    std::numeric_limits<float>::quiet_NaN()};
    bool persistent = false;
    uint32_t dims[3] = {0, 0, 0};  // array messages: length along each dimension (0: unset)
    // bucket messages: keys lower .. upper, both inclusive (upper unset: INT32_MAX)
    int32_t bucket_lower = 0;
    int32_t bucket_upper = std::numeric_limits<int32_t>::max();
    const Variable* find(const std::string& n) const {
        for (const auto& v : variables)
            if (v.name == n) return &v;
        return nullptr;
    }
};

struct LayerData {
    std::string name;
    std::vector<AgentFunctionData*> functions;
    std::vector<FLAMEGPU_HOST_FUNCTION_POINTER> host_functions;
};

struct EnvProperty {
    std::string name;
    std::type_index type = std::type_index(typeid(void));
    uint32_t type_size = 0;
    uint32_t elements = 1;
    std::vector<char> value;
    bool is_const = false;
};

/** An environment macro property: a zero-initialised array of up to four
 *  dimensions that agent functions update atomically
 *  (include/flamegpu/model/EnvironmentDescription.h newMacroProperty). */
struct MacroProperty {
    std::string name;
    std::type_index type = std::type_index(typeid(void));
    uint32_t type_size = 0;
    uint32_t dims[4] = {1, 1, 1, 1};
    uint32_t elements() const { return dims[0] * dims[1] * dims[2] * dims[3]; }
};

struct ModelData {
    std::string name;
    std::vector<MacroProperty> macro_environment;
    std::vector<std::shared_ptr<AgentData>> agents;
    std::vector<std::shared_ptr<MessageData>> messages;
    std::vector<std::shared_ptr<LayerData>> layers;
    std::vector<EnvProperty> environment;
    std::vector<FLAMEGPU_HOST_FUNCTION_POINTER> init_functions, step_functions, exit_functions;
    std::vector<FLAMEGPU_EXIT_CONDITION_POINTER> exit_conditions;
    std::vector<AgentFunctionData*> execution_roots;
    uint32_t next_fn_uid = 1;
    AgentData* agent(const std::string& n) const {
        for (const auto& a : agents)
            if (a->name == n) return a.get();
        return nullptr;
    }
    MessageData* message(const std::string& n) const {
        for (const auto& m : messages)
            if (m->name == n) return m.get();
        return nullptr;
    }
    EnvProperty* property(const std::string& n) {
        for (auto& p : environment)
            if (p.name == n) return &p;
        return nullptr;
    }
    MacroProperty* macro_property(const std::string& n) {
        for (auto& p : macro_environment)
            if (p.name == n) return &p;
        return nullptr;
    }
};

template <typename F>
void add_host_fn(std::vector<F>& list, F fn, const char* kind) {
    for (F g : list)
        if (g == fn)
            THROW exception::InvalidHostFunc(exception::format("This %s function has already been added", kind));
    list.push_back(fn);
}

template <typename T>
Variable make_variable(const std::string& name, const T* def, uint32_t elements) {
    Variable v;
    v.name = name;
    v.type = std::type_index(typeid(T));
    v.type_size = sizeof(T);
    v.elements = elements;
    v.default_value.resize(sizeof(T) * elements);
    std::memcpy(v.default_value.data(), def, sizeof(T) * elements);
    return v;
}

inline void check_name(const std::string& n, const char* what) {
    if (n.empty()) THROW exception::InvalidArgument(exception::format("%s name may not be empty", what));
}

}  // namespace detail

// ---------------------------------------------------------------- messages

/** Base description of a message list: its variables (MessageBruteForce::Description). */
class MessageBruteForce::Description {
 public:
    explicit Description(std::shared_ptr<detail::ModelData> m, detail::MessageData* d) : model(std::move(m)), data(d) {}
    template <typename T>
    void newVariable(const std::string& name) {
        detail::check_name(name, "Message variable");
        if (!name.empty() && name[0] == '_')
            THROW exception::ReservedName(exception::format("Message variable '%s' starts with '_'", name.c_str()));
        if (data->find(name))
            THROW exception::InvalidMessageVar(exception::format("Message '%s' already has variable '%s'",
                                                                 data->name.c_str(), name.c_str()));
        T zero{};
        data->variables.push_back(detail::make_variable<T>(name, &zero, 1));
    }
    template <typename T, flamegpu::size_type N>
    void newVariable(const std::string& name) {
        detail::check_name(name, "Message variable");
        if (data->find(name))
            THROW exception::InvalidMessageVar(exception::format("Message '%s' already has variable '%s'",
                                                                 data->name.c_str(), name.c_str()));
        std::array<T, N> zero{};
        data->variables.push_back(detail::make_variable<T>(name, zero.data(), N));
    }
    void setPersistent(bool p) { data->persistent = p; }
    bool getPersistent() const { return data->persistent; }
    std::string getName() const { return data->name; }
    bool hasVariable(const std::string& name) const { return data->find(name) != nullptr; }
    flamegpu::size_type getVariablesCount() const { return static_cast<flamegpu::size_type>(data->variables.size()); }
    detail::MessageData* getData() const { return data; }

 protected:
    std::shared_ptr<detail::ModelData> model;
    detail::MessageData* data;
};

/** MessageSpatial2D::Description (MessageSpatial2DHost.h): radius and 2D bounds; x, y implicit. */
class MessageSpatial2D::Description : public MessageBruteForce::Description {
 public:
    using MessageBruteForce::Description::Description;
    void setRadius(float r) {
        if (!(r > 0.0f)) THROW exception::InvalidArgument(exception::format("Spatial radius must be > 0, %g given", r));
        data->radius = r;
    }
    void setMin(float x, float y) {
        check_min(0, x);
        check_min(1, y);
        data->min[0] = x;
        data->min[1] = y;
    }
    void setMax(float x, float y) {
        check_max(0, x);
        check_max(1, y);
        data->max[0] = x;
        data->max[1] = y;
    }
    void setMinX(float v) { check_min(0, v); data->min[0] = v; }
    void setMinY(float v) { check_min(1, v); data->min[1] = v; }
    void setMaxX(float v) { check_max(0, v); data->max[0] = v; }
    void setMaxY(float v) { check_max(1, v); data->max[1] = v; }
    float getRadius() const { return data->radius; }
    float getMinX() const { return data->min[0]; }
    float getMinY() const { return data->min[1]; }
    float getMaxX() const { return data->max[0]; }
    float getMaxY() const { return data->max[1]; }

 protected:
    void check_min(int a, float v) const {
        if (!std::isnan(data->max[a]) && !(v < data->max[a]))
            THROW exception::InvalidArgument(exception::format("Spatial min (%g) must be below max (%g)", v, data->max[a]));
    }
    void check_max(int a, float v) const {
        if (!std::isnan(data->min[a]) && !(v > data->min[a]))
            THROW exception::InvalidArgument(exception::format("Spatial max (%g) must be above min (%g)", v, data->min[a]));
    }
};

/** MessageSpatial3D::Description (MessageSpatial3DHost.h:225-240): x, y, z implicit. */
class MessageSpatial3D::Description : public MessageSpatial2D::Description {
 public:
    using MessageSpatial2D::Description::Description;
    void setMin(float x, float y, float z) {
        MessageSpatial2D::Description::setMin(x, y);
        check_min(2, z);
        data->min[2] = z;
    }
    void setMax(float x, float y, float z) {
        MessageSpatial2D::Description::setMax(x, y);
        check_max(2, z);
        data->max[2] = z;
    }
    void setMinZ(float v) { check_min(2, v); data->min[2] = v; }
    void setMaxZ(float v) { check_max(2, v); data->max[2] = v; }
    float getMinZ() const { return data->min[2]; }
    float getMaxZ() const { return data->max[2]; }
};

/** MessageArray::Description (MessageArrayHost.h): a list of setLength() messages,
 *  each output to the index its agent sets. */
class MessageArray::Description : public MessageBruteForce::Description {
 public:
    using MessageBruteForce::Description::Description;
    void setLength(flamegpu::size_type len) {
        if (len == 0) THROW exception::InvalidArgument("Array message length must be above zero");
        data->dims[0] = len;
        data->dims[1] = data->dims[2] = 1;
    }
    flamegpu::size_type getLength() const { return data->dims[0]; }
};

/** MessageArray2D::Description (MessageArray2DHost.h, MessageArray2D.cu:139-148). */
class MessageArray2D::Description : public MessageBruteForce::Description {
 public:
    using MessageBruteForce::Description::Description;
    void setDimensions(flamegpu::size_type x, flamegpu::size_type y) {
        if (x == 0 || y == 0) THROW exception::InvalidArgument("All dimensions must be above zero in array2D message");
        data->dims[0] = x;
        data->dims[1] = y;
        data->dims[2] = 1;
    }
    void setDimensions(const std::array<flamegpu::size_type, 2>& d) { setDimensions(d[0], d[1]); }
    std::array<flamegpu::size_type, 2> getDimensions() const { return {data->dims[0], data->dims[1]}; }
    flamegpu::size_type getDimX() const { return data->dims[0]; }
    flamegpu::size_type getDimY() const { return data->dims[1]; }
};

/** MessageArray3D::Description (MessageArray3DHost.h). */
class MessageArray3D::Description : public MessageBruteForce::Description {
 public:
    using MessageBruteForce::Description::Description;
    void setDimensions(flamegpu::size_type x, flamegpu::size_type y, flamegpu::size_type z) {
        if (x == 0 || y == 0 || z == 0) THROW exception::InvalidArgument("All dimensions must be above zero in array3D message");
        data->dims[0] = x;
        data->dims[1] = y;
        data->dims[2] = z;
    }
    void setDimensions(const std::array<flamegpu::size_type, 3>& d) { setDimensions(d[0], d[1], d[2]); }
    std::array<flamegpu::size_type, 3> getDimensions() const { return {data->dims[0], data->dims[1], data->dims[2]}; }
    flamegpu::size_type getDimX() const { return data->dims[0]; }
    flamegpu::size_type getDimY() const { return data->dims[1]; }
    flamegpu::size_type getDimZ() const { return data->dims[2]; }
};

/** MessageBucket::Description (MessageBucketHost.h:180-245, MessageBucket.cu:190-215):
 *  integer keys lowerBound .. upperBound, both inclusive. */
class MessageBucket::Description : public MessageBruteForce::Description {
 public:
    using MessageBruteForce::Description::Description;
    void setLowerBound(int32_t min) {
        if (data->bucket_upper != std::numeric_limits<int32_t>::max() && min >= data->bucket_upper)
            THROW exception::InvalidArgument(exception::format("Bucket lower bound %d must be below the upper bound %d", min,
                                                               data->bucket_upper));
        data->bucket_lower = min;
    }
    void setUpperBound(int32_t max) {
        if (max <= data->bucket_lower)
            THROW exception::InvalidArgument(exception::format("Bucket upper bound %d must be above the lower bound %d", max,
                                                               data->bucket_lower));
        data->bucket_upper = max;
    }
    void setBounds(int32_t min, int32_t max) {
        if (max <= min)
            THROW exception::InvalidArgument(exception::format("Bucket upper bound %d must be above the lower bound %d", max, min));
        data->bucket_lower = min;
        data->bucket_upper = max;
    }
    int32_t getLowerBound() const { return data->bucket_lower; }
    int32_t getUpperBound() const { return data->bucket_upper; }
};

// --------------------------------------------------------- agent functions

class AgentFunctionDescription {
 public:
    AgentFunctionDescription(std::shared_ptr<detail::ModelData> m, detail::AgentFunctionData* f)
        : model(std::move(m)), fn(f) {}
    void setMessageInput(const std::string& message_name);
    void setMessageInput(const MessageBruteForce::Description& message) { setMessageInput(message.getName()); }
    void setMessageOutput(const std::string& message_name);
    void setMessageOutput(const MessageBruteForce::Description& message) { setMessageOutput(message.getName()); }
    void setMessageOutputOptional(bool optional) { fn->message_output_optional = optional; }
    void setAgentOutput(const std::string& agent_name, const std::string& state = "");
    void setAgentOutput(const AgentDescription& agent, const std::string& state = "");
    void setAllowAgentDeath(bool allow) { fn->has_agent_death = allow; }
    void setInitialState(const std::string& s);
    void setEndState(const std::string& s);
    void dependsOn(const AgentFunctionDescription& other) { fn->dependencies.push_back(other.fn); }
    /** AgentFunctionDescription::setFunctionCondition (AgentFunctionDescription.h:263-271):
     *  only agents for which the FLAMEGPU_AGENT_FUNCTION_CONDITION holds run the function. */
    template <typename C>
    void setFunctionCondition(C) { fn->condition = C::launcher(); }
    bool hasFunctionCondition() const { return fn->condition != nullptr; }
    std::string getName() const { return fn->name; }
    std::string getMessageInputName() const { return fn->message_input; }
    std::string getMessageOutputName() const { return fn->message_output; }
    bool getMessageOutputOptional() const { return fn->message_output_optional; }
    bool getAllowAgentDeath() const { return fn->has_agent_death; }
    bool hasMessageInput() const { return !fn->message_input.empty(); }
    bool hasMessageOutput() const { return !fn->message_output.empty(); }
    bool hasAgentOutput() const { return !fn->agent_output.empty(); }
    std::string getInitialState() const { return fn->initial_state; }
    std::string getEndState() const { return fn->end_state; }
    detail::AgentFunctionData* getData() const { return fn; }

 private:
    std::shared_ptr<detail::ModelData> model;
    detail::AgentFunctionData* fn;
};

class AgentDescription {
 public:
    AgentDescription(std::shared_ptr<detail::ModelData> m, detail::AgentData* a) : model(std::move(m)), agent(a) {}
    template <typename T>
    void newVariable(const std::string& name, T default_value = {}) {
        add_variable(detail::make_variable<T>(name, &default_value, 1));
    }
    template <typename T, flamegpu::size_type N>
    void newVariable(const std::string& name, const std::array<T, N>& default_value = {}) {
        add_variable(detail::make_variable<T>(name, default_value.data(), N));
    }
    template <typename F>
    AgentFunctionDescription newFunction(const std::string& name, F) {
        detail::check_name(name, "Agent function");
        for (const auto& f : agent->functions)
            if (f->name == name)
                THROW exception::InvalidAgentFunc(exception::format("Agent '%s' already has function '%s'",
                                                                    agent->name.c_str(), name.c_str()));
        auto f = std::make_shared<detail::AgentFunctionData>();
        f->name = name;
        f->parent = agent;
        f->launcher = F::launcher();
        f->msg_in_type = F::inType();
        f->msg_out_type = F::outType();
        f->initial_state = agent->initial_state;
        f->end_state = agent->initial_state;
        f->uid = model->next_fn_uid++;
        agent->functions.push_back(f);
        return AgentFunctionDescription(model, f.get());
    }
    AgentFunctionDescription Function(const std::string& name) const {
        for (const auto& f : agent->functions)
            if (f->name == name) return AgentFunctionDescription(model, f.get());
        THROW exception::InvalidAgentFunc(exception::format("Agent '%s' has no function '%s'", agent->name.c_str(), name.c_str()));
    }
    void newState(const std::string& state);
    void setInitialState(const std::string& state);
    void setSortPeriod(unsigned int period) { agent->sort_period = period; }
    unsigned int getSortPeriod() const { return agent->sort_period; }
    std::string getName() const { return agent->name; }
    bool hasVariable(const std::string& name) const { return agent->find(name) != nullptr; }
    flamegpu::size_type getVariablesCount() const { return static_cast<flamegpu::size_type>(agent->variables.size() - 1); }
    std::type_index getVariableType(const std::string& name) const;
    flamegpu::size_type getVariableLength(const std::string& name) const;
    detail::AgentData* getData() const { return agent; }
    const std::shared_ptr<detail::ModelData>& getModel() const { return model; }

 private:
    void add_variable(detail::Variable v);
    std::shared_ptr<detail::ModelData> model;
    detail::AgentData* agent;
};

class LayerDescription {
 public:
    LayerDescription(std::shared_ptr<detail::ModelData> m, detail::LayerData* l) : model(std::move(m)), layer(l) {}
    template <typename F>
    void addAgentFunction(const F&) {
        const detail::AgentFunctionLauncher l = F::launcher();
        for (const auto& a : model->agents)
            for (const auto& f : a->functions)
                if (f->launcher == l) {
                    add(f.get());
                    return;
                }
        THROW exception::InvalidAgentFunc("Agent function passed to addAgentFunction() is not part of the model");
    }
    void addAgentFunction(const AgentFunctionDescription& f) { add(f.getData()); }
    void addAgentFunction(const std::string& agent_name, const std::string& function_name);
    /** LayerDescription::addHostFunction (LayerDescription.h:120-127): a function
     *  may be in several layers, once per layer. */
    void addHostFunction(FLAMEGPU_HOST_FUNCTION_POINTER fn) { detail::add_host_fn(layer->host_functions, fn, "host layer"); }
    std::string getName() const { return layer->name; }
    flamegpu::size_type getAgentFunctionsCount() const { return static_cast<flamegpu::size_type>(layer->functions.size()); }

 private:
    void add(detail::AgentFunctionData* f);
    std::shared_ptr<detail::ModelData> model;
    detail::LayerData* layer;
};

class EnvironmentDescription {
 public:
    explicit EnvironmentDescription(std::shared_ptr<detail::ModelData> m) : model(std::move(m)) {}
    template <typename T>
    void newProperty(const std::string& name, T value, bool isConst = false) {
        add(name, std::type_index(typeid(T)), sizeof(T), 1, &value, isConst);
    }
    template <typename T, flamegpu::size_type N>
    void newProperty(const std::string& name, const std::array<T, N>& value, bool isConst = false) {
        add(name, std::type_index(typeid(T)), sizeof(T), N, value.data(), isConst);
    }
    template <typename T>
    T getProperty(const std::string& name) const {
        const detail::EnvProperty* p = find(name, typeid(T), sizeof(T));
        T v;
        std::memcpy(&v, p->value.data(), sizeof(T));
        return v;
    }
    template <typename T, flamegpu::size_type N>
    std::array<T, N> getProperty(const std::string& name) const {
        const detail::EnvProperty* p = find(name, typeid(T), sizeof(T));
        std::array<T, N> v;
        std::memcpy(v.data(), p->value.data(), sizeof(T) * N);
        return v;
    }
    template <typename T>
    T setProperty(const std::string& name, T value) {
        detail::EnvProperty* p = const_cast<detail::EnvProperty*>(find(name, typeid(T), sizeof(T)));
        T old;
        std::memcpy(&old, p->value.data(), sizeof(T));
        std::memcpy(p->value.data(), &value, sizeof(T));
        return old;
    }
    bool hasProperty(const std::string& name) const { return model->property(name) != nullptr; }
    /** EnvironmentDescription::newMacroProperty<T, I, J, K, W>
     *  (include/flamegpu/model/EnvironmentDescription.h:271-285): a property of
     *  I x J x K x W elements, zero at the start of a simulation, written by
     *  agent functions with atomic operations and by host functions. Its name
     *  is not also a plain property's (the two share one device table). */
    template <typename T, flamegpu::size_type I = 1, flamegpu::size_type J = 1, flamegpu::size_type K = 1,
              flamegpu::size_type W = 1>
    void newMacroProperty(const std::string& name) {
        static_assert(I > 0 && J > 0 && K > 0 && W > 0, "macro property dimensions must be positive");
        const uint32_t dims[4] = {I, J, K, W};
        add_macro(name, std::type_index(typeid(T)), sizeof(T), dims);
    }
    bool hasMacroProperty(const std::string& name) const { return model->macro_property(name) != nullptr; }

 private:
    void add_macro(const std::string& name, std::type_index t, uint32_t size, const uint32_t (&dims)[4]);
    void add(const std::string& name, std::type_index t, uint32_t size, uint32_t n, const void* v, bool c);
    const detail::EnvProperty* find(const std::string& name, const std::type_info& t, size_t size) const;
    std::shared_ptr<detail::ModelData> model;
};

class ModelDescription {
 public:
    explicit ModelDescription(const std::string& name);
    AgentDescription newAgent(const std::string& name);
    AgentDescription Agent(const std::string& name) const;
    template <typename MsgType>
    typename MsgType::Description newMessage(const std::string& name) {
        detail::MessageData* d = new_message(name, kind_of<MsgType>());
        return typename MsgType::Description(model, d);
    }
    /** ModelDescription::newMessage(name) (include/flamegpu/model/ModelDescription.h:110): a brute-force message list. */
    MessageBruteForce::Description newMessage(const std::string& name) { return newMessage<MessageBruteForce>(name); }
    template <typename MsgType>
    typename MsgType::Description Message(const std::string& name) const {
        detail::MessageData* d = model->message(name);
        if (!d || d->kind != kind_of<MsgType>())
            THROW exception::InvalidMessageName(exception::format("Model has no message '%s' of that type", name.c_str()));
        return typename MsgType::Description(model, d);
    }
    LayerDescription newLayer(const std::string& name = "");
    LayerDescription Layer(flamegpu::size_type index) const;
    LayerDescription Layer(const std::string& name) const;
    EnvironmentDescription Environment() const { return EnvironmentDescription(model); }
    /** ModelDescription::addInitFunction / addStepFunction / addExitFunction /
     *  addExitCondition (ModelDescription.h:150-200): each runs in the order
     *  added; adding one twice is InvalidHostFunc. Exit conditions run after
     *  the step functions of every step; the first to return EXIT ends
     *  simulate() after that step (with SimulationConfig().steps == 0 a
     *  simulation runs until one does). */
    void addInitFunction(FLAMEGPU_HOST_FUNCTION_POINTER fn) { detail::add_host_fn(model->init_functions, fn, "init"); }
    void addStepFunction(FLAMEGPU_HOST_FUNCTION_POINTER fn) { detail::add_host_fn(model->step_functions, fn, "step"); }
    void addExitFunction(FLAMEGPU_HOST_FUNCTION_POINTER fn) { detail::add_host_fn(model->exit_functions, fn, "exit"); }
    void addExitCondition(FLAMEGPU_EXIT_CONDITION_POINTER fn) { detail::add_host_fn(model->exit_conditions, fn, "exit condition"); }
    void addExecutionRoot(const AgentFunctionDescription& f) { model->execution_roots.push_back(f.getData()); }
    /** Layers from the dependency graph (src/flamegpu/model/DependencyGraph.cpp:89-180). */
    void generateLayers();
    std::string getName() const { return model->name; }
    flamegpu::size_type getLayersCount() const { return static_cast<flamegpu::size_type>(model->layers.size()); }
    flamegpu::size_type getAgentsCount() const { return static_cast<flamegpu::size_type>(model->agents.size()); }
    flamegpu::size_type getMessagesCount() const { return static_cast<flamegpu::size_type>(model->messages.size()); }
    const std::shared_ptr<detail::ModelData>& getData() const { return model; }

 private:
    template <typename MsgType>
    static detail::MessageKind kind_of() {
        if constexpr (std::is_same_v<MsgType, MessageSpatial3D>) return detail::MessageKind::Spatial3D;
        else if constexpr (std::is_same_v<MsgType, MessageSpatial2D>) return detail::MessageKind::Spatial2D;
        else if constexpr (std::is_same_v<MsgType, MessageArray>) return detail::MessageKind::Array1D;
        else if constexpr (std::is_same_v<MsgType, MessageArray2D>) return detail::MessageKind::Array2D;
        else if constexpr (std::is_same_v<MsgType, MessageArray3D>) return detail::MessageKind::Array3D;
        else if constexpr (std::is_same_v<MsgType, MessageBucket>) return detail::MessageKind::Bucket;
        else return detail::MessageKind::BruteForce;
    }
    detail::MessageData* new_message(const std::string& name, detail::MessageKind kind);
    std::shared_ptr<detail::ModelData> model;
};

}  // namespace flamegpu

#define FLAMEGPU_INIT_FUNCTION(name) void name(flamegpu::HostAPI* FLAMEGPU)
#define FLAMEGPU_STEP_FUNCTION(name) void name(flamegpu::HostAPI* FLAMEGPU)
#define FLAMEGPU_EXIT_FUNCTION(name) void name(flamegpu::HostAPI* FLAMEGPU)
#define FLAMEGPU_HOST_FUNCTION(name) void name(flamegpu::HostAPI* FLAMEGPU)
#define FLAMEGPU_EXIT_CONDITION(name) flamegpu::CONDITION_RESULT name(flamegpu::HostAPI* FLAMEGPU)

#endif  // INCLUDE_FLAMEGPU_MODEL_MODELDESCRIPTION_H_
