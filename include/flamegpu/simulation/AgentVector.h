#ifndef INCLUDE_FLAMEGPU_SIMULATION_AGENTVECTOR_H_
#define INCLUDE_FLAMEGPU_SIMULATION_AGENTVECTOR_H_
// Host-side population container (include/flamegpu/simulation/AgentVector.h in
// the reference): a vector of agents of one AgentDescription, accessed through
// AgentVector::Agent views. Stored as one byte column per variable (the same
// struct-of-arrays layout the device uses), including the internal _id.
#include <array>
#include <cstring>
#include <memory>
#include <string>
#include <typeindex>
#include <vector>

#include "flamegpu/model/ModelDescription.h"

namespace flamegpu {

class AgentInstance;

class AgentVector {
 public:
    class Agent {
     public:
        Agent(AgentVector* v, flamegpu::size_type i) : vec(v), index(i) {}
        template <typename T>
        void setVariable(const std::string& name, T value) {
            if (!name.empty() && name[0] == '_')
                THROW exception::ReservedName(exception::format("Variable '%s' is internal", name.c_str()));
            std::memcpy(vec->ptr(name, typeid(T), sizeof(T), index, 0), &value, sizeof(T));
        }
        template <typename T, flamegpu::size_type N>
        void setVariable(const std::string& name, const std::array<T, N>& value) {
            for (flamegpu::size_type k = 0; k < N; ++k)
                std::memcpy(vec->ptr(name, typeid(T), sizeof(T), index, k, N), &value[k], sizeof(T));
        }
        template <typename T, flamegpu::size_type N = 0>
        void setVariable(const std::string& name, flamegpu::size_type element, T value) {
            std::memcpy(vec->ptr(name, typeid(T), sizeof(T), index, element), &value, sizeof(T));
        }
        template <typename T>
        T getVariable(const std::string& name) const {
            T v;
            std::memcpy(&v, vec->ptr(name, typeid(T), sizeof(T), index, 0), sizeof(T));
            return v;
        }
        template <typename T, flamegpu::size_type N>
        std::array<T, N> getVariable(const std::string& name) const {
            std::array<T, N> v;
            for (flamegpu::size_type k = 0; k < N; ++k)
                std::memcpy(&v[k], vec->ptr(name, typeid(T), sizeof(T), index, k, N), sizeof(T));
            return v;
        }
        template <typename T, flamegpu::size_type N = 0>
        T getVariable(const std::string& name, flamegpu::size_type element) const {
            T v;
            std::memcpy(&v, vec->ptr(name, typeid(T), sizeof(T), index, element), sizeof(T));
            return v;
        }
        id_t getID() const {
            id_t v;
            std::memcpy(&v, vec->ptr("_id", typeid(id_t), sizeof(id_t), index, 0), sizeof(id_t));
            return v;
        }
        flamegpu::size_type getIndex() const { return index; }

     private:
        friend class AgentInstance;
        AgentVector* vec;
        flamegpu::size_type index;
    };

    class iterator {
     public:
        iterator(AgentVector* v, flamegpu::size_type i) : vec(v), index(i) {}
        Agent operator*() const { return Agent(vec, index); }
        iterator& operator++() {
            ++index;
            return *this;
        }
        bool operator!=(const iterator& o) const { return index != o.index; }
        bool operator==(const iterator& o) const { return index == o.index; }

     private:
        AgentVector* vec;
        flamegpu::size_type index;
    };

    explicit AgentVector(const AgentDescription& agent, flamegpu::size_type count = 0);
    /** One agent's values (of row i) as a vector of one agent. */
    AgentVector row(flamegpu::size_type i) const;
    flamegpu::size_type size() const { return count; }
    bool empty() const { return count == 0; }
    Agent operator[](flamegpu::size_type i) { return Agent(this, i); }
    Agent at(flamegpu::size_type i);
    Agent front() { return at(0); }
    Agent back() { return at(count - 1); }
    void push_back();
    /** Append a copy of `agent` (it gets a fresh id when the vector is set). */
    void push_back(const AgentInstance& agent) { insert(count, 1, agent); }
    /** Insert n copies of `agent` before pos (AgentVector::insert,
     *  AgentVector.h:376-420); the copies have no id until the vector is set,
     *  when they get fresh ones. */
    void insert(flamegpu::size_type pos, flamegpu::size_type n, const AgentInstance& agent);
    void insert(flamegpu::size_type pos, const AgentInstance& agent) { insert(pos, 1, agent); }
    void pop_back() { resize(count ? count - 1 : 0); }
    /** Remove the agent at pos, or the agents of [first, last); the agents after them move up in order. */
    void erase(flamegpu::size_type pos) { erase(pos, pos + 1); }
    void erase(flamegpu::size_type first, flamegpu::size_type last);
    void resize(flamegpu::size_type n);
    void reserve(flamegpu::size_type n);
    void clear() { resize(0); }
    iterator begin() { return iterator(this, 0); }
    iterator end() { return iterator(this, count); }
    std::string getAgentName() const { return agent->name; }
    const detail::AgentData* getAgentData() const { return agent; }

    // Raw column access (struct of arrays), used by CUDASimulation.
    char* column(const std::string& name);
    const char* column(const std::string& name) const;
    size_t columnIndex(const std::string& name) const;
    std::vector<std::vector<char>>& columns() { return cols; }
    const std::vector<std::vector<char>>& columns() const { return cols; }
    void setCountRaw(flamegpu::size_type n);

 private:
    char* ptr(const std::string& name, const std::type_info& t, size_t size, flamegpu::size_type i,
              flamegpu::size_type element, flamegpu::size_type expect_len = 0);
    std::shared_ptr<detail::ModelData> model;
    detail::AgentData* agent;
    std::vector<std::vector<char>> cols;
    flamegpu::size_type count = 0;
};

/**
 * AgentInstance (include/flamegpu/simulation/AgentInstance.h): one agent's
 * variables outside a population, made with the agent's default values or
 * copied from an agent of a vector; AgentVector::insert / push_back copy it in.
 */
class AgentInstance {
 public:
    explicit AgentInstance(const AgentDescription& agent) : one(agent, 1) {}
    AgentInstance(const AgentVector::Agent& agent) : one(agent.vec->row(agent.index)) {}  // NOLINT: implicit as in the reference
    template <typename T>
    void setVariable(const std::string& name, T value) { one[0].setVariable<T>(name, value); }
    template <typename T, flamegpu::size_type N>
    void setVariable(const std::string& name, const std::array<T, N>& value) { one[0].setVariable<T, N>(name, value); }
    template <typename T>
    T getVariable(const std::string& name) const { return const_cast<AgentVector&>(one)[0].getVariable<T>(name); }
    template <typename T, flamegpu::size_type N>
    std::array<T, N> getVariable(const std::string& name) const {
        return const_cast<AgentVector&>(one)[0].getVariable<T, N>(name);
    }
    const AgentVector& values() const { return one; }

 private:
    AgentVector one;
};

}  // namespace flamegpu

#endif  // INCLUDE_FLAMEGPU_SIMULATION_AGENTVECTOR_H_
