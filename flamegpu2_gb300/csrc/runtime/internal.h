// Helpers shared by the simulation and ensemble runtimes (not installed).
#pragma once

#include <cstdint>
#include <vector>

#include "flamegpu/detail/device_types.cuh"

namespace flamegpu {
namespace detail {

struct TableEntry {
    uint32_t hash;
    char* ptr;
    uint32_t stride;
    uint32_t elem_bytes;
    uint32_t elements;
};

/** Collision-free multiplicative lookup table over the given variables:
 * slot = (hash * mult) >> shift; throws if no multiplier up to 64 slots works. */
VarTable make_table(const std::vector<TableEntry>& e, const char* what);

}  // namespace detail
}  // namespace flamegpu
