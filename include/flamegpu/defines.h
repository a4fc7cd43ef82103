#ifndef INCLUDE_FLAMEGPU_DEFINES_H_
#define INCLUDE_FLAMEGPU_DEFINES_H_
// Basic types of the public API (include/flamegpu/defines.h:10-46 in the reference).
#include <cstdint>

namespace flamegpu {
/** Agent id type; ids are unique per simulation, 0 means "not set". */
typedef unsigned int id_t;
/** Value of an id that has not been assigned. */
constexpr id_t ID_NOT_SET = 0;
/** Unsigned type of counts and indices. */
typedef unsigned int size_type;
/** Return value of an agent function (include/flamegpu/runtime/AgentFunction.cuh:19). */
enum AGENT_STATUS { ALIVE = 1, DEAD = 0 };
}  // namespace flamegpu

#define FLAMEGPU_DEVICE_FUNCTION __device__ __forceinline__
#define FLAMEGPU_HOST_DEVICE_FUNCTION __host__ FLAMEGPU_DEVICE_FUNCTION

#endif  // INCLUDE_FLAMEGPU_DEFINES_H_
