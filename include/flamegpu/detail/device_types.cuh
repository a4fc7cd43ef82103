#ifndef INCLUDE_FLAMEGPU_DETAIL_DEVICE_TYPES_CUH_
#define INCLUDE_FLAMEGPU_DETAIL_DEVICE_TYPES_CUH_
// Types shared by the host runtime and the header-only device API.
//
// Variable lookup. The reference resolves getVariable("x") at run time with a
// 512-slot open-addressing table of FNV-1a hashes copied into shared memory by
// every block (include/flamegpu/runtime/detail/curve/Curve.cuh:21-84,
// DeviceCurve.cuh:111-122,342-374). Here the FNV-1a hash of a name literal is
// computed at compile time (consteval), and the host builds, per agent
// function, a collision-free multiplicative hash over that function's own
// variables: slot = (hash * mult) >> shift. A lookup is one multiply, one
// shift and one read of a read-only table that the compiler hoists out of
// loops; no shared memory, no probing.
#include <cstdint>
#include <string_view>

#include "flamegpu/defines.h"
#include "flamegpu/detail/spatial_keys.cuh"
#include "flamegpu_gb300/fg_capi.h"

namespace flamegpu {
namespace detail {

/** 32-bit FNV-1a, the hash the reference's curve uses for names (Curve.cuh:66-84). */
constexpr uint32_t fnv1a32(const char* s, unsigned n) {
    uint32_t h = 2166136261u;
    for (unsigned i = 0; i < n && s[i]; ++i) {
        h ^= static_cast<uint8_t>(s[i]);
        h *= 16777619u;
    }
    return h;
}
inline uint32_t fnv1a32(const std::string_view s) { return fnv1a32(s.data(), static_cast<unsigned>(s.size())); }

/** A variable name given as a string literal, hashed at compile time. */
struct VarName {
    uint32_t hash;
    bool reserved;  // starts with '_' (internal variables such as _id)
    template <unsigned N>
    __host__ __device__ consteval VarName(const char (&s)[N]) : hash(fnv1a32(s, N - 1)), reserved(s[0] == '_') {}
};

constexpr int kMaxVarSlots = 64;

struct VarSlot {
    char* ptr;            // element 0 of the column (or of field 0 in a record)
    uint32_t stride;      // bytes between consecutive rows
    uint32_t hash;        // FNV-1a of the name (0 = empty slot)
    uint32_t elem_bytes;  // sizeof(T) of one element
    uint32_t elements;    // array length (1 for scalars)
};

struct VarTable {
    uint32_t mult;
    uint32_t shift;
    uint32_t count;
    uint32_t pad;
    VarSlot slot[kMaxVarSlots];
};

__host__ __device__ inline uint32_t table_slot(uint32_t mult, uint32_t shift, uint32_t hash) {
    return (hash * mult) >> shift;
}

/** Read-only tables of one agent function launch (kernel parameters). */
struct FunctionTables {
    VarTable agent;      // the agent's own variables (SoA columns)
    VarTable msg_out;    // output message list (unsorted SoA columns)
    VarTable msg_in;     // input message list (sorted records, or SoA for brute force)
    VarTable birth;      // agent_out staging rows (SoA, indexed by parent)
    VarTable birth_def;  // default value of each agent_out variable (ptr -> value bytes)
    VarTable env;        // environment properties (ptr -> value bytes)
};

/** One instance of a batched launch (device array, LaunchParams::batch). Rows
 * [row_begin, row_begin + row_capacity) of every column belong to it; its
 * input messages' PBM is pbm + in_bucket_begin. */
struct BatchInstanceRT {
    uint32_t row_begin;
    uint32_t row_capacity;
    uint32_t in_bucket_begin;
    uint32_t step_offset;   // the instance's step = launch step - step_offset
    fg_spatial_grid in_grid;
    const char* env;        // the instance's environment buffer
    uint64_t seed;
};

/** What an agent function's block needs about the instance it runs for; in
 * shared memory, filled at the start of every grid-stride round. */
struct InstanceCtx {
    fg_spatial_grid grid;   // message input grid
    const uint32_t* pbm;    // PBM of the instance's input messages
    uint32_t pbm_alloc;     // PBM entries readable from pbm
    uint32_t step;
    const char* env;        // environment buffer
    uint64_t seed;
    uint32_t row_begin;     // first row of the instance
    uint32_t count;         // agents in the instance
    uint32_t inst;          // index of the instance in its batch (0 for a single simulation)
};

/** Header of the shared-memory staging window of one block (spatial input). */
struct StageHeader {
    uint32_t rec_lo;   // first staged sorted message index
    uint32_t rec_n;    // staged messages (0 = window empty)
    uint32_t pbm_lo;   // first staged PBM entry
    uint32_t pbm_n;    // staged PBM entries
    uint32_t rec_bytes;
    uint32_t phase;    // mbarrier phase of the next wait
    uint32_t pad[1];   // bytes expected by the current window's copies
    uint32_t off;      // non-zero once a wait gave up: this block stages nothing more
    unsigned long long mbar;
    unsigned long long pad2[3];
};
static_assert(sizeof(StageHeader) == 64, "staging header is 64 bytes");

/** Device error codes recorded in LaunchParams::error[0]. */
enum DeviceErrorCode : uint32_t {
    kDevOk = 0,
    kDevUnknownVariable = 1,
    kDevTypeMismatch = 2,
    kDevArrayIndex = 3,
    kDevWrapOutOfBounds = 4,
    kDevWrapIncompatible = 5,
    kDevDeathNotEnabled = 6,
    kDevBirthNotEnabled = 7,
    kDevReservedName = 8,
    kDevUnsupported = 9,
    kDevMessageOutNotEnabled = 10,
    kDevStageTimeout = 11,
    kDevRandomRange = 12,
    kDevArrayMessage = 13,
    kDevBucketMessage = 14,
    kDevMacroConflict = 15,
};

/** Kernel parameters of one agent function launch (passed __grid_constant__).
 * The lookup tables travel in the parameter space: table reads are
 * constant-bank loads the compiler hoists and shares between accesses. */
struct LaunchParams {
    FunctionTables T;
    uint32_t max_n;              // capacity of the agent list (grid sizing bound)
    const uint32_t* d_n;         // agents in the list (device)
    // Agent function condition (single simulations): rows [0, *d_first) failed
    // the condition and are not run (their death / birth flags are written as
    // alive / not born); rows [*d_first, n) are, and their message rows start
    // at 0. Null: every row runs.
    const uint32_t* d_first;
    uint32_t* cond_fail;         // condition kernels: 1 per row that fails, 0 past the population
    // message output
    uint32_t* msg_out_valid;     // per-row output flag (lists with an optional output), or null
    uint32_t* msg_out_count;     // set to the message count by the launch
    const uint32_t* msg_out_base;  // messages already in the list this step (append), or null (truncate)
    uint32_t* msg_out_filled;    // set to 1 by a launch that ran over at least one agent (null: none)
    int msg_out_enabled;
    int msg_out_always;          // every running agent outputs (not optional): valid = 1
    // message input
    fg_spatial_grid in_grid;     // spatial metadata (MessageSpatial3D::MetaData)
    const uint32_t* in_pbm;      // partition boundary matrix, binCount + 1 entries
    const uint32_t* in_count;    // messages in the input list
    const char* in_records;      // sorted message records (spatial input)
    uint32_t in_record_bytes;    // bytes per record (multiple of 16)
    // record layout: location words first, then each other variable at byte
    // 4 * dims + slot * in_pay_stride, slot = table_slot(in_pay_mult, in_pay_shift, hash)
    uint32_t in_pay_mult, in_pay_shift, in_pay_stride;
    uint32_t in_pbm_alloc;       // PBM entries readable (multiple of 4, >= binCount + 1)
    uint32_t in_dims[3];         // array message input: dimensions (1 past the last used)
    uint32_t out_dims[3];        // array message output: dimensions
    int32_t in_key_lo, in_key_hi;    // bucket message input: keys [lo, hi) (PBM in in_pbm)
    int32_t out_key_lo, out_key_hi;  // bucket message output: keys [lo, hi)
    uint32_t stage_bytes;        // shared memory for staging neighbour records (0 = off)
    // birth / death
    uint32_t* birth_flags;       // 1 where agent_out was used, 2 if its id was also claimed (null if disabled)
    uint32_t* birth_next_id;     // next id of the output agent (agent_out.getID() claims from it; one per instance in a batch)
    uint32_t* death_flags;       // ALIVE / DEAD per agent (null if death disabled)
    uint32_t* alive_count;       // the survivors are added here, one atomic per block (null: not counted)
    // step data
    const uint32_t* d_step;      // step counter
    uint64_t seed;               // simulation random seed
    uint32_t fn_uid;             // unique id of this agent function (random streams)
    uint32_t agent_hash;         // FNV-1a of the function's agent name and initial state (isAgent / isState)
    uint32_t state_hash;
    uint32_t* error;             // device error record: [code, hash, index, count]
    const char* env;             // environment buffer (env table pointers are offsets into it)
    // batched launch (null batch: a single simulation)
    const BatchInstanceRT* batch;
    const uint32_t* batch_counts;
    uint32_t batch_n;
    // keys of the message build of this function's output and of its agents'
    // spatial sort, when the runtime has the launch compute them (single
    // simulations, rows not offset by a condition or an append)
    KeyTarget keyed[2];
};

}  // namespace detail
}  // namespace flamegpu

#endif  // INCLUDE_FLAMEGPU_DETAIL_DEVICE_TYPES_CUH_
