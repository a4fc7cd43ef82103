/*
 * fg_oracle.h — TEST INFRASTRUCTURE ONLY.
 *
 * Deterministic serial host restatement of FLAME GPU 2's spatial-message
 * build, neighbour iteration, auto spatial agent sort and birth/death
 * compaction, plus the three models (Boids, birth/death stress,
 * predator-prey) run on them. It is the CHECKER for the CUDA path: only the
 * test-suite, the smoke check and the CPU-baseline leg of the benchmark load
 * it. Nothing in the product links or calls it.
 *
 * Every function cites the reference file:line whose behaviour it restates
 * (paths relative to the FLAMEGPU2 project root).
 *
 * Within-bin order: the reference assigns a message's slot inside its bin with
 * atomicInc (src/flamegpu/runtime/messaging/MessageSpatial3D.cu:70), so its
 * within-bin order is unspecified. This oracle defines it as ascending
 * original message index (a stable counting sort); the CUDA build must match
 * that order bit-exactly. Against the reference itself only per-bin multisets
 * are comparable.
 */
#ifndef FG_ORACLE_H_
#define FG_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Spatial grid metadata: MessageSpatial3D::MetaData / MessageSpatial2D::MetaData
 * (include/flamegpu/runtime/messaging/MessageSpatial3D.h:38-68). */
typedef struct or_grid {
    int32_t dims;           /* 2 or 3 */
    float min[3];
    float max[3];
    float radius;
    float width[3];         /* environmentWidth */
    uint32_t gridDim[3];    /* gridDim[2] = 1 for 2D */
    uint32_t binCount;
    int32_t wrapCompatible;
} or_grid;

/* MessageSpatial3D.cu:31-52, MessageSpatial2D.cu:36-54 */
void or_grid_init(or_grid* g, int32_t dims, const float* mn, const float* mx, float radius);
/* include/flamegpu/detail/numeric.h:24-31 */
int32_t or_approx_exactly_divisible(float x, float y);

/* getGridPosition3D + getHash3D (MessageSpatial3DDevice.cuh:646-672);
 * 2D: MessageSpatial2DDevice.cuh:605-627. z ignored for 2D. */
uint32_t or_bin(const or_grid* g, float x, float y, float z);

/* Message build: histogram, exclusive scan to PBM (binCount+1 entries) and a
 * stable scatter. perm[sorted_pos] = original index.
 * MessageSpatial3D.cu:113-146, CUDAScatter.cu:276-337. z may be NULL in 2D. */
void or_spatial_build(const or_grid* g, uint32_t n, const float* x, const float* y, const float* z,
                      uint32_t* pbm, uint32_t* perm, uint32_t* bin_of_msg);

/* Candidate enumeration of MessageSpatial{2,3}D::In::Filter (clamped strips) or
 * WrapFilter (27/9 single bins, modulo per axis), in the reference's visit
 * order. Writes sorted-message indices; returns the count (may exceed cap; only
 * the first cap are written).
 * 3D: MessageSpatial3DDevice.cuh:40-59,199-202,252-276,686-749.
 * 2D: MessageSpatial2DDevice.cuh:39-59,190,241-263,640-698. */
uint32_t or_neighbours(const or_grid* g, const uint32_t* pbm, float x, float y, float z, int32_t wrap,
                       uint32_t* out, uint32_t cap);

/* Auto spatial sort key (unclamped, width-based) and its bit width.
 * CUDASimulation.cu:335-408 (calculateSpatialHash*), :544-571. */
void or_sort_grid(const or_grid* msg_grid, uint32_t gridDim_out[3], float envWidth_out[3]);
uint32_t or_sort_key(const or_grid* msg_grid, float x, float y, float z);
int32_t or_sort_max_bit(const or_grid* msg_grid);
/* Stable ascending sort of (key & ((1<<bits)-1)), as cub::DeviceRadixSort::SortPairs
 * with begin_bit 0 (include/flamegpu/runtime/agent/HostAgentAPI.cuh:858-915).
 * perm[sorted_pos] = original index. */
void or_stable_sort_perm(uint32_t n, const uint32_t* keys, int32_t bits, uint32_t* perm);

/* Order-preserving compaction: out positions of flagged rows.
 * CUDAFatAgent.cu:105-137, CUDAScatter.cu:67-88. Returns survivors. */
uint32_t or_compact(uint32_t n, const uint32_t* alive, uint32_t* perm_out);

/* ------------------------------------------------------------------ models */

/* Boids on MessageSpatial3D; agent SoA in/out, n agents, steps steps.
 * Clamped variant: examples/cpp/boids_spatial3D/src/main.cu:134-309.
 * Wrapped variant: examples/python_native/boids_spatial3D_wrapped/boids_spatial3D.py:123-255
 * (wing animation variables omitted). Layers: outputdata | inputdata; the
 * inputdata layer auto-sorts agents first (sortPeriod, CUDASimulation.cu:670-681).
 * threads > 1 splits the per-agent loop of inputdata over host threads (the
 * arithmetic and its order per agent are unchanged). */
typedef struct or_boids_params {
    float min_pos, max_pos;          /* environment bounds, cube */
    float interaction_radius, separation_radius;
    float time_scale, global_scale, steer_scale, collision_scale, match_scale;
    int32_t wrap;                    /* 1: wrapped iterator + position wrap; 0: clamped */
    uint32_t sort_period;            /* 0 disables auto spatial sort */
} or_boids_params;

void or_boids_run(const or_boids_params* p, uint32_t n, uint32_t* id, float* x, float* y, float* z,
                  float* fx, float* fy, float* fz, uint32_t steps, uint32_t first_step, int32_t threads);

/* Neighbour count test models (tests/test_cases/runtime/messaging/test_spatial_3d.cu:37-66 in3D,
 * :855-900 inWrapped3D; 2D: test_spatial_2d.cu). Outputs per-agent count / badCount /
 * virtual-offset sums after one step (layers out | in, sorted as the reference does). */
void or_count_model(const or_grid* g, int32_t wrap, uint32_t n, const uint32_t* id, float* x, float* y, float* z,
                    const int32_t* do_output, uint32_t* count, uint32_t* badCount, float* rx, float* ry, float* rz,
                    uint32_t* order_out);

/* Birth/death stress model. 8 float vars (f[v*cap + i]), counter (int32) and _id.
 * Per step: counter += 1; die with p_death; a survivor spawns a child with p_birth
 * (copies f0..f7, counter = 0). Survivors keep order, children follow in
 * parent order with _id = nextID + birth rank (CUDAAgentStateList.cu:189-250,
 * CUDAFatAgent.cu:311-346). Population never exceeds cap (births beyond cap are
 * dropped in parent order). Returns final population; *next_id updated.
 * pop_per_step (optional, length steps) receives the population entering each step. */
uint32_t or_birth_death_run(uint32_t n, uint32_t cap, float* f, int32_t* counter, uint32_t* id,
                            uint32_t* next_id, float p_death, float p_birth, uint64_t seed,
                            uint32_t steps, uint32_t first_step, uint32_t* pop_per_step);

/* Model-level counter-based RNG shared by the CUDA models and the oracle:
 * SplitMix64 finaliser (Steele, Lea & Flood 2014) over (seed, key, step, stream);
 * uniform = top 24 bits * 2^-24. */
uint64_t or_mix64(uint64_t z);
float or_hash_uniform(uint64_t seed, uint64_t key, uint32_t step, uint32_t stream);

/* Predator-prey on MessageSpatial2D (the model of examples/predprey2D/predprey.cu).
 * Per step: predators and prey output locations; prey are auto-sorted and
 * count the other prey within radius; each prey dies if a predator message
 * lies within radius (clamped Filter), else moves and, if its count is below
 * max_crowd, may give birth; predators die or move. Prey arrays
 * have room for cap_prey rows. Returns via *n_prey / *n_pred. */
typedef struct or_predprey_params {
    float edge, radius, p_prey_birth, p_pred_death, step;
    uint64_t seed;
    uint32_t max_crowd;  /* prey breed only with fewer other prey than this within radius */
} or_predprey_params;

void or_predprey_run(const or_predprey_params* p, uint32_t steps, uint32_t first_step,
                     uint32_t* n_prey, uint32_t cap_prey, float* prey_x, float* prey_y, uint32_t* prey_id,
                     uint32_t* next_prey_id, uint32_t* n_pred, float* pred_x, float* pred_y, uint32_t* pred_id);

/* The large spatial workloads' model (examples/spatial_payload/spatial_payload.cu):
 * agents with a position and payload p0..p3 (p[k*n + i]) output a spatial
 * message each step, are auto-sorted (every sort_period steps; 0 = never),
 * then average the payload of the messages within the radius (clamped Filter,
 * or WrapFilter with virtual positions when wrap != 0) and mix it into their
 * own. z is ignored (may be NULL) in 2D. threads > 1 splits the per-agent
 * loop over host threads. */
void or_payload_run(const or_grid* g, int32_t wrap, uint32_t sort_period, uint32_t n, uint32_t* id,
                    float* x, float* y, float* z, float* p, uint32_t steps, uint32_t first_step, int32_t threads);
/* One step of the same model in which only the m agents sample[0..m) (indices
 * after the step's automatic sort) run the iterate layer, serially: the CPU
 * baseline's bounded sample of a full-size population. times[0] receives the
 * seconds of the sort and the message build (whole population), times[1]
 * those of the sample's iterate. */
void or_payload_step_sampled(const or_grid* g, int32_t wrap, uint32_t n, uint32_t* id, float* x, float* y,
                             float* z, float* p, uint32_t m, const uint32_t* sample, double* times);

#ifdef __cplusplus
}
#endif

#endif  /* FG_ORACLE_H_ */
