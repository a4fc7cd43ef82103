// fg_oracle.cpp — TEST INFRASTRUCTURE ONLY (see fg_oracle.h).
//
// Serial host restatement of the reference's hot path. Compiled with
// -ffp-contract=off so that float results do not depend on whether the host
// compiler contracts a*b+c into an FMA (x86-64 and aarch64 differ there); the
// CUDA model sources are compiled with --fmad=false for the same reason, which
// makes Boids positions bit-comparable with this file.
#include "fg_oracle.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

namespace {

inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// getHash3D (MessageSpatial3DDevice.cuh:660-672): x is clamped, y/z are taken as given.
inline uint32_t hash3(const or_grid* g, int gx, int gy, int gz) {
    const int dx = static_cast<int>(g->gridDim[0]);
    const uint32_t ux = static_cast<uint32_t>(gx < 0 ? 0 : (gx >= dx - 1 ? dx - 1 : gx));
    return static_cast<uint32_t>(gz) * g->gridDim[0] * g->gridDim[1] + static_cast<uint32_t>(gy) * g->gridDim[0] + ux;
}
// getHash2D (MessageSpatial2DDevice.cuh:616-627).
inline uint32_t hash2(const or_grid* g, int gx, int gy) {
    const int dx = static_cast<int>(g->gridDim[0]);
    const uint32_t ux = static_cast<uint32_t>(gx < 0 ? 0 : (gx >= dx - 1 ? dx - 1 : gx));
    return static_cast<uint32_t>(gy) * g->gridDim[0] + ux;
}

// getGridPosition3D / getGridPosition2D: clamp(floorf((p - min) / radius)).
inline void grid_pos(const or_grid* g, float x, float y, float z, int out[3]) {
    const float p[3] = {x, y, z};
    for (int a = 0; a < 3; ++a) {
        if (a >= g->dims) { out[a] = 0; continue; }
        const int v = static_cast<int>(floorf((p[a] - g->min[a]) / g->radius));
        out[a] = clampi(v, 0, static_cast<int>(g->gridDim[a]) - 1);
    }
}

}  // namespace

extern "C" {

int32_t or_approx_exactly_divisible(float x, float y) {
    // include/flamegpu/detail/numeric.h:24-31
    const float scaledEpsilon = std::max(std::abs(x), std::abs(y)) * std::numeric_limits<float>::epsilon();
    const float v = std::fmod(x, y);
    return (v <= scaledEpsilon || v > y - scaledEpsilon) ? 1 : 0;
}

void or_grid_init(or_grid* g, int32_t dims, const float* mn, const float* mx, float radius) {
    // MessageSpatial3D.cu:31-52 (3D), MessageSpatial2D.cu:36-54 (2D)
    std::memset(g, 0, sizeof(*g));
    g->dims = dims;
    g->radius = radius;
    g->binCount = 1;
    g->wrapCompatible = 1;
    for (int a = 0; a < 3; ++a) {
        if (a < dims) {
            g->min[a] = mn[a];
            g->max[a] = mx[a];
            g->width[a] = g->max[a] - g->min[a];
            g->gridDim[a] = static_cast<uint32_t>(std::ceil(g->width[a] / g->radius));
            g->binCount *= g->gridDim[a];
            g->wrapCompatible = g->wrapCompatible && or_approx_exactly_divisible(g->width[a], g->radius);
        } else {
            g->gridDim[a] = 1;
        }
    }
}

uint32_t or_bin(const or_grid* g, float x, float y, float z) {
    int gp[3];
    grid_pos(g, x, y, z, gp);
    return g->dims == 3 ? hash3(g, gp[0], gp[1], gp[2]) : hash2(g, gp[0], gp[1]);
}

void or_spatial_build(const or_grid* g, uint32_t n, const float* x, const float* y, const float* z,
                      uint32_t* pbm, uint32_t* perm, uint32_t* bin_of_msg) {
    // Histogram (atomicHistogram3D, MessageSpatial3D.cu:54-72), exclusive scan
    // (cub::DeviceScan::ExclusiveSum over binCount+1, :134) and a stable scatter
    // (pbm_reorder, CUDAScatter.cu:276-294, with the within-bin slot defined as
    // ascending original index).
    const uint32_t B = g->binCount;
    std::vector<uint32_t> hist(static_cast<size_t>(B) + 1, 0), bins(n);
    for (uint32_t i = 0; i < n; ++i) {
        bins[i] = or_bin(g, x[i], y[i], z ? z[i] : 0.0f);
        hist[bins[i]]++;
    }
    uint32_t run = 0;
    for (uint32_t b = 0; b <= B; ++b) {
        pbm[b] = run;
        run += hist[b];
    }
    std::vector<uint32_t> cursor(pbm, pbm + B + 1);
    for (uint32_t i = 0; i < n; ++i) perm[cursor[bins[i]]++] = i;
    if (bin_of_msg) std::memcpy(bin_of_msg, bins.data(), sizeof(uint32_t) * n);
}

uint32_t or_neighbours(const or_grid* g, const uint32_t* pbm, float x, float y, float z, int32_t wrap,
                       uint32_t* out, uint32_t cap) {
    uint32_t cnt = 0;
    auto emit = [&](uint32_t b0, uint32_t b1) {  // messages PBM[b0] .. PBM[b1+1]
        for (uint32_t m = pbm[b0]; m < pbm[b1 + 1]; ++m) {
            if (cnt < cap) out[cnt] = m;
            ++cnt;
        }
    };
    int c[3];
    grid_pos(g, x, y, z, c);
    if (g->dims == 3) {
        const int gd[3] = {static_cast<int>(g->gridDim[0]), static_cast<int>(g->gridDim[1]), static_cast<int>(g->gridDim[2])};
        if (!wrap) {
            // Filter: strips along x, y-offset outer, z-offset inner (MessageSpatial3DDevice.cuh:693-719)
            for (int ry = -1; ry <= 1; ++ry) {
                for (int rz = -1; rz <= 1; ++rz) {
                    const int ay = c[1] + ry, az = c[2] + rz;
                    if (ay >= 0 && az >= 0 && ay < gd[1] && az < gd[2]) {
                        emit(hash3(g, c[0] - 1, ay, az), hash3(g, c[0] + 1, ay, az));
                    }
                }
            }
        } else {
            // WrapFilter: 27 single bins, x outer, y, z inner, each axis modulo gridDim
            // (MessageSpatial3DDevice.cuh:727-749)
            for (int rx = -1; rx <= 1; ++rx)
                for (int ry = -1; ry <= 1; ++ry)
                    for (int rz = -1; rz <= 1; ++rz) {
                        const int ax = static_cast<int>(static_cast<uint32_t>(c[0] + rx + gd[0]) % g->gridDim[0]);
                        const int ay = static_cast<int>(static_cast<uint32_t>(c[1] + ry + gd[1]) % g->gridDim[1]);
                        const int az = static_cast<int>(static_cast<uint32_t>(c[2] + rz + gd[2]) % g->gridDim[2]);
                        const uint32_t h = hash3(g, ax, ay, az);
                        emit(h, h);
                    }
        }
    } else {
        const int gd[2] = {static_cast<int>(g->gridDim[0]), static_cast<int>(g->gridDim[1])};
        if (!wrap) {
            // Filter: 3 strips along x (MessageSpatial2DDevice.cuh:646-672)
            for (int ry = -1; ry <= 1; ++ry) {
                const int ay = c[1] + ry;
                if (ay >= 0 && ay < gd[1]) emit(hash2(g, c[0] - 1, ay), hash2(g, c[0] + 1, ay));
            }
        } else {
            // WrapFilter: 9 bins, x outer, y inner (MessageSpatial2DDevice.cuh:673-698)
            for (int rx = -1; rx <= 1; ++rx)
                for (int ry = -1; ry <= 1; ++ry) {
                    const int ax = static_cast<int>(static_cast<uint32_t>(c[0] + rx + gd[0]) % g->gridDim[0]);
                    const int ay = static_cast<int>(static_cast<uint32_t>(c[1] + ry + gd[1]) % g->gridDim[1]);
                    const uint32_t h = hash2(g, ax, ay);
                    emit(h, h);
                }
        }
    }
    return cnt;
}

void or_sort_grid(const or_grid* mg, uint32_t gd[3], float w[3]) {
    // CUDASimulation.cu:494-507: width from the message bounds, gridDim =
    // ceilf(width / radius), 1 for a zero-width axis (z of a 2D message).
    for (int a = 0; a < 3; ++a) {
        w[a] = a < mg->dims ? (mg->max[a] - mg->min[a]) : 0.0f;
        gd[a] = w[a] != 0.0f ? static_cast<uint32_t>(ceilf(w[a] / mg->radius)) : 1u;
    }
}

uint32_t or_sort_key(const or_grid* mg, float x, float y, float z) {
    // calculateSpatialHash (CUDASimulation.cu:380-408): unclamped, width based.
    uint32_t gd[3];
    float w[3];
    or_sort_grid(mg, gd, w);
    const int gx = static_cast<int>(floorf(((x - mg->min[0]) / w[0]) * static_cast<float>(gd[0])));
    const int gy = static_cast<int>(floorf(((y - mg->min[1]) / w[1]) * static_cast<float>(gd[1])));
    if (mg->dims == 3) {
        const int gz = static_cast<int>(floorf(((z - mg->min[2]) / w[2]) * static_cast<float>(gd[2])));
        return static_cast<uint32_t>(gz * gd[0] * gd[1] + (gy * gd[0]) + gx);
    }
    return static_cast<uint32_t>((gy * gd[0]) + gx);
}

int32_t or_sort_max_bit(const or_grid* mg) {
    // CUDASimulation.cu:569-571
    uint32_t gd[3];
    float w[3];
    or_sort_grid(mg, gd, w);
    return static_cast<int32_t>(std::floor(std::log2(gd[0] * gd[1] * gd[2]))) + 1;
}

void or_stable_sort_perm(uint32_t n, const uint32_t* keys, int32_t bits, uint32_t* perm) {
    const uint32_t mask = bits >= 32 ? 0xFFFFFFFFu : ((1u << bits) - 1u);
    std::vector<uint32_t> idx(n);
    for (uint32_t i = 0; i < n; ++i) idx[i] = i;
    std::stable_sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) { return (keys[a] & mask) < (keys[b] & mask); });
    std::memcpy(perm, idx.data(), sizeof(uint32_t) * n);
}

uint32_t or_compact(uint32_t n, const uint32_t* alive, uint32_t* perm_out) {
    uint32_t k = 0;
    for (uint32_t i = 0; i < n; ++i)
        if (alive[i]) perm_out[k++] = i;
    return k;
}

uint64_t or_mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

float or_hash_uniform(uint64_t seed, uint64_t key, uint32_t step, uint32_t stream) {
    const uint64_t h = or_mix64(or_mix64(or_mix64(seed) ^ key) ^ ((static_cast<uint64_t>(step) << 8) | stream));
    return static_cast<float>(h >> 40) * (1.0f / 16777216.0f);
}

}  // extern "C"

// ---------------------------------------------------------------------- Boids

namespace {

template <typename T>
void apply_perm(std::vector<T>& tmp, T* a, const uint32_t* perm, uint32_t n) {
    tmp.resize(n);
    for (uint32_t i = 0; i < n; ++i) tmp[i] = a[perm[i]];
    std::memcpy(a, tmp.data(), sizeof(T) * n);
}

inline float vec3Length(const float x, const float y, const float z) { return sqrtf(x * x + y * y + z * z); }

struct BoidsMsgs {
    std::vector<uint32_t> id;
    std::vector<float> x, y, z, fx, fy, fz;
};

// inputdata for one agent. Clamped: examples/cpp/boids_spatial3D/src/main.cu:146-309.
// Wrapped: examples/python_native/boids_spatial3D_wrapped/boids_spatial3D.py:95-255.
void boids_agent(const or_boids_params* p, const or_grid* g, const uint32_t* pbm, const BoidsMsgs& m,
                 uint32_t& id_, float& ax, float& ay, float& az, float& afx, float& afy, float& afz,
                 std::vector<uint32_t>& cand) {
    const uint32_t id = id_;
    float agent_x = ax, agent_y = ay, agent_z = az;
    float agent_fx = afx, agent_fy = afy, agent_fz = afz;
    float perceived_centre_x = 0.0f, perceived_centre_y = 0.0f, perceived_centre_z = 0.0f;
    int perceived_count = 0;
    float global_velocity_x = 0.0f, global_velocity_y = 0.0f, global_velocity_z = 0.0f;
    float velocity_change_x = 0.f, velocity_change_y = 0.f, velocity_change_z = 0.f;
    const float INTERACTION_RADIUS = p->interaction_radius;
    const float SEPARATION_RADIUS = p->separation_radius;
    uint32_t nc = or_neighbours(g, pbm, agent_x, agent_y, agent_z, p->wrap, cand.data(), static_cast<uint32_t>(cand.size()));
    if (nc > cand.size()) {
        cand.resize(nc);
        nc = or_neighbours(g, pbm, agent_x, agent_y, agent_z, p->wrap, cand.data(), nc);
    }
    for (uint32_t c = 0; c < nc; ++c) {
        const uint32_t mi = cand[c];
        if (m.id[mi] != id) {
            float message_x, message_y, message_z;
            if (p->wrap) {
                // getVirtualX/Y/Z (MessageSpatial3DDevice.cuh:373-397)
                const float x2 = m.x[mi], y2 = m.y[mi], z2 = m.z[mi];
                const float x21 = x2 - agent_x, y21 = y2 - agent_y, z21 = z2 - agent_z;
                message_x = std::abs(x21) > g->width[0] / 2.0f ? x2 - (x21 / std::abs(x21) * g->width[0]) : x2;
                message_y = std::abs(y21) > g->width[1] / 2.0f ? y2 - (y21 / std::abs(y21) * g->width[1]) : y2;
                message_z = std::abs(z21) > g->width[2] / 2.0f ? z2 - (z21 / std::abs(z21) * g->width[2]) : z2;
            } else {
                message_x = m.x[mi];
                message_y = m.y[mi];
                message_z = m.z[mi];
            }
            const float separation = vec3Length(agent_x - message_x, agent_y - message_y, agent_z - message_z);
            if (separation < INTERACTION_RADIUS) {
                perceived_centre_x += message_x;
                perceived_centre_y += message_y;
                perceived_centre_z += message_z;
                perceived_count++;
                global_velocity_x += m.fx[mi];
                global_velocity_y += m.fy[mi];
                global_velocity_z += m.fz[mi];
                if (separation < (SEPARATION_RADIUS)) {
                    const float normalizedSeparation = (separation / SEPARATION_RADIUS);
                    const float invNormSep = (1.0f - normalizedSeparation);
                    const float invSqSep = invNormSep * invNormSep;
                    const float collisionScale = p->collision_scale;
                    velocity_change_x += collisionScale * (agent_x - message_x) * invSqSep;
                    velocity_change_y += collisionScale * (agent_y - message_y) * invSqSep;
                    velocity_change_z += collisionScale * (agent_z - message_z) * invSqSep;
                }
            }
        }
    }
    if (perceived_count) {
        perceived_centre_x /= perceived_count;
        perceived_centre_y /= perceived_count;
        perceived_centre_z /= perceived_count;
        global_velocity_x /= perceived_count;
        global_velocity_y /= perceived_count;
        global_velocity_z /= perceived_count;
        const float STEER_SCALE = p->steer_scale;
        const float steer_velocity_x = (perceived_centre_x - agent_x) * STEER_SCALE;
        const float steer_velocity_y = (perceived_centre_y - agent_y) * STEER_SCALE;
        const float steer_velocity_z = (perceived_centre_z - agent_z) * STEER_SCALE;
        velocity_change_x += steer_velocity_x;
        velocity_change_y += steer_velocity_y;
        velocity_change_z += steer_velocity_z;
        const float MATCH_SCALE = p->match_scale;
        const float match_velocity_x = global_velocity_x * MATCH_SCALE;
        const float match_velocity_y = global_velocity_y * MATCH_SCALE;
        const float match_velocity_z = global_velocity_z * MATCH_SCALE;
        velocity_change_x += match_velocity_x - agent_fx;
        velocity_change_y += match_velocity_y - agent_fy;
        velocity_change_z += match_velocity_z - agent_fz;
    }
    velocity_change_x *= p->global_scale;
    velocity_change_y *= p->global_scale;
    velocity_change_z *= p->global_scale;
    agent_fx += velocity_change_x;
    agent_fy += velocity_change_y;
    agent_fz += velocity_change_z;
    float agent_fscale = vec3Length(agent_fx, agent_fy, agent_fz);
    if (agent_fscale > 1) {
        agent_fx /= agent_fscale;
        agent_fy /= agent_fscale;
        agent_fz /= agent_fscale;
    }
    const float minSpeed = 0.5f;
    if (agent_fscale < minSpeed) {
        agent_fx /= agent_fscale;
        agent_fy /= agent_fscale;
        agent_fz /= agent_fscale;
        agent_fx *= minSpeed;
        agent_fy *= minSpeed;
        agent_fz *= minSpeed;
    }
    const float minPosition = p->min_pos;
    const float maxPosition = p->max_pos;
    if (!p->wrap) {
        const float wallInteractionDistance = 0.10f;
        const float wallSteerStrength = 0.05f;
        if (agent_x - minPosition < wallInteractionDistance) agent_fx += wallSteerStrength;
        if (agent_y - minPosition < wallInteractionDistance) agent_fy += wallSteerStrength;
        if (agent_z - minPosition < wallInteractionDistance) agent_fz += wallSteerStrength;
        if (maxPosition - agent_x < wallInteractionDistance) agent_fx -= wallSteerStrength;
        if (maxPosition - agent_y < wallInteractionDistance) agent_fy -= wallSteerStrength;
        if (maxPosition - agent_z < wallInteractionDistance) agent_fz -= wallSteerStrength;
    }
    const float TIME_SCALE = p->time_scale;
    agent_x += agent_fx * TIME_SCALE;
    agent_y += agent_fy * TIME_SCALE;
    agent_z += agent_fz * TIME_SCALE;
    if (p->wrap) {
        const float width = maxPosition - minPosition;
        if (agent_x < minPosition) agent_x += width;
        if (agent_y < minPosition) agent_y += width;
        if (agent_z < minPosition) agent_z += width;
        if (agent_x > maxPosition) agent_x -= width;
        if (agent_y > maxPosition) agent_y -= width;
        if (agent_z > maxPosition) agent_z -= width;
    } else {
        agent_x = (agent_x < minPosition) ? minPosition : agent_x;
        agent_x = (agent_x > maxPosition) ? maxPosition : agent_x;
        agent_y = (agent_y < minPosition) ? minPosition : agent_y;
        agent_y = (agent_y > maxPosition) ? maxPosition : agent_y;
        agent_z = (agent_z < minPosition) ? minPosition : agent_z;
        agent_z = (agent_z > maxPosition) ? maxPosition : agent_z;
    }
    ax = agent_x;
    ay = agent_y;
    az = agent_z;
    afx = agent_fx;
    afy = agent_fy;
    afz = agent_fz;
}

}  // namespace

extern "C" void or_boids_run(const or_boids_params* p, uint32_t n, uint32_t* id, float* x, float* y, float* z,
                             float* fx, float* fy, float* fz, uint32_t steps, uint32_t first_step, int32_t threads) {
    or_grid g;
    const float mn[3] = {p->min_pos, p->min_pos, p->min_pos};
    const float mx[3] = {p->max_pos, p->max_pos, p->max_pos};
    or_grid_init(&g, 3, mn, mx, p->interaction_radius);
    std::vector<uint32_t> pbm(static_cast<size_t>(g.binCount) + 1), perm(n), keys(n), tmpu;
    std::vector<float> tmpf;
    BoidsMsgs msg, sorted;
    const int nt = threads < 1 ? 1 : threads;
    for (uint32_t s = 0; s < steps; ++s) {
        const uint32_t step = first_step + s;
        // Layer 1, outputdata (main.cu:134-144): one message per agent, in agent order.
        msg.id.assign(id, id + n);
        msg.x.assign(x, x + n);
        msg.y.assign(y, y + n);
        msg.z.assign(z, z + n);
        msg.fx.assign(fx, fx + n);
        msg.fy.assign(fy, fy + n);
        msg.fz.assign(fz, fz + n);
        // Layer 2: auto spatial sort of the agents (CUDASimulation.cu:670-681), then the
        // message index build (:864), then inputdata.
        if (p->sort_period && step % p->sort_period == 0) {
            for (uint32_t i = 0; i < n; ++i) keys[i] = or_sort_key(&g, x[i], y[i], z[i]);
            or_stable_sort_perm(n, keys.data(), or_sort_max_bit(&g), perm.data());
            apply_perm(tmpu, id, perm.data(), n);
            apply_perm(tmpf, x, perm.data(), n);
            apply_perm(tmpf, y, perm.data(), n);
            apply_perm(tmpf, z, perm.data(), n);
            apply_perm(tmpf, fx, perm.data(), n);
            apply_perm(tmpf, fy, perm.data(), n);
            apply_perm(tmpf, fz, perm.data(), n);
        }
        or_spatial_build(&g, n, msg.x.data(), msg.y.data(), msg.z.data(), pbm.data(), perm.data(), nullptr);
        sorted.id.resize(n); sorted.x.resize(n); sorted.y.resize(n); sorted.z.resize(n);
        sorted.fx.resize(n); sorted.fy.resize(n); sorted.fz.resize(n);
        for (uint32_t j = 0; j < n; ++j) {
            const uint32_t i = perm[j];
            sorted.id[j] = msg.id[i]; sorted.x[j] = msg.x[i]; sorted.y[j] = msg.y[i]; sorted.z[j] = msg.z[i];
            sorted.fx[j] = msg.fx[i]; sorted.fy[j] = msg.fy[i]; sorted.fz[j] = msg.fz[i];
        }
        auto work = [&](uint32_t lo, uint32_t hi) {
            std::vector<uint32_t> cand(256);
            for (uint32_t i = lo; i < hi; ++i)
                boids_agent(p, &g, pbm.data(), sorted, id[i], x[i], y[i], z[i], fx[i], fy[i], fz[i], cand);
        };
        if (nt == 1 || n < 1024) {
            work(0, n);
        } else {
            std::vector<std::thread> pool;
            const uint32_t chunk = (n + nt - 1) / nt;
            for (int t = 0; t < nt; ++t) {
                const uint32_t lo = std::min<uint32_t>(n, t * chunk), hi = std::min<uint32_t>(n, lo + chunk);
                pool.emplace_back(work, lo, hi);
            }
            for (auto& th : pool) th.join();
        }
    }
}

// ---------------------------------------------------------- count test model

extern "C" void or_count_model(const or_grid* g, int32_t wrap, uint32_t n, const uint32_t* id, float* x, float* y,
                               float* z, const int32_t* do_output, uint32_t* count, uint32_t* badCount, float* rx,
                               float* ry, float* rz, uint32_t* order_out) {
    // Layer 1 "out" (test_spatial_3d.cu:16-33): one message per outputting agent, in
    // agent order (optional output is compacted stably, CUDAMessage.cu:171-208).
    std::vector<uint32_t> mid;
    std::vector<float> mx, my, mz;
    for (uint32_t i = 0; i < n; ++i) {
        if (do_output && !do_output[i]) continue;
        mid.push_back(id[i]);
        mx.push_back(x[i]);
        my.push_back(y[i]);
        mz.push_back(g->dims == 3 ? z[i] : 0.0f);
    }
    const uint32_t nm = static_cast<uint32_t>(mid.size());
    // Layer 2 "in": auto-sort (step 0, sortPeriod 1) then build then iterate.
    std::vector<uint32_t> keys(n), sperm(n);
    for (uint32_t i = 0; i < n; ++i) keys[i] = or_sort_key(g, x[i], y[i], g->dims == 3 ? z[i] : 0.0f);
    or_stable_sort_perm(n, keys.data(), or_sort_max_bit(g), sperm.data());
    std::vector<float> tf;
    apply_perm(tf, x, sperm.data(), n);
    apply_perm(tf, y, sperm.data(), n);
    if (g->dims == 3) apply_perm(tf, z, sperm.data(), n);
    if (order_out) std::memcpy(order_out, sperm.data(), sizeof(uint32_t) * n);
    std::vector<uint32_t> pbm(static_cast<size_t>(g->binCount) + 1), perm(nm + 1), cand(64);
    or_spatial_build(g, nm, mx.data(), my.data(), g->dims == 3 ? mz.data() : nullptr, pbm.data(), perm.data(), nullptr);
    for (uint32_t a = 0; a < n; ++a) {
        const uint32_t self_id = id[sperm[a]];
        const float x1 = x[a], y1 = y[a], z1 = g->dims == 3 ? z[a] : 0.0f;
        uint32_t nc = or_neighbours(g, pbm.data(), x1, y1, z1, wrap, cand.data(), static_cast<uint32_t>(cand.size()));
        if (nc > cand.size()) {
            cand.resize(nc);
            nc = or_neighbours(g, pbm.data(), x1, y1, z1, wrap, cand.data(), nc);
        }
        uint32_t c = 0, bad = 0;
        float sx = 0, sy = 0, sz = 0;
        for (uint32_t k = 0; k < nc; ++k) {
            const uint32_t mi = perm[cand[k]];
            if (!wrap) {
                // in3D (test_spatial_3d.cu:37-66) / in2D: Moore-neighbourhood check on truncated coords.
                const int myBin[3] = {static_cast<int>(x1), static_cast<int>(y1), static_cast<int>(z1)};
                const int mb[3] = {static_cast<int>(mx[mi]), static_cast<int>(my[mi]), static_cast<int>(mz[mi])};
                bool isBad = false;
                for (int ax = 0; ax < g->dims; ++ax) {
                    const int d = myBin[ax] - mb[ax];
                    if (d > 1 || d < -1) isBad = true;
                }
                c++;
                bad = isBad ? bad + 1 : bad;
            } else {
                // inWrapped3D (test_spatial_3d.cu:855-900)
                const float p1[3] = {x1, y1, z1};
                const float p2raw[3] = {mx[mi], my[mi], mz[mi]};
                float p2[3], d[3];
                for (int ax = 0; ax < 3; ++ax) {
                    if (ax < g->dims) {
                        const float v21 = p2raw[ax] - p1[ax];
                        p2[ax] = std::abs(v21) > g->width[ax] / 2.0f ? p2raw[ax] - (v21 / std::abs(v21) * g->width[ax]) : p2raw[ax];
                    } else {
                        p2[ax] = p1[ax];
                    }
                    d[ax] = p2[ax] - p1[ax];
                }
                const float distance = g->dims == 3 ? sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
                                                    : sqrtf(d[0] * d[0] + d[1] * d[1]);
                bool isBad = distance > g->radius;
                for (int ax = 0; ax < g->dims; ++ax)
                    if (std::abs(d[ax]) != 2.0f && p2[ax] != p1[ax]) isBad = true;
                if (isBad) {
                    bad++;
                } else {
                    c++;
                    if (mid[mi] != self_id) {
                        sx += d[0];
                        sy += d[1];
                        sz += d[2];
                    }
                }
            }
        }
        count[a] = c;
        badCount[a] = bad;
        if (rx) rx[a] = sx;
        if (ry) ry[a] = sy;
        if (rz) rz[a] = sz;
    }
}

// ------------------------------------------------------- birth/death model

extern "C" uint32_t or_birth_death_run(uint32_t n, uint32_t cap, float* f, int32_t* counter, uint32_t* id,
                                       uint32_t* next_id, float p_death, float p_birth, uint64_t seed,
                                       uint32_t steps, uint32_t first_step, uint32_t* pop_per_step) {
    // f is [8][cap] (variable-major). Death: CUDAFatAgent.cu:105-137 (stable);
    // birth: CUDAAgentStateList.cu:189-250 (children after survivors, parent order).
    std::vector<float> nf(static_cast<size_t>(8) * cap);
    std::vector<int32_t> nc(cap);
    std::vector<uint32_t> nid(cap);
    std::vector<uint32_t> parents;
    for (uint32_t s = 0; s < steps; ++s) {
        const uint32_t step = first_step + s;
        if (pop_per_step) pop_per_step[s] = n;
        uint32_t k = 0;
        parents.clear();
        for (uint32_t i = 0; i < n; ++i) {
            const uint32_t key = id[i];
            const bool dead = or_hash_uniform(seed, key, step, 0) < p_death;
            if (!dead) {
                for (int v = 0; v < 8; ++v) nf[static_cast<size_t>(v) * cap + k] = f[static_cast<size_t>(v) * cap + i];
                nc[k] = counter[i] + 1;
                nid[k] = id[i];
                ++k;
                if (or_hash_uniform(seed, key, step, 1) < p_birth) parents.push_back(i);
            }
        }
        uint32_t born = 0;
        for (uint32_t pi : parents) {
            if (k >= cap) break;
            for (int v = 0; v < 8; ++v) nf[static_cast<size_t>(v) * cap + k] = f[static_cast<size_t>(v) * cap + pi];
            nc[k] = 0;
            nid[k] = *next_id + born;
            ++born;
            ++k;
        }
        *next_id += born;
        n = k;
        for (int v = 0; v < 8; ++v)
            std::memcpy(f + static_cast<size_t>(v) * cap, nf.data() + static_cast<size_t>(v) * cap, sizeof(float) * n);
        std::memcpy(counter, nc.data(), sizeof(int32_t) * n);
        std::memcpy(id, nid.data(), sizeof(uint32_t) * n);
    }
    return n;
}

// ---------------------------------------------------------- predator-prey

extern "C" void or_predprey_run(const or_predprey_params* p, uint32_t steps, uint32_t first_step, uint32_t* n_prey,
                                uint32_t cap_prey, float* prey_x, float* prey_y, uint32_t* prey_id,
                                uint32_t* next_prey_id, uint32_t* n_pred, float* pred_x, float* pred_y,
                                uint32_t* pred_id) {
    // examples/predprey2D/predprey.cu restated serially; layers as in that model.
    or_grid g;
    const float mn[3] = {0.0f, 0.0f, 0.0f};
    const float mx[3] = {p->edge, p->edge, 0.0f};
    or_grid_init(&g, 2, mn, mx, p->radius);
    auto clampf = [](float v, float lo, float hi) { return v < lo ? lo : (v > hi ? hi : v); };
    std::vector<uint32_t> pbm(static_cast<size_t>(g.binCount) + 1), perm, keys, cand(64), tmpu;
    std::vector<float> mxs, mys, tmpf;
    for (uint32_t s = 0; s < steps; ++s) {
        const uint32_t step = first_step + s;
        // layer 1: predator messages (in predator order)
        const uint32_t np = *n_pred;
        std::vector<float> msg_x(pred_x, pred_x + np), msg_y(pred_y, pred_y + np);
        // prey auto-sort before prey_crowd (CUDASimulation.cu:670-681); the sort
        // before prey_step finds them already in key order (stable: no change)
        uint32_t n = *n_prey;
        keys.resize(n);
        perm.resize(std::max<uint32_t>(n, np));
        for (uint32_t i = 0; i < n; ++i) keys[i] = or_sort_key(&g, prey_x[i], prey_y[i], 0.0f);
        or_stable_sort_perm(n, keys.data(), or_sort_max_bit(&g), perm.data());
        apply_perm(tmpf, prey_x, perm.data(), n);
        apply_perm(tmpf, prey_y, perm.data(), n);
        apply_perm(tmpu, prey_id, perm.data(), n);
        std::vector<uint32_t> mperm(np + 1);
        or_spatial_build(&g, np, msg_x.data(), msg_y.data(), nullptr, pbm.data(), mperm.data(), nullptr);
        std::vector<float> sx(np), sy(np);
        for (uint32_t j = 0; j < np; ++j) {
            sx[j] = msg_x[mperm[j]];
            sy[j] = msg_y[mperm[j]];
        }
        // layer 2: prey_crowd over the prey messages of layer 1 (the count does
        // not depend on message order; the positions are the sorted prey's)
        std::vector<uint32_t> crowd(n, 0), ppbm(static_cast<size_t>(g.binCount) + 1), pperm(n + 1);
        or_spatial_build(&g, n, prey_x, prey_y, nullptr, ppbm.data(), pperm.data(), nullptr);
        for (uint32_t i = 0; i < n; ++i) {
            const float x = prey_x[i], y = prey_y[i];
            uint32_t nc = or_neighbours(&g, ppbm.data(), x, y, 0.0f, 0, cand.data(), static_cast<uint32_t>(cand.size()));
            if (nc > cand.size()) {
                cand.resize(nc);
                nc = or_neighbours(&g, ppbm.data(), x, y, 0.0f, 0, cand.data(), nc);
            }
            for (uint32_t c = 0; c < nc; ++c) {
                const uint32_t j = pperm[cand[c]];
                const float dx = prey_x[j] - x, dy = prey_y[j] - y;
                if (dx * dx + dy * dy < p->radius * p->radius && prey_id[j] != prey_id[i]) ++crowd[i];
            }
        }
        // layer 3: prey_step / predator_step
        std::vector<float> ox, oy, bx, by;
        std::vector<uint32_t> oid;
        for (uint32_t i = 0; i < n; ++i) {
            const float x = prey_x[i], y = prey_y[i];
            uint32_t nc = or_neighbours(&g, pbm.data(), x, y, 0.0f, 0, cand.data(), static_cast<uint32_t>(cand.size()));
            if (nc > cand.size()) {
                cand.resize(nc);
                nc = or_neighbours(&g, pbm.data(), x, y, 0.0f, 0, cand.data(), nc);
            }
            bool eaten = false;
            for (uint32_t c = 0; c < nc && !eaten; ++c) {
                const float dx = sx[cand[c]] - x, dy = sy[cand[c]] - y;
                if (dx * dx + dy * dy < p->radius * p->radius) eaten = true;
            }
            if (eaten) continue;
            const uint64_t key = prey_id[i];
            const float nx = clampf(x + p->step * (2.0f * or_hash_uniform(p->seed, key, step, 2) - 1.0f), 0.0f, p->edge);
            const float ny = clampf(y + p->step * (2.0f * or_hash_uniform(p->seed, key, step, 3) - 1.0f), 0.0f, p->edge);
            ox.push_back(nx);
            oy.push_back(ny);
            oid.push_back(prey_id[i]);
            if (or_hash_uniform(p->seed, key, step, 1) < p->p_prey_birth && crowd[i] < p->max_crowd) {
                bx.push_back(nx);
                by.push_back(ny);
            }
        }
        // survivors, then children in parent order with fresh ids
        uint32_t k = 0;
        for (size_t i = 0; i < ox.size() && k < cap_prey; ++i, ++k) {
            prey_x[k] = ox[i];
            prey_y[k] = oy[i];
            prey_id[k] = oid[i];
        }
        for (size_t i = 0; i < bx.size() && k < cap_prey; ++i, ++k) {
            prey_x[k] = bx[i];
            prey_y[k] = by[i];
            prey_id[k] = *next_prey_id + static_cast<uint32_t>(i);
        }
        *next_prey_id += static_cast<uint32_t>(bx.size());
        *n_prey = k;
        // predators
        uint32_t q = 0;
        for (uint32_t i = 0; i < np; ++i) {
            const uint64_t key = pred_id[i];
            if (or_hash_uniform(p->seed, key, step, 4) < p->p_pred_death) continue;
            const float x = pred_x[i], y = pred_y[i];
            pred_x[q] = clampf(x + p->step * (2.0f * or_hash_uniform(p->seed, key, step, 5) - 1.0f), 0.0f, p->edge);
            pred_y[q] = clampf(y + p->step * (2.0f * or_hash_uniform(p->seed, key, step, 6) - 1.0f), 0.0f, p->edge);
            pred_id[q] = pred_id[i];
            ++q;
        }
        *n_pred = q;
    }
}

// ------------------------------------------------------- spatial payload model

// The large spatial workloads' model (examples/spatial_payload/spatial_payload.cu,
// written against the reference API; the reference has no such example). Per
// step: layer 1 outputs one message per agent (position + p0..p3, in agent
// order); before layer 2 the agents are auto-sorted by the reference's sort key
// (CUDASimulation.cu:670-681, as or_boids_run); layer 2 averages the payload of
// the messages within the radius, visited in the order of the clamped Filter
// (MessageSpatial3DDevice.cuh:693-719, 2D MessageSpatial2DDevice.cuh:646-672)
// or the WrapFilter (:727-749, 2D :673-698) with distances to the virtual
// positions (MessageSpatial3DDevice.cuh:373-397), and mixes it into its own:
// p_k <- 0.5 p_k + 0.5 (sum_k / count).
namespace {
// sample (m rows, optional): only these agents run layer 2; times (optional)
// receives the seconds spent in the sort + build and in layer 2.
void payload_impl(const or_grid* g, int32_t wrap, uint32_t sort_period, uint32_t n, uint32_t* id, float* x, float* y,
                  float* z, float* p, uint32_t steps, uint32_t first_step, int32_t threads, const uint32_t* sample,
                  uint32_t m, double* times) {
    const int dims = g->dims;
    std::vector<uint32_t> pbm(static_cast<size_t>(g->binCount) + 1), perm(n), keys(n), tmpu;
    std::vector<float> tmpf, mx, my, mz, mp[4], sx, sy, sz, sp[4];
    const int nt = threads < 1 ? 1 : threads;
    const float r = g->radius;
    const float r2 = r * r;
    auto virt = [](float p1, float p2, float width) {  // getVirtualX: p2 - (d / |d|) * width
        const float d = p2 - p1;
        return std::fabs(d) > width / 2.0f ? p2 - (d / std::fabs(d) * width) : p2;
    };
    if (times) times[0] = times[1] = 0.0;
    for (uint32_t s = 0; s < steps; ++s) {
        const uint32_t step = first_step + s;
        const auto t0 = std::chrono::steady_clock::now();
        mx.assign(x, x + n);
        my.assign(y, y + n);
        if (dims == 3) mz.assign(z, z + n);
        for (int k = 0; k < 4; ++k) mp[k].assign(p + static_cast<size_t>(k) * n, p + static_cast<size_t>(k + 1) * n);
        if (sort_period && step % sort_period == 0) {
            for (uint32_t i = 0; i < n; ++i) keys[i] = or_sort_key(g, x[i], y[i], dims == 3 ? z[i] : 0.0f);
            or_stable_sort_perm(n, keys.data(), or_sort_max_bit(g), perm.data());
            apply_perm(tmpu, id, perm.data(), n);
            apply_perm(tmpf, x, perm.data(), n);
            apply_perm(tmpf, y, perm.data(), n);
            if (dims == 3) apply_perm(tmpf, z, perm.data(), n);
            for (int k = 0; k < 4; ++k) apply_perm(tmpf, p + static_cast<size_t>(k) * n, perm.data(), n);
        }
        or_spatial_build(g, n, mx.data(), my.data(), dims == 3 ? mz.data() : nullptr, pbm.data(), perm.data(), nullptr);
        sx.resize(n); sy.resize(n); sz.resize(n);
        for (int k = 0; k < 4; ++k) sp[k].resize(n);
        for (uint32_t j = 0; j < n; ++j) {
            const uint32_t i = perm[j];
            sx[j] = mx[i];
            sy[j] = my[i];
            sz[j] = dims == 3 ? mz[i] : 0.0f;
            for (int k = 0; k < 4; ++k) sp[k][j] = mp[k][i];
        }
        const auto t1 = std::chrono::steady_clock::now();
        const uint32_t rows = sample ? m : n;
        auto work = [&](uint32_t lo, uint32_t hi) {
            std::vector<uint32_t> cand(1024);
            for (uint32_t r = lo; r < hi; ++r) {
                const uint32_t i = sample ? sample[r] : r;
                const float ax = x[i], ay = y[i], az = dims == 3 ? z[i] : 0.0f;
                uint32_t nc = or_neighbours(g, pbm.data(), ax, ay, az, wrap, cand.data(), static_cast<uint32_t>(cand.size()));
                if (nc > cand.size()) {
                    cand.resize(nc);
                    nc = or_neighbours(g, pbm.data(), ax, ay, az, wrap, cand.data(), nc);
                }
                float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
                uint32_t c = 0;
                for (uint32_t q = 0; q < nc; ++q) {
                    const uint32_t m = cand[q];
                    float dx, dy, dz;
                    if (wrap) {
                        dx = virt(ax, sx[m], g->width[0]) - ax;
                        dy = virt(ay, sy[m], g->width[1]) - ay;
                        dz = dims == 3 ? virt(az, sz[m], g->width[2]) - az : 0.0f;
                    } else {
                        dx = sx[m] - ax;
                        dy = sy[m] - ay;
                        dz = dims == 3 ? sz[m] - az : 0.0f;
                    }
                    if (dx * dx + dy * dy + dz * dz < r2) {
                        s0 += sp[0][m];
                        s1 += sp[1][m];
                        s2 += sp[2][m];
                        s3 += sp[3][m];
                        ++c;
                    }
                }
                if (c) {
                    const float inv = 1.0f / static_cast<float>(c);
                    float* pk[4] = {p + i, p + static_cast<size_t>(n) + i, p + 2 * static_cast<size_t>(n) + i,
                                    p + 3 * static_cast<size_t>(n) + i};
                    *pk[0] = 0.5f * *pk[0] + 0.5f * s0 * inv;
                    *pk[1] = 0.5f * *pk[1] + 0.5f * s1 * inv;
                    *pk[2] = 0.5f * *pk[2] + 0.5f * s2 * inv;
                    *pk[3] = 0.5f * *pk[3] + 0.5f * s3 * inv;
                }
            }
        };
        if (nt == 1 || rows < 1024) {
            work(0, rows);
        } else {
            std::vector<std::thread> pool;
            const uint32_t chunk = (rows + nt - 1) / nt;
            for (int t = 0; t < nt; ++t) {
                const uint32_t lo = std::min<uint32_t>(rows, t * chunk), hi = std::min<uint32_t>(rows, lo + chunk);
                pool.emplace_back(work, lo, hi);
            }
            for (auto& th : pool) th.join();
        }
        if (times) {
            const auto t2 = std::chrono::steady_clock::now();
            times[0] += std::chrono::duration<double>(t1 - t0).count();
            times[1] += std::chrono::duration<double>(t2 - t1).count();
        }
    }
}
}  // namespace

extern "C" void or_payload_run(const or_grid* g, int32_t wrap, uint32_t sort_period, uint32_t n, uint32_t* id,
                               float* x, float* y, float* z, float* p, uint32_t steps, uint32_t first_step,
                               int32_t threads) {
    payload_impl(g, wrap, sort_period, n, id, x, y, z, p, steps, first_step, threads, nullptr, 0, nullptr);
}

extern "C" void or_payload_step_sampled(const or_grid* g, int32_t wrap, uint32_t n, uint32_t* id, float* x, float* y,
                                        float* z, float* p, uint32_t m, const uint32_t* sample, double* times) {
    payload_impl(g, wrap, 1, n, id, x, y, z, p, 1, 0, 1, sample, m, times);
}
