#ifndef INCLUDE_FLAMEGPU_RUNTIME_DEVICEAPI_CUH_
#define INCLUDE_FLAMEGPU_RUNTIME_DEVICEAPI_CUH_
// Header-only device API used inside FLAMEGPU_AGENT_FUNCTION bodies: agent
// variables, message input/output iterators (MessageNone, MessageBruteForce,
// MessageSpatial2D, MessageSpatial3D), agent output (birth), environment
// properties and random numbers. Mirrors the reference's device API
// (include/flamegpu/runtime/DeviceAPI.cuh:163-557,
// include/flamegpu/runtime/messaging/*/*Device.cuh) with the same names and
// iteration semantics; the storage behind it is the GB300 layout (sorted
// message records, per-function lookup tables).
#include <cstdint>
#include <type_traits>

#include "flamegpu/defines.h"
#include "flamegpu/detail/device_types.cuh"

#ifndef FLAMEGPU_SEATBELTS
#define FLAMEGPU_SEATBELTS 1
#endif

namespace flamegpu {

class MessageNone;
class MessageBruteForce;
class MessageSpatial2D;
class MessageSpatial3D;
class MessageArray;
class MessageArray2D;
class MessageArray3D;
class MessageBucket;

namespace detail {

#ifdef __CUDACC__
__device__ __forceinline__ void device_error(const LaunchParams& P, uint32_t code, uint32_t hash, uint32_t idx) {
    if (P.error) {
        if (atomicCAS(&P.error[0], 0u, code) == 0u) {
            P.error[1] = hash;
            P.error[2] = idx;
        }
        atomicAdd(&P.error[3], 1u);
    }
}

// The calling block's instance context (shared memory).
__device__ __forceinline__ InstanceCtx& ctx() {
    __shared__ InstanceCtx c;
    return c;
}

// Address of element `elem` of variable `hash` in row `row` of table `t`.
// Returns null (after recording a device error) when seatbelts are on and the
// name, the type size or the array index is wrong.
template <typename T>
__device__ __forceinline__ T* var_addr(const LaunchParams& P, const VarTable* __restrict__ t, uint32_t hash,
                                       uint32_t row, uint32_t elem) {
    // t points into the kernel's parameter space: plain loads, constant bank
    const uint32_t s = table_slot(t->mult, t->shift, hash);
    const VarSlot* vs = &t->slot[s];
    char* base = vs->ptr;
    const uint32_t stride = vs->stride;
#if FLAMEGPU_SEATBELTS
    if (vs->hash != hash) {
        device_error(P, kDevUnknownVariable, hash, row);
        return nullptr;
    }
    if (vs->elem_bytes != sizeof(T)) {
        device_error(P, kDevTypeMismatch, hash, row);
        return nullptr;
    }
    if (elem >= vs->elements) {
        device_error(P, kDevArrayIndex, hash, row);
        return nullptr;
    }
#endif
    return reinterpret_cast<T*>(base + static_cast<size_t>(row) * stride + static_cast<size_t>(elem) * sizeof(T));
}

template <typename T>
__device__ __forceinline__ T ldg_any(const T* p) {
    if constexpr (sizeof(T) == 4 || sizeof(T) == 8 || sizeof(T) == 2 || sizeof(T) == 1) {
        return __ldg(p);
    } else {
        return *p;
    }
}
template <>
__device__ __forceinline__ bool ldg_any<bool>(const bool* p) {
    return *p;
}

// Read-only read of a variable (messages, environment): non-coherent path.
template <typename T>
__device__ __forceinline__ T read_ro(const LaunchParams& P, const VarTable* t, uint32_t hash, uint32_t row,
                                     uint32_t elem = 0) {
    const T* a = var_addr<T>(P, t, hash, row, elem);
    return a ? ldg_any(a) : T{};
}
template <typename T>
__device__ __forceinline__ T read_rw(const LaunchParams& P, const VarTable* t, uint32_t hash, uint32_t row,
                                     uint32_t elem = 0) {
    const T* a = var_addr<T>(P, t, hash, row, elem);
    return a ? *a : T{};
}
template <typename T>
__device__ __forceinline__ void write_var(const LaunchParams& P, const VarTable* t, uint32_t hash, uint32_t row, T v,
                                          uint32_t elem = 0) {
    T* a = var_addr<T>(P, t, hash, row, elem);
    if (a) *a = v;
}

// SplitMix64 finaliser (Steele, Lea & Flood, OOPSLA 2014).
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

__device__ __forceinline__ int clamp_cell(int v, uint32_t dim) {
    const int d = static_cast<int>(dim);
    return v < 0 ? 0 : (v >= d ? d - 1 : v);
}
// getGridPosition3D / getGridPosition2D (MessageSpatial3DDevice.cuh:646-659)
__device__ __forceinline__ int grid_cell(const fg_spatial_grid& g, int axis, float p) {
    return clamp_cell(static_cast<int>(floorf((p - g.min[axis]) / g.radius)), g.gridDim[axis]);
}
// getHash3D / getHash2D (MessageSpatial3DDevice.cuh:660-672): x clamped
__device__ __forceinline__ uint32_t grid_hash(const fg_spatial_grid& g, int x, int y, int z) {
    const uint32_t ux = static_cast<uint32_t>(clamp_cell(x, g.gridDim[0]));
    return static_cast<uint32_t>(z) * g.gridDim[0] * g.gridDim[1] + static_cast<uint32_t>(y) * g.gridDim[0] + ux;
}
__device__ __forceinline__ float virtual_coord(float p1, float p2, float width) {
    // getVirtualX (MessageSpatial3DDevice.cuh:373-397): p2 - (d / |d|) * width
    // when |d| > width / 2. For the finite non-zero d of that branch, d / |d| is
    // exactly +-1 and width / 2 exactly width * 0.5, so the same value comes
    // from a sign copy, without the division.
    const float d = p2 - p1;
    return fabsf(d) > width * 0.5f ? p2 - copysignf(width, d) : p2;
}

// ---- shared-memory staging window of a block's spatial neighbourhood ----
// Layout of the dynamic shared memory: StageHeader (64 B) | PBM slice | records.
__device__ __forceinline__ char* dyn_smem() {
    extern __shared__ __align__(128) char fg_dyn_smem[];
    return fg_dyn_smem;
}
__device__ __forceinline__ StageHeader* stage_hdr() { return reinterpret_cast<StageHeader*>(dyn_smem()); }
__device__ __forceinline__ const uint32_t* stage_pbm() {
    return reinterpret_cast<const uint32_t*>(dyn_smem() + sizeof(StageHeader));
}
__device__ __forceinline__ const char* stage_records(const StageHeader* h) {
    return dyn_smem() + sizeof(StageHeader) + static_cast<size_t>(h->pbm_n) * 4u;
}

// PBM entry h of the input message list: from the staged slice when inside it.
__device__ __forceinline__ uint32_t pbm_at(const LaunchParams& P, uint32_t h) {
    if (P.stage_bytes) {
        const StageHeader* s = stage_hdr();
        const uint32_t r = h - s->pbm_lo;
        if (r < s->pbm_n) return stage_pbm()[r];
    }
    return __ldg(ctx().pbm + h);
}

// Read of a variable of message `index` of the input list: staged copy when
// the message is inside the block's window, else the sorted records in HBM.
template <typename T>
__device__ __forceinline__ T read_msg(const LaunchParams& P, uint32_t hash, uint32_t index, uint32_t elem) {
    const T* a = var_addr<T>(P, &P.T.msg_in, hash, index, elem);
    if (!a) return T{};
    if (P.stage_bytes) {
        const StageHeader* s = stage_hdr();
        const uint32_t r = index - s->rec_lo;
        if (r < s->rec_n) {
            const size_t row = static_cast<size_t>(index) * P.in_record_bytes;
            const size_t off = static_cast<size_t>(reinterpret_cast<const char*>(a) - P.in_records) - row;
            return *reinterpret_cast<const T*>(stage_records(s) + static_cast<size_t>(r) * P.in_record_bytes + off);
        }
    }
    return ldg_any(a);
}

// Byte offset of element `elem` of variable `hash` inside a sorted message
// record: a per-name constant of the launch (slot pointer minus records base).
template <typename T>
__device__ __forceinline__ size_t record_offset(const LaunchParams& P, uint32_t hash, uint32_t elem) {
    const VarTable* t = &P.T.msg_in;
    const VarSlot* vs = &t->slot[table_slot(t->mult, t->shift, hash)];
#if FLAMEGPU_SEATBELTS
    if (vs->hash != hash || vs->ptr == nullptr) {
        device_error(P, kDevUnknownVariable, hash, 0);
        return 0;
    }
    if (vs->elem_bytes != sizeof(T)) {
        device_error(P, kDevTypeMismatch, hash, 0);
        return 0;
    }
    if (elem >= vs->elements) {
        device_error(P, kDevArrayIndex, hash, 0);
        return 0;
    }
#endif
    return static_cast<size_t>(vs->ptr - P.in_records) + static_cast<size_t>(elem) * sizeof(T);
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Bounded wait on the staging mbarrier; false if it gave up.
__device__ __forceinline__ bool stage_wait(StageHeader* h, uint32_t phase) {
    const uint32_t mb = smem_addr(&h->mbar);
    for (uint32_t it = 0; it < (1u << 20); ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(mb), "r"(phase)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Stage the window of sorted messages every agent of this block can see:
// the bins between (lowest agent bin - one z/y/x slab) and (highest + one),
// a contiguous range of the sorted records, copied with TMA bulk copies
// (cp.async.bulk) completing on an mbarrier. All threads of the block call it.
template <int DIMS>
__device__ void stage_window(const LaunchParams& P, uint32_t idx, bool active, bool first) {
    __shared__ uint32_t s_min, s_max;
    StageHeader* h = stage_hdr();
    if (threadIdx.x == 0) {
        s_min = 0xFFFFFFFFu;
        s_max = 0u;
        if (first) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&h->mbar)) : "memory");
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
            h->phase = 0;
            h->off = 0;
        }
    }
    uint32_t key = 0xFFFFFFFFu, kmax = 0u;
    if (active) {
        const fg_spatial_grid& g = ctx().grid;
        const float x = read_rw<float>(P, &P.T.agent, VarName("x").hash, idx);
        const float y = read_rw<float>(P, &P.T.agent, VarName("y").hash, idx);
        const float z = DIMS == 3 ? read_rw<float>(P, &P.T.agent, VarName("z").hash, idx) : 0.0f;
        const int cx = clamp_cell(static_cast<int>(floorf((x - g.min[0]) / g.radius)), g.gridDim[0]);
        const int cy = clamp_cell(static_cast<int>(floorf((y - g.min[1]) / g.radius)), g.gridDim[1]);
        const int cz = DIMS == 3 ? clamp_cell(static_cast<int>(floorf((z - g.min[2]) / g.radius)), g.gridDim[2]) : 0;
        key = static_cast<uint32_t>(cz) * g.gridDim[0] * g.gridDim[1] + static_cast<uint32_t>(cy) * g.gridDim[0] +
              static_cast<uint32_t>(cx);
        kmax = key;
    }
    key = __reduce_min_sync(0xFFFFFFFFu, key);
    kmax = __reduce_max_sync(0xFFFFFFFFu, kmax);
    __syncthreads();  // everyone is done with the previous window; s_min/s_max initialised
    if ((threadIdx.x & 31u) == 0) {
        atomicMin(&s_min, key);
        atomicMax(&s_max, kmax);
    }
    __syncthreads();
    uint32_t tx = 0;
    if (threadIdx.x == 0) {
        h->rec_n = 0;
        h->pbm_n = 0;
        h->rec_lo = 0;
        h->pbm_lo = 0;
        // after a wait that gave up, copies of that window may still land on
        // the mbarrier and in the buffer: the block reads from HBM from then on
        if (s_min != 0xFFFFFFFFu && !h->off) {
            const fg_spatial_grid& g = ctx().grid;
            const uint32_t* pbm = ctx().pbm;
            const uint32_t B = g.binCount;
            const uint32_t span = DIMS == 3 ? g.gridDim[0] * g.gridDim[1] + g.gridDim[0] + 1u : g.gridDim[0] + 1u;
            const uint32_t hlo = s_min > span ? s_min - span : 0u;
            const uint32_t hhi = (s_max + span < B) ? s_max + span : B - 1u;
            const uint32_t plo = hlo & ~3u;
            uint32_t pend = (hhi + 2u + 3u) & ~3u;
            if (pend > ctx().pbm_alloc) pend = ctx().pbm_alloc;
            const uint32_t pn = pend - plo;
            const uint32_t rlo = __ldg(pbm + hlo), rhi = __ldg(pbm + hhi + 1u);
            const size_t pbytes = static_cast<size_t>(pn) * 4u;
            const size_t rbytes = static_cast<size_t>(rhi - rlo) * P.in_record_bytes;
            // bulk copies need 16-byte aligned addresses and sizes; anything else
            // (a caller's layout mistake) is not staged: reads then go to HBM
            const bool aligned = ((pbytes | rbytes) & 15u) == 0 &&
                                 (reinterpret_cast<uintptr_t>(pbm + plo) & 15u) == 0 &&
                                 (reinterpret_cast<uintptr_t>(P.in_records) & 15u) == 0 &&
                                 (P.in_record_bytes & 15u) == 0;
            if (aligned && pbytes + rbytes <= P.stage_bytes && pn > 0) {
                h->pbm_lo = plo;
                h->pbm_n = pn;
                h->rec_lo = rlo;
                h->rec_n = rhi - rlo;
                tx = static_cast<uint32_t>(pbytes + rbytes);
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                const uint32_t mb = smem_addr(&h->mbar);
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(tx) : "memory");
                // PBM slice, then the records, in chunks of at most 32 KiB
                auto copy = [&](char* dst, const char* src, size_t bytes) {
                    while (bytes) {
                        const uint32_t c = bytes > 32768 ? 32768u : static_cast<uint32_t>(bytes);
                        asm volatile(
                            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                                smem_addr(dst)),
                            "l"(src), "r"(c), "r"(mb)
                            : "memory");
                        dst += c;
                        src += c;
                        bytes -= c;
                    }
                };
                char* base = dyn_smem() + sizeof(StageHeader);
                copy(base, reinterpret_cast<const char*>(pbm + plo), pbytes);
                if (rbytes) copy(base + pbytes, P.in_records + static_cast<size_t>(rlo) * P.in_record_bytes, rbytes);
            }
        }
        h->pad[0] = tx;
    }
    __syncthreads();
    if (h->pad[0]) {
        const uint32_t phase = h->phase;
        // a copy that has not landed after the bounded wait is waited for once
        // more (bounded), then the window is dropped and staging is switched
        // off for the rest of this block: reads fall back to HBM
        bool ok = stage_wait(h, phase);
        if (!ok) ok = stage_wait(h, phase);
        __syncthreads();
        if (threadIdx.x == 0) {
            h->phase = phase ^ 1u;
            if (!ok) {
                device_error(P, kDevStageTimeout, 0, idx);
                h->rec_n = 0;
                h->pbm_n = 0;
                h->off = 1;
            }
        }
    }
    __syncthreads();
}
#endif  // __CUDACC__

}  // namespace detail

#ifdef __CUDACC__

// ------------------------------------------------------------------ messages

/** No message input/output (include/flamegpu/runtime/messaging/MessageNone.h). */
class MessageNone {
 public:
    class Description;
    class In {
     public:
        __device__ explicit In(const detail::LaunchParams&) {}
    };
    class Out {
     public:
        __device__ Out(const detail::LaunchParams&, uint32_t) {}
        __device__ uint32_t written() const { return 0; }
    };
};

/** Output half shared by every message type (MessageBruteForceDevice.cuh:259-294). */
class MessageOutBase {
 public:
    __device__ MessageOutBase(const detail::LaunchParams& p, uint32_t idx) : P(p), index(idx) {}
    template <typename T>
    __device__ void setVariable(detail::VarName name, T value) const {
        if (!P.msg_out_enabled) {
            detail::device_error(P, detail::kDevMessageOutNotEnabled, name.hash, index);
            return;
        }
        detail::write_var<T>(P, &P.T.msg_out, name.hash, index, value);
        flag = 1;
        if constexpr (std::is_same<T, float>::value) {  // the location, kept for the launch's epilogue
            if (name.hash == detail::VarName("x").hash) loc[0] = value;
            if (name.hash == detail::VarName("y").hash) loc[1] = value;
            if (name.hash == detail::VarName("z").hash) loc[2] = value;
        }
    }
    template <typename T, flamegpu::size_type N>
    __device__ void setVariable(detail::VarName name, unsigned int i, T value) const {
        if (!P.msg_out_enabled) {
            detail::device_error(P, detail::kDevMessageOutNotEnabled, name.hash, index);
            return;
        }
        detail::write_var<T>(P, &P.T.msg_out, name.hash, index, value, i);
        flag = 1;
    }
    __device__ uint32_t written() const { return flag; }
    /** The message's x, y, z as last set (spatial messages). */
    __device__ float location(int a) const { return loc[a]; }

 protected:
    const detail::LaunchParams& P;
    uint32_t index;
    mutable uint32_t flag = 0;
    mutable float loc[3] = {0.0f, 0.0f, 0.0f};
};

/** Message in an input list, addressed by its (sorted) index. */
class MessageView {
 public:
    __device__ MessageView(const detail::LaunchParams& p, uint32_t i) : P(p), index(i) {}
    template <typename T>
    __device__ T getVariable(detail::VarName name) const {
        return detail::read_msg<T>(P, name.hash, index, 0);
    }
    template <typename T, flamegpu::size_type N>
    __device__ T getVariable(detail::VarName name, unsigned int i) const {
        return detail::read_msg<T>(P, name.hash, index, i);
    }
    __device__ uint32_t getIndex() const { return index; }

 protected:
    const detail::LaunchParams& P;

 public:
    uint32_t index;
};

/** Every message of the list (MessageBruteForceDevice.cuh:19-172,222-257). */
class MessageBruteForce {
 public:
    class Description;
    class Out : public MessageOutBase {
     public:
        __device__ Out(const detail::LaunchParams& p, uint32_t idx) : MessageOutBase(p, idx) {}
    };
    class In {
     public:
        class Message : public MessageView {
         public:
            __device__ Message(const detail::LaunchParams& p, uint32_t i) : MessageView(p, i) {}
        };
        class iterator {
         public:
            __device__ iterator(const detail::LaunchParams& p, uint32_t i) : m(p, i) {}
            __device__ iterator& operator++() {
                ++m.index;
                return *this;
            }
            __device__ bool operator!=(const iterator& o) const { return m.index != o.m.index; }
            __device__ bool operator==(const iterator& o) const { return m.index == o.m.index; }
            __device__ const Message& operator*() const { return m; }
            __device__ const Message* operator->() const { return &m; }

         private:
            Message m;
        };
        __device__ explicit In(const detail::LaunchParams& p) : P(p), len(p.in_count ? *p.in_count : 0u) {}
        __device__ iterator begin() const { return iterator(P, 0); }
        __device__ iterator end() const { return iterator(P, len); }
        __device__ uint32_t size() const { return len; }

     private:
        const detail::LaunchParams& P;
        uint32_t len;
    };
};


/**
 * Array messages (MessageArrayDevice.cuh, MessageArray2DDevice.cuh,
 * MessageArray3DDevice.cuh): the input list is the array itself, index
 * x + dim_x * (y + dim_y * z), holding the message output to that index this
 * step or zeros. A search iterates the Moore (or von Neumann, |dx| + |dy| +
 * |dz| <= radius) neighbourhood of a cell, origin excluded, x offset outermost
 * and z innermost, clamped to the array or wrapped around it.
 */
template <int D>
class ArrayIn {
 public:
    /** A message of the array (at(), or a neighbour of a search; an index past
     *  the array is an invalid message whose variables read 0). */
    class Message : public MessageView {
     public:
        __device__ Message(const detail::LaunchParams& p, uint32_t i, int ox = 0, int oy = 0, int oz = 0)
            : MessageView(p, i), off{ox, oy, oz} {}
        template <typename T>
        __device__ T getVariable(detail::VarName name) const {
            if (index >= P.in_dims[0] * P.in_dims[1] * P.in_dims[2]) {
                detail::device_error(P, detail::kDevArrayMessage, name.hash, index);
                return T{};
            }
            return MessageView::getVariable<T>(name);
        }
        template <typename T, flamegpu::size_type N>
        __device__ T getVariable(detail::VarName name, unsigned int i) const {
            if (index >= P.in_dims[0] * P.in_dims[1] * P.in_dims[2]) {
                detail::device_error(P, detail::kDevArrayMessage, name.hash, index);
                return T{};
            }
            return MessageView::getVariable<T, N>(name, i);
        }
        __device__ uint32_t getX() const { return index % P.in_dims[0]; }
        __device__ uint32_t getY() const { return (index / P.in_dims[0]) % P.in_dims[1]; }
        __device__ uint32_t getZ() const { return index / (P.in_dims[0] * P.in_dims[1]); }
        __device__ int getOffsetX() const { return off[0]; }
        __device__ int getOffsetY() const { return off[1]; }
        __device__ int getOffsetZ() const { return off[2]; }

     private:
        int off[3];
    };

    /** The neighbourhood of loc within radius: clamped to the array (WRAP
     *  false) or wrapped around it, Moore (VN false) or von Neumann. */
    template <bool WRAP, bool VN>
    class Filter {
     public:
        class iterator {
         public:
            __device__ iterator(const Filter& f, bool at_end) : F(f) {
                for (int a = 0; a < 3; ++a) d[a] = F.lo[a];
                if (at_end || F.empty) {
                    d[0] = F.hi[0] + 1;
                    return;
                }
                skip();
            }
            __device__ iterator& operator++() {
                step();
                skip();
                return *this;
            }
            __device__ bool operator!=(const iterator& o) const { return d[0] != o.d[0] || d[1] != o.d[1] || d[2] != o.d[2]; }
            __device__ bool operator==(const iterator& o) const { return !(*this != o); }
            __device__ Message operator*() const {
                uint32_t idx = 0, mul = 1;
                for (int a = 0; a < D; ++a) {
                    const int dim = static_cast<int>(F.P.in_dims[a]);
                    int c = static_cast<int>(F.loc[a]) + d[a];
                    if (WRAP) c = (c % dim + dim) % dim;
                    idx += static_cast<uint32_t>(c) * mul;
                    mul *= static_cast<uint32_t>(dim);
                }
                return Message(F.P, idx, d[0], d[1], d[2]);
            }

         private:
            // next offset: the innermost axis first
            __device__ void step() {
                for (int a = D - 1; a >= 0; --a) {
                    if (d[a] < F.hi[a] || a == 0) {
                        ++d[a];
                        return;
                    }
                    d[a] = F.lo[a];
                }
            }
            // past the origin and, for von Neumann, the cells beyond the radius
            __device__ void skip() {
                while (d[0] <= F.hi[0]) {
                    const int manhattan = abs(d[0]) + abs(d[1]) + abs(d[2]);
                    if (manhattan != 0 && (!VN || manhattan <= F.radius)) return;
                    step();
                }
            }
            const Filter& F;
            int d[3];
        };
        __device__ Filter(const detail::LaunchParams& p, const uint32_t (&l)[3], uint32_t r, bool bad)
            : P(p), radius(static_cast<int>(r)), empty(bad) {
            for (int a = 0; a < 3; ++a) {
                loc[a] = l[a];
                if (a >= D) {
                    lo[a] = hi[a] = 0;
                } else if (WRAP) {
                    lo[a] = -radius;
                    hi[a] = radius;
                } else {
                    const int x = static_cast<int>(l[a]), dim = static_cast<int>(p.in_dims[a]);
                    lo[a] = x - radius < 0 ? -x : -radius;
                    hi[a] = x + radius >= dim ? dim - 1 - x : radius;
                }
            }
        }
        __device__ iterator begin() const { return iterator(*this, false); }
        __device__ iterator end() const { return iterator(*this, true); }

        const detail::LaunchParams& P;
        uint32_t loc[3];
        int lo[3], hi[3];
        int radius;
        bool empty;
    };

    __device__ explicit ArrayIn(const detail::LaunchParams& p) : P(p) {}
    __device__ uint32_t getDimX() const { return P.in_dims[0]; }
    __device__ uint32_t getDimY() const { return P.in_dims[1]; }
    __device__ uint32_t getDimZ() const { return P.in_dims[2]; }
    __device__ uint32_t size() const { return P.in_dims[0] * P.in_dims[1] * P.in_dims[2]; }

 protected:
    // The message at loc (an invalid one, reading 0, outside the array).
    __device__ Message at_loc(const uint32_t (&l)[3]) const {
        bool out = false;
        for (int a = 0; a < D; ++a) out = out || l[a] >= P.in_dims[a];
        if (out) {
#if FLAMEGPU_SEATBELTS
            detail::device_error(P, detail::kDevArrayMessage, 0, 0);
#endif
            return Message(P, size());
        }
        return Message(P, l[0] + P.in_dims[0] * (l[1] + P.in_dims[1] * l[2]));
    }
    // Whether a search at loc within radius is invalid (MessageArray2DDevice.cuh:1013-1025,
    // :1043-1058): radius 0, an origin outside the array, or for a wrapped
    // search a diameter wider than the array (cells would be read twice).
    __device__ bool bad_search(const uint32_t (&l)[3], uint32_t radius, bool wrap) const {
        bool bad = radius == 0;
        for (int a = 0; a < D; ++a) {
            bad = bad || l[a] >= P.in_dims[a];
            if (wrap) bad = bad || 2u * radius + 1u > P.in_dims[a];
        }
#if FLAMEGPU_SEATBELTS
        if (bad) detail::device_error(P, detail::kDevArrayMessage, 0, radius);
#endif
        return bad;
    }
    template <bool WRAP, bool VN>
    __device__ Filter<WRAP, VN> search(const uint32_t (&l)[3], uint32_t radius) const {
        return Filter<WRAP, VN>(P, l, radius, bad_search(l, radius, WRAP));
    }
    const detail::LaunchParams& P;
};

/** Output half of the array messages: setIndex places the message. */
template <int D>
class ArrayOut : public MessageOutBase {
 public:
    __device__ ArrayOut(const detail::LaunchParams& p, uint32_t idx) : MessageOutBase(p, idx) {}
    /** Whether setIndex was called: the message is output (MessageArray2DDevice.cuh:1360-1375). */
    __device__ uint32_t written() const { return index_set; }

 protected:
    __device__ void set_index(const uint32_t (&l)[3]) const {
        bool out = false;
        for (int a = 0; a < D; ++a) out = out || l[a] >= P.out_dims[a];
        if (out) {
            detail::device_error(P, detail::kDevArrayMessage, 0, index);
            return;
        }
        detail::write_var<uint32_t>(P, &P.T.msg_out, detail::VarName("___INDEX").hash, index,
                                    l[0] + P.out_dims[0] * (l[1] + P.out_dims[1] * l[2]));
        index_set = 1;
    }
    mutable uint32_t index_set = 0;
};

class MessageArray {
 public:
    class Description;
    class In : public ArrayIn<1> {
     public:
        __device__ explicit In(const detail::LaunchParams& p) : ArrayIn<1>(p) {}
        __device__ Message at(uint32_t x) const { return at_loc({x, 0u, 0u}); }
        __device__ Filter<false, false> operator()(uint32_t x, uint32_t radius = 1) const {
            return search<false, false>({x, 0u, 0u}, radius);
        }
        __device__ Filter<true, false> wrap(uint32_t x, uint32_t radius = 1) const {
            return search<true, false>({x, 0u, 0u}, radius);
        }
    };
    class Out : public ArrayOut<1> {
     public:
        __device__ Out(const detail::LaunchParams& p, uint32_t idx) : ArrayOut<1>(p, idx) {}
        __device__ void setIndex(uint32_t x) const { set_index({x, 0u, 0u}); }
    };
};

class MessageArray2D {
 public:
    class Description;
    class In : public ArrayIn<2> {
     public:
        __device__ explicit In(const detail::LaunchParams& p) : ArrayIn<2>(p) {}
        __device__ Message at(uint32_t x, uint32_t y) const { return at_loc({x, y, 0u}); }
        __device__ Filter<false, false> operator()(uint32_t x, uint32_t y, uint32_t radius = 1) const {
            return search<false, false>({x, y, 0u}, radius);
        }
        __device__ Filter<true, false> wrap(uint32_t x, uint32_t y, uint32_t radius = 1) const {
            return search<true, false>({x, y, 0u}, radius);
        }
        __device__ Filter<false, true> vn(uint32_t x, uint32_t y, uint32_t radius = 1) const {
            return search<false, true>({x, y, 0u}, radius);
        }
        __device__ Filter<true, true> vn_wrap(uint32_t x, uint32_t y, uint32_t radius = 1) const {
            return search<true, true>({x, y, 0u}, radius);
        }
    };
    class Out : public ArrayOut<2> {
     public:
        __device__ Out(const detail::LaunchParams& p, uint32_t idx) : ArrayOut<2>(p, idx) {}
        __device__ void setIndex(uint32_t x, uint32_t y) const { set_index({x, y, 0u}); }
    };
};

class MessageArray3D {
 public:
    class Description;
    class In : public ArrayIn<3> {
     public:
        __device__ explicit In(const detail::LaunchParams& p) : ArrayIn<3>(p) {}
        __device__ Message at(uint32_t x, uint32_t y, uint32_t z) const { return at_loc({x, y, z}); }
        __device__ Filter<false, false> operator()(uint32_t x, uint32_t y, uint32_t z, uint32_t radius = 1) const {
            return search<false, false>({x, y, z}, radius);
        }
        __device__ Filter<true, false> wrap(uint32_t x, uint32_t y, uint32_t z, uint32_t radius = 1) const {
            return search<true, false>({x, y, z}, radius);
        }
        __device__ Filter<false, true> vn(uint32_t x, uint32_t y, uint32_t z, uint32_t radius = 1) const {
            return search<false, true>({x, y, z}, radius);
        }
        __device__ Filter<true, true> vn_wrap(uint32_t x, uint32_t y, uint32_t z, uint32_t radius = 1) const {
            return search<true, true>({x, y, z}, radius);
        }
    };
    class Out : public ArrayOut<3> {
     public:
        __device__ Out(const detail::LaunchParams& p, uint32_t idx) : ArrayOut<3>(p, idx) {}
        __device__ void setIndex(uint32_t x, uint32_t y, uint32_t z) const { set_index({x, y, z}); }
    };
};

/**
 * Bucket messages (MessageBucketDevice.cuh): each message carries an integer
 * key in [lowerBound, upperBound]; the input iterates the messages of one key,
 * or of the keys [begin, end), in the order they were output.
 */
class MessageBucket {
 public:
    class Description;
    class In {
     public:
        class Message : public MessageView {
         public:
            __device__ Message(const detail::LaunchParams& p, uint32_t i) : MessageView(p, i) {}
        };
        class Filter {
         public:
            class iterator {
             public:
                __device__ iterator(const detail::LaunchParams& p, uint32_t i) : m(p, i) {}
                __device__ iterator& operator++() {
                    ++m.index;
                    return *this;
                }
                __device__ bool operator!=(const iterator& o) const { return m.index != o.m.index; }
                __device__ bool operator==(const iterator& o) const { return m.index == o.m.index; }
                __device__ const Message& operator*() const { return m; }
                __device__ const Message* operator->() const { return &m; }

             private:
                Message m;
            };
            __device__ Filter(const detail::LaunchParams& p, uint32_t b, uint32_t e) : P(p), first(b), last(e) {}
            __device__ iterator begin() const { return iterator(P, first); }
            __device__ iterator end() const { return iterator(P, last); }
            __device__ uint32_t size() const { return last - first; }

         private:
            const detail::LaunchParams& P;
            uint32_t first, last;
        };
        __device__ explicit In(const detail::LaunchParams& p) : P(p) {}
        /** The messages of one key (MessageBucketDevice.cuh:207-221). */
        __device__ Filter operator()(int32_t key) const {
            if (key < P.in_key_lo || key >= P.in_key_hi) {
                detail::device_error(P, detail::kDevBucketMessage, 0, static_cast<uint32_t>(key));
                return Filter(P, 0, 0);
            }
            const uint32_t k = static_cast<uint32_t>(key - P.in_key_lo);
            return Filter(P, __ldg(P.in_pbm + k), __ldg(P.in_pbm + k + 1));
        }
        /** The messages of the keys [beginKey, endKey) (:228-245). */
        __device__ Filter operator()(int32_t beginKey, int32_t endKey) const {
            if (beginKey < P.in_key_lo || endKey > P.in_key_hi || endKey <= beginKey) {
                detail::device_error(P, detail::kDevBucketMessage, 0, static_cast<uint32_t>(beginKey));
                return Filter(P, 0, 0);
            }
            return Filter(P, __ldg(P.in_pbm + (beginKey - P.in_key_lo)), __ldg(P.in_pbm + (endKey - P.in_key_lo)));
        }

     private:
        const detail::LaunchParams& P;
    };
    class Out : public MessageOutBase {
     public:
        __device__ Out(const detail::LaunchParams& p, uint32_t idx) : MessageOutBase(p, idx) {}
        /** The message's key (MessageBucketDevice.cuh:275-290); a key outside the bounds is a device error. */
        __device__ void setKey(int32_t key) const {
            if (key < P.out_key_lo || key >= P.out_key_hi) {
                detail::device_error(P, detail::kDevBucketMessage, 0, index);
                return;
            }
            detail::write_var<int32_t>(P, &P.T.msg_out, detail::VarName("___KEY").hash, index, key);
            key_set = 1;
        }
        /** Whether setKey was called: the message is output. */
        __device__ uint32_t written() const { return key_set; }

     private:
        mutable uint32_t key_set = 0;
    };
};

/**
 * A message of a spatial input list: a view of its sorted record. `row` is
 * the record's address — in the block's shared-memory window when the
 * message is inside it, else in HBM — computed once per message by the
 * iterator; a field read is then one load at row + field offset, the offset
 * being a per-name constant of the launch. Every spatial record starts with
 * its location (x, y and, in 3D, z: the message type's first variables) and
 * is 16-byte aligned, so with device checks off those reads use constant
 * offsets from an aligned address, which the compiler can fold and merge;
 * every other field's offset is arithmetic on launch constants (its slot in
 * the record's own perfect hash), which the compiler hoists out of the loop.
 * With device checks on, reads go through the checked name table, whose
 * entries point at the same fields.
 */
template <int DIMS>
class RecordView {
 public:
    __device__ RecordView(const detail::LaunchParams& p, uint32_t i) : P(p), index(i), row(nullptr) {}
    template <typename T>
    __device__ T getVariable(detail::VarName name) const {
#if !FLAMEGPU_SEATBELTS
        const char* r = static_cast<const char*>(__builtin_assume_aligned(row, 16));
        if constexpr (sizeof(T) == 4) {
            if (name.hash == detail::VarName("x").hash) return *reinterpret_cast<const T*>(r);
            if (name.hash == detail::VarName("y").hash) return *reinterpret_cast<const T*>(r + 4);
            if (DIMS == 3 && name.hash == detail::VarName("z").hash) return *reinterpret_cast<const T*>(r + 8);
        }
        return *reinterpret_cast<const T*>(r + payload_offset(name.hash));
#else
        return *reinterpret_cast<const T*>(row + detail::record_offset<T>(P, name.hash, 0));
#endif
    }
    template <typename T, flamegpu::size_type N>
    __device__ T getVariable(detail::VarName name, unsigned int i) const {
#if !FLAMEGPU_SEATBELTS
        return *reinterpret_cast<const T*>(row + payload_offset(name.hash) + static_cast<size_t>(i) * sizeof(T));
#else
        return *reinterpret_cast<const T*>(row + detail::record_offset<T>(P, name.hash, i));
#endif
    }
    __device__ uint32_t getIndex() const { return index; }

 protected:
    // byte offset of a non-location field: arithmetic on launch constants only
    // (the slot of the name in the record's perfect hash), so the compiler
    // computes it once outside the neighbour loop
    __device__ __forceinline__ uint32_t payload_offset(uint32_t hash) const {
        return 4u * DIMS + detail::table_slot(P.in_pay_mult, P.in_pay_shift, hash) * P.in_pay_stride;
    }
    const detail::LaunchParams& P;

 public:
    uint32_t index;
    const char* row;
};

/**
 * Spatially partitioned messages; the iterators visit the reference's
 * Moore neighbourhood in the reference's order. DIMS = 2 or 3.
 * Filter: 3^(DIMS-1) x-strips, y-offset outer, z-offset inner, each strip
 * PBM[hash(x-1)] .. PBM[hash(x+1)+1] with x clamped (MessageSpatial3DDevice.cuh:693-719).
 * WrapFilter: 3^DIMS single bins, x offset outer, then y, z offset inner
 * (nextCell, MessageSpatial3DDevice.cuh:264-276), every axis taken modulo
 * gridDim (:727-749); no radius test — user code filters.
 * Both iterators first read the PBM bounds of all their strips or cells in
 * lock step (unrolled, so every hash is a sum of registers) and keep one bit
 * per non-empty one; they then visit only those, in order, loading the next
 * one's bounds while the current one is being read. A lane whose strip or
 * cell ends thus moves to the next non-empty one in one step, so the lanes of
 * a warp advance at most once per message visited instead of each stepping
 * through empty cells on its own (in sparse neighbourhoods most are empty).
 * A cell lies wholly inside or wholly outside the block's staged window, so
 * within a cell the record address just advances by one record.
 */
__device__ __forceinline__ uint32_t pick(int r, uint32_t a, uint32_t b, uint32_t c) {
    return r == 0 ? a : (r == 1 ? b : c);
}

/** The staged window of the calling block, cached in registers by a filter. */
struct Window {
    uint32_t rec_lo = 0, rec_n = 0, pbm_lo = 0, pbm_n = 0;
    const char* rec = nullptr;
    const uint32_t* pbm = nullptr;
    const uint32_t* gpbm = nullptr;  // the instance's PBM in HBM
    __device__ void load(const detail::LaunchParams& P) {
        gpbm = detail::ctx().pbm;
        if (!P.stage_bytes) return;
        const detail::StageHeader* h = detail::stage_hdr();
        rec_lo = h->rec_lo;
        rec_n = h->rec_n;
        pbm_lo = h->pbm_lo;
        pbm_n = h->pbm_n;
        pbm = detail::stage_pbm();
        rec = detail::stage_records(h);
    }
    __device__ uint32_t pbm_at(const detail::LaunchParams& P, uint32_t h) const {
        const uint32_t r = h - pbm_lo;
        return r < pbm_n ? pbm[r] : __ldg(gpbm + h);
    }
    __device__ const char* row(const detail::LaunchParams& P, uint32_t index) const {
        const uint32_t r = index - rec_lo;
        return r < rec_n ? rec + static_cast<size_t>(r) * P.in_record_bytes
                         : P.in_records + static_cast<size_t>(index) * P.in_record_bytes;
    }
};

template <int DIMS>
class SpatialIn {
 public:
    static constexpr int kStrips = DIMS == 3 ? 9 : 3;
    static constexpr int kCells = DIMS == 3 ? 27 : 9;

    class Filter {
     public:
        class Message : public RecordView<DIMS> {
         public:
            __device__ Message(const detail::LaunchParams& p, uint32_t i) : RecordView<DIMS>(p, i) {}
        };
        class iterator {
         public:
            __device__ iterator(const Filter& f, bool at_end) : F(f), m(f.P, 0), end_(0) {
                if (at_end) return;
#pragma unroll
                for (int t = 0; t < kStrips; ++t) {
                    uint32_t b, e;
                    bounds(t, b, e);
                    todo_ |= (b < e ? 1u : 0u) << t;
                }
                prefetch();
                advance();
            }
            __device__ iterator& operator++() {
                m.row += F.P.in_record_bytes;
                if (++m.index >= end_) advance();
                return *this;
            }
            __device__ bool operator!=(const iterator&) const { return m.index < end_; }
            __device__ bool operator==(const iterator& o) const { return !(*this != o); }
            __device__ const Message& operator*() const { return m; }
            __device__ const Message* operator->() const { return &m; }

         private:
            // PBM bounds of strip t (empty when the strip lies outside the grid)
            __device__ void bounds(int t, uint32_t& b, uint32_t& e) const {
                b = e = 0;
                const int ry = DIMS == 3 ? t / 3 - 1 : t - 1;
                const int rz = DIMS == 3 ? t % 3 - 1 : 0;
                const int ay = F.cell[1] + ry, az = F.cell[2] + rz;
                const fg_spatial_grid& g = detail::ctx().grid;
                if (ay < 0 || ay >= static_cast<int>(g.gridDim[1])) return;
                if (DIMS == 3 && (az < 0 || az >= static_cast<int>(g.gridDim[2]))) return;
                const uint32_t h0 = detail::grid_hash(g, F.cell[0] - 1, ay, az);
                const uint32_t h1 = detail::grid_hash(g, F.cell[0] + 1, ay, az);
                b = F.win.pbm_at(F.P, h0);
                e = F.win.pbm_at(F.P, h1 + 1);
            }
            // bounds of the next non-empty strip (an empty pair when none is left)
            __device__ void prefetch() {
                nb_ = ne_ = 0;
                if (todo_) {
                    const int t = __ffs(todo_) - 1;
                    todo_ &= todo_ - 1u;
                    bounds(t, nb_, ne_);
                }
            }
            // enter the prefetched strip (index == end ends the loop)
            __device__ void advance() {
                m.index = nb_;
                m.row = F.win.row(F.P, nb_);
                end_ = ne_;
                prefetch();  // in flight while this strip is read
            }
            const Filter& F;
            Message m;
            uint32_t end_;
            uint32_t todo_ = 0;         // non-empty strips not yet entered
            uint32_t nb_ = 0, ne_ = 0;  // bounds of the next one
        };
        __device__ Filter(const detail::LaunchParams& p, float x, float y, float z) : P(p) {
            loc[0] = x;
            loc[1] = y;
            loc[2] = z;
            const fg_spatial_grid& gc = detail::ctx().grid;
            cell[0] = detail::grid_cell(gc, 0, x);
            cell[1] = detail::grid_cell(gc, 1, y);
            cell[2] = DIMS == 3 ? detail::grid_cell(gc, 2, z) : 0;
            win.load(p);
        }
        __device__ iterator begin() const { return iterator(*this, false); }
        __device__ iterator end() const { return iterator(*this, true); }

        const detail::LaunchParams& P;
        float loc[3];
        int cell[3];
        Window win;
    };

    class WrapFilter {
     public:
        class Message : public RecordView<DIMS> {
         public:
            __device__ Message(const detail::LaunchParams& p, uint32_t i, const WrapFilter* f)
                : RecordView<DIMS>(p, i), F(f) {}
            __device__ float getVirtualX() const { return getVirtualX(F->loc[0]); }
            __device__ float getVirtualY() const { return getVirtualY(F->loc[1]); }
            __device__ float getVirtualZ() const { return getVirtualZ(F->loc[2]); }
            __device__ float getVirtualX(float x1) const {
                return detail::virtual_coord(x1, this->template getVariable<float>("x"),
                                             detail::ctx().grid.width[0]);
            }
            __device__ float getVirtualY(float y1) const {
                return detail::virtual_coord(y1, this->template getVariable<float>("y"),
                                             detail::ctx().grid.width[1]);
            }
            __device__ float getVirtualZ(float z1) const {
                return detail::virtual_coord(z1, this->template getVariable<float>("z"),
                                             detail::ctx().grid.width[2]);
            }

         private:
            const WrapFilter* F;
        };
        class iterator {
         public:
            __device__ iterator(const WrapFilter& f, bool at_end) : F(f), m(f.P, 0, &f), end_(0) {
                if (at_end) return;
#pragma unroll
                for (int t = 0; t < kCells; ++t) {
                    const uint32_t h = hash(t);
                    todo_ |= (F.win.pbm_at(F.P, h) < F.win.pbm_at(F.P, h + 1) ? 1u : 0u) << t;
                }
                prefetch();
                advance();
            }
            __device__ iterator& operator++() {
                m.row += F.P.in_record_bytes;
                if (++m.index >= end_) advance();
                return *this;
            }
            __device__ bool operator!=(const iterator&) const { return m.index < end_; }
            __device__ bool operator==(const iterator& o) const { return !(*this != o); }
            __device__ const Message& operator*() const { return m; }
            __device__ const Message* operator->() const { return &m; }

         private:
            // hash of cell t of the visit order (x offset outer, z inner)
            __device__ uint32_t hash(int t) const {
                if (DIMS == 3)
                    return pick(t / 9, F.hx0, F.hx1, F.hx2) + pick((t / 3) % 3, F.hy0, F.hy1, F.hy2) +
                           pick(t % 3, F.hz0, F.hz1, F.hz2);
                return pick(t / 3, F.hx0, F.hx1, F.hx2) + pick(t % 3, F.hy0, F.hy1, F.hy2);
            }
            // bounds of the next non-empty cell (an empty pair when none is left)
            __device__ void prefetch() {
                nb_ = ne_ = 0;
                if (todo_) {
                    const int t = __ffs(todo_) - 1;
                    todo_ &= todo_ - 1u;
                    const uint32_t h = hash(t);
                    nb_ = F.win.pbm_at(F.P, h);
                    ne_ = F.win.pbm_at(F.P, h + 1);
                }
            }
            // enter the prefetched cell (index == end ends the loop)
            __device__ void advance() {
                m.index = nb_;
                m.row = F.win.row(F.P, nb_);
                end_ = ne_;
                prefetch();  // in flight while this cell is read
            }
            const WrapFilter& F;
            Message m;
            uint32_t end_;
            uint32_t todo_ = 0;         // non-empty cells not yet entered
            uint32_t nb_ = 0, ne_ = 0;  // bounds of the next one
        };
        __device__ WrapFilter(const detail::LaunchParams& p, float x, float y, float z) : P(p) {
            loc[0] = x;
            loc[1] = y;
            loc[2] = z;
            const fg_spatial_grid& gc = detail::ctx().grid;
            cell[0] = detail::grid_cell(gc, 0, x);
            cell[1] = detail::grid_cell(gc, 1, y);
            cell[2] = DIMS == 3 ? detail::grid_cell(gc, 2, z) : 0;
            // wrapped coordinates of the offsets -1, 0, +1 on each axis (modulo gridDim,
            // MessageSpatial3DDevice.cuh:736-738), pre-multiplied into hash terms.
            const fg_spatial_grid& g = detail::ctx().grid;
            auto wrapc = [](int c, int r, uint32_t d) {
                return static_cast<uint32_t>(c + r + static_cast<int>(d)) % d;
            };
            hx0 = wrapc(cell[0], -1, g.gridDim[0]);
            hx1 = wrapc(cell[0], 0, g.gridDim[0]);
            hx2 = wrapc(cell[0], 1, g.gridDim[0]);
            hy0 = wrapc(cell[1], -1, g.gridDim[1]) * g.gridDim[0];
            hy1 = wrapc(cell[1], 0, g.gridDim[1]) * g.gridDim[0];
            hy2 = wrapc(cell[1], 1, g.gridDim[1]) * g.gridDim[0];
            if (DIMS == 3) {
                const uint32_t s2 = g.gridDim[0] * g.gridDim[1];
                hz0 = wrapc(cell[2], -1, g.gridDim[2]) * s2;
                hz1 = wrapc(cell[2], 0, g.gridDim[2]) * s2;
                hz2 = wrapc(cell[2], 1, g.gridDim[2]) * s2;
            } else {
                hz0 = hz1 = hz2 = 0;
            }
            win.load(p);
        }
        __device__ iterator begin() const { return iterator(*this, false); }
        __device__ iterator end() const { return iterator(*this, true); }

        const detail::LaunchParams& P;
        float loc[3];
        int cell[3];
        uint32_t hx0, hx1, hx2, hy0, hy1, hy2, hz0, hz1, hz2;
        Window win;
    };

    __device__ explicit SpatialIn(const detail::LaunchParams& p) : P(p) {}
    __device__ float radius() const { return detail::ctx().grid.radius; }

 protected:
    // MessageSpatial3D::In::wrap seatbelts (MessageSpatial3DDevice.cuh:527-549)
    __device__ bool wrap_ok(float x, float y, float z) const {
#if FLAMEGPU_SEATBELTS
        const fg_spatial_grid& g = detail::ctx().grid;
        bool out = x > g.max[0] || y > g.max[1] || x < g.min[0] || y < g.min[1];
        if (DIMS == 3) out = out || z > g.max[2] || z < g.min[2];
        if (out) {
            detail::device_error(P, detail::kDevWrapOutOfBounds, 0, 0);
            return false;
        }
        if (!g.wrapCompatible) detail::device_error(P, detail::kDevWrapIncompatible, 0, 0);
#endif
        return true;
    }
    const detail::LaunchParams& P;
};

/** MessageSpatial2D (include/flamegpu/runtime/messaging/MessageSpatial2D/MessageSpatial2DDevice.cuh). */
class MessageSpatial2D {
 public:
    class Description;
    class In : public SpatialIn<2> {
     public:
        __device__ explicit In(const detail::LaunchParams& p) : SpatialIn<2>(p) {}
        __device__ Filter operator()(float x, float y) const { return Filter(P, x, y, 0.0f); }
        __device__ WrapFilter wrap(float x, float y) const {
            if (!wrap_ok(x, y, 0.0f)) return WrapFilter(P, detail::ctx().grid.min[0], detail::ctx().grid.min[1], 0.0f);
            return WrapFilter(P, x, y, 0.0f);
        }
    };
    class Out : public MessageOutBase {
     public:
        __device__ Out(const detail::LaunchParams& p, uint32_t idx) : MessageOutBase(p, idx) {}
        __device__ void setLocation(float x, float y) const {
            setVariable<float>("x", x);
            setVariable<float>("y", y);
        }
    };
};

/** MessageSpatial3D (include/flamegpu/runtime/messaging/MessageSpatial3D/MessageSpatial3DDevice.cuh). */
class MessageSpatial3D {
 public:
    class Description;
    class In : public SpatialIn<3> {
     public:
        __device__ explicit In(const detail::LaunchParams& p) : SpatialIn<3>(p) {}
        __device__ Filter operator()(float x, float y, float z) const { return Filter(P, x, y, z); }
        __device__ WrapFilter wrap(float x, float y, float z) const {
            if (!wrap_ok(x, y, z)) return WrapFilter(P, detail::ctx().grid.min[0], detail::ctx().grid.min[1], detail::ctx().grid.min[2]);
            return WrapFilter(P, x, y, z);
        }
    };
    class Out : public MessageOutBase {
     public:
        __device__ Out(const detail::LaunchParams& p, uint32_t idx) : MessageOutBase(p, idx) {}
        __device__ void setLocation(float x, float y, float z) const {
            setVariable<float>("x", x);
            setVariable<float>("y", y);
            setVariable<float>("z", z);
        }
    };
};

// ------------------------------------------------------- environment, random

namespace detail {
// Atomic operations on a 4- or 8-byte macro property element, through the
// native atomics where the type has them and a compare-and-swap loop on the
// element's bits otherwise.
template <typename T>
__device__ __forceinline__ auto as_word(T v) {
    static_assert(sizeof(T) == 4 || sizeof(T) == 8, "macro property atomics need 4- or 8-byte types");
    if constexpr (sizeof(T) == 4) {
        unsigned int u;
        memcpy(&u, &v, 4);
        return u;
    } else {
        unsigned long long u;
        memcpy(&u, &v, 8);
        return u;
    }
}
template <typename T, typename U>
__device__ __forceinline__ T from_word(U u) {
    T v;
    memcpy(&v, &u, sizeof(T));
    return v;
}
template <typename T>
__device__ __forceinline__ auto word_ptr(T* p) {
    if constexpr (sizeof(T) == 4) return reinterpret_cast<unsigned int*>(p);
    else return reinterpret_cast<unsigned long long*>(p);
}
// old value of *p, *p replaced by f(old)
template <typename T, typename F>
__device__ __forceinline__ T atomic_update(T* p, F f) {
    auto* w = word_ptr(p);
    auto old = *reinterpret_cast<volatile decltype(as_word(T{}))*>(w);
    while (true) {
        const auto seen = atomicCAS(w, old, as_word<T>(f(from_word<T>(old))));
        if (seen == old) return from_word<T>(old);
        old = seen;
    }
}
template <typename T>
__device__ __forceinline__ T atomic_add(T* p, T v) {
    if constexpr (std::is_same<T, float>::value || std::is_same<T, double>::value || std::is_same<T, int>::value ||
                  std::is_same<T, unsigned int>::value || std::is_same<T, unsigned long long>::value) {
        return atomicAdd(p, v);
    } else if constexpr (std::is_integral<T>::value && sizeof(T) == 8) {
        // two's complement: the unsigned sum has the same bits
        return static_cast<T>(atomicAdd(reinterpret_cast<unsigned long long*>(p), static_cast<unsigned long long>(v)));
    } else if constexpr (std::is_integral<T>::value && sizeof(T) == 4) {
        return static_cast<T>(atomicAdd(reinterpret_cast<unsigned int*>(p), static_cast<unsigned int>(v)));
    } else {
        return atomic_update(p, [v](T o) { return o + v; });
    }
}
template <typename T>
__device__ __forceinline__ T atomic_sub(T* p, T v) {
    if constexpr (std::is_integral<T>::value) {
        using U = typename std::conditional<sizeof(T) == 8, unsigned long long, unsigned int>::type;
        return static_cast<T>(atomicAdd(reinterpret_cast<U*>(p), static_cast<U>(0) - static_cast<U>(v)));
    } else {
        return atomic_add(p, static_cast<T>(-v));
    }
}
template <typename T>
__device__ __forceinline__ T atomic_min(T* p, T v) {
    if constexpr (std::is_same<T, int>::value || std::is_same<T, unsigned int>::value ||
                  std::is_same<T, long long>::value || std::is_same<T, unsigned long long>::value) {
        return atomicMin(p, v);
    } else if constexpr (std::is_same<T, long>::value || std::is_same<T, unsigned long>::value) {
        using U = typename std::conditional<std::is_signed<T>::value, long long, unsigned long long>::type;
        return static_cast<T>(atomicMin(reinterpret_cast<U*>(p), static_cast<U>(v)));
    } else {
        return atomic_update(p, [v](T o) { return v < o ? v : o; });
    }
}
template <typename T>
__device__ __forceinline__ T atomic_max(T* p, T v) {
    if constexpr (std::is_same<T, int>::value || std::is_same<T, unsigned int>::value ||
                  std::is_same<T, long long>::value || std::is_same<T, unsigned long long>::value) {
        return atomicMax(p, v);
    } else if constexpr (std::is_same<T, long>::value || std::is_same<T, unsigned long>::value) {
        using U = typename std::conditional<std::is_signed<T>::value, long long, unsigned long long>::type;
        return static_cast<T>(atomicMax(reinterpret_cast<U*>(p), static_cast<U>(v)));
    } else {
        return atomic_update(p, [v](T o) { return v > o ? v : o; });
    }
}
}  // namespace detail

/**
 * DeviceMacroProperty<T, I, J, K, W> (include/flamegpu/runtime/environment/
 * DeviceMacroProperty.cuh:88-205): an agent function's view of an
 * environment macro property. operator[] selects along the first dimension
 * (an index past it is a device error, and the view stays at element 0); a
 * view of one element reads as T and updates atomically: +=, -=, addAtomic /
 * subAtomic (the new value), + and - (plain reads), ++ and -- (pre: the new
 * value, post: the old), min / max (the value left), CAS (the old value),
 * exchange (the old value). Within one agent function a property is either
 * read or updated (the reference's rule; not checked here).
 */
template <typename T, flamegpu::size_type I = 1, flamegpu::size_type J = 1, flamegpu::size_type K = 1,
          flamegpu::size_type W = 1>
class DeviceMacroProperty {
 public:
    __device__ DeviceMacroProperty(const detail::LaunchParams& p, T* at, uint32_t* f) : P(p), ptr(at), flag(f) {}
    __device__ DeviceMacroProperty<T, J, K, W, 1> operator[](unsigned int i) const {
        if (i >= I) {
            detail::device_error(P, detail::kDevArrayIndex, 0, i);
            return DeviceMacroProperty<T, J, K, W, 1>(P, nullptr, nullptr);
        }
        return DeviceMacroProperty<T, J, K, W, 1>(P, ptr ? ptr + static_cast<size_t>(i) * J * K * W : nullptr, flag);
    }
    __device__ operator T() const { return read() ? *reinterpret_cast<const volatile T*>(ptr) : T{}; }
    __device__ DeviceMacroProperty& operator+=(T v) {
        if (update()) detail::atomic_add(ptr, v);
        return *this;
    }
    __device__ DeviceMacroProperty& operator-=(T v) {
        if (update()) detail::atomic_sub(ptr, v);
        return *this;
    }
    __device__ T addAtomic(T v) { return update() ? detail::atomic_add(ptr, v) + v : T{}; }
    __device__ T subAtomic(T v) { return update() ? detail::atomic_sub(ptr, v) - v : T{}; }
    __device__ T operator+(T v) const { return static_cast<T>(*this) + v; }
    __device__ T operator-(T v) const { return static_cast<T>(*this) - v; }
    __device__ T operator++() { return update() ? detail::atomic_add(ptr, static_cast<T>(1)) + static_cast<T>(1) : T{}; }
    __device__ T operator--() { return update() ? detail::atomic_sub(ptr, static_cast<T>(1)) - static_cast<T>(1) : T{}; }
    __device__ T operator++(int) { return update() ? detail::atomic_add(ptr, static_cast<T>(1)) : T{}; }
    __device__ T operator--(int) { return update() ? detail::atomic_sub(ptr, static_cast<T>(1)) : T{}; }
    __device__ T min(T v) {
        if (!update()) return T{};
        const T old = detail::atomic_min(ptr, v);
        return v < old ? v : old;
    }
    __device__ T max(T v) {
        if (!update()) return T{};
        const T old = detail::atomic_max(ptr, v);
        return v > old ? v : old;
    }
    __device__ T CAS(T compare, T v) {
        if (!update()) return T{};
        return detail::from_word<T>(atomicCAS(detail::word_ptr(ptr), detail::as_word(compare), detail::as_word(v)));
    }
    __device__ T exchange(T v) {
        if (!update()) return T{};
        return detail::from_word<T>(atomicExch(detail::word_ptr(ptr), detail::as_word(v)));
    }

 private:
    // With device checks on, the property's flag word records a read (1) and
    // an update (2) in this agent function; both is a device error
    // (DeviceMacroProperty.cuh:219-235).
    __device__ bool read() const {
        if (!ptr) return false;
#if FLAMEGPU_SEATBELTS
        if ((atomicOr(flag, 1u) & 2u) != 0u) detail::device_error(P, detail::kDevMacroConflict, 0, 0);
#endif
        return true;
    }
    __device__ bool update() const {
        if (!ptr) return false;
#if FLAMEGPU_SEATBELTS
        if ((atomicOr(flag, 2u) & 1u) != 0u) detail::device_error(P, detail::kDevMacroConflict, 0, 0);
#endif
        return true;
    }
    const detail::LaunchParams& P;
    T* ptr;         // null after a device error: reads give 0, updates do nothing
    uint32_t* flag;  // read / update record of the whole property
};

/** Read-only environment properties (include/flamegpu/runtime/environment/DeviceEnvironment.cuh). */
class DeviceEnvironment {
 public:
    __device__ explicit DeviceEnvironment(const detail::LaunchParams& p) : P(p) {}
    // env table pointers are offsets into the instance's environment buffer
    template <typename T>
    __device__ T getProperty(detail::VarName name) const {
        const T* off = detail::var_addr<T>(P, &P.T.env, name.hash, 0, 0);
        return detail::ldg_any(reinterpret_cast<const T*>(detail::ctx().env + reinterpret_cast<size_t>(off)));
    }
    template <typename T, flamegpu::size_type N>
    __device__ T getProperty(detail::VarName name, unsigned int i) const {
        const T* off = detail::var_addr<T>(P, &P.T.env, name.hash, 0, i);
        return detail::ldg_any(reinterpret_cast<const T*>(detail::ctx().env + reinterpret_cast<size_t>(off)));
    }
    /** DeviceEnvironment::getMacroProperty (DeviceEnvironment.cuh:95-112). A
     *  name that is not a macro property of this type and these dimensions is
     *  a device error, and the view then reads 0 and ignores updates. */
    template <typename T, flamegpu::size_type I = 1, flamegpu::size_type J = 1, flamegpu::size_type K = 1,
              flamegpu::size_type W = 1>
    __device__ DeviceMacroProperty<T, I, J, K, W> getMacroProperty(detail::VarName name) const {
        const detail::VarTable* t = &P.T.env;
        const detail::VarSlot* vs = &t->slot[detail::table_slot(t->mult, t->shift, name.hash)];
        // a macro property's slot holds the offset of its flag word as its stride (never 0)
        if (vs->hash != name.hash || vs->stride == 0 || vs->elem_bytes != sizeof(T) || vs->elements != I * J * K * W) {
            detail::device_error(P, vs->hash != name.hash ? detail::kDevUnknownVariable : detail::kDevTypeMismatch,
                                 name.hash, 0);
            return DeviceMacroProperty<T, I, J, K, W>(P, nullptr, nullptr);
        }
        char* env = const_cast<char*>(detail::ctx().env);
        return DeviceMacroProperty<T, I, J, K, W>(P, reinterpret_cast<T*>(env + reinterpret_cast<size_t>(vs->ptr)),
                                                  reinterpret_cast<uint32_t*>(env + vs->stride));
    }

 private:
    const detail::LaunchParams& P;
};

/**
 * Per-agent random numbers (include/flamegpu/runtime/random/AgentRandom.cuh).
 * Counter-based: draw k of agent index i in step s of function f is a
 * SplitMix64 hash of (seed, f, s, i, k); no per-thread generator state is
 * kept. The reference's curand Philox values are not reproduced; the
 * distributions and ranges are the reference's: uniform() in [0, 1),
 * uniform(min, max) in [min, max] for integers and min + (max - min) * [0, 1)
 * for floating point (min > max is a device error with seatbelts on),
 * normal() standard normal, logNormal(mean, stddev) = exp(mean + stddev *
 * normal()), poisson(mean) Poisson distributed.
 */
class AgentRandom {
 public:
    __device__ AgentRandom(const detail::LaunchParams& p, uint32_t idx) : P(p), index(idx) {}
    template <typename T>
    __device__ T uniform() const;
    template <typename T>
    __device__ T uniform(T min, T max) const;
    template <typename T>
    __device__ T normal() const;
    template <typename T>
    __device__ T logNormal(T mean, T stddev) const;
    /** Poisson distributed count with the given mean (AgentRandom.cuh:50; 0 for mean <= 0). */
    __device__ unsigned int poisson(double mean = 1.0) const;

 private:
    __device__ uint64_t next() const {
        const uint64_t key = detail::mix64(detail::ctx().seed ^ (static_cast<uint64_t>(P.fn_uid) << 40) ^ detail::ctx().step);
        return detail::mix64(detail::mix64(key + index) + (counter++));
    }
    const detail::LaunchParams& P;
    uint32_t index;
    mutable uint32_t counter = 0;
};
template <>
__device__ inline float AgentRandom::uniform<float>() const {
    return static_cast<float>(next() >> 40) * (1.0f / 16777216.0f);
}
template <>
__device__ inline double AgentRandom::uniform<double>() const {
    return static_cast<double>(next() >> 11) * (1.0 / 9007199254740992.0);
}
template <>
__device__ inline float AgentRandom::normal<float>() const {
    const float u1 = 1.0f - uniform<float>(), u2 = uniform<float>();
    return sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
}
template <>
__device__ inline double AgentRandom::normal<double>() const {
    const double u1 = 1.0 - uniform<double>(), u2 = uniform<double>();
    return sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
}
template <>
__device__ inline float AgentRandom::logNormal<float>(float mean, float stddev) const {
    return expf(mean + stddev * normal<float>());
}
template <>
__device__ inline double AgentRandom::logNormal<double>(double mean, double stddev) const {
    return exp(mean + stddev * normal<double>());
}
// Means below kPoissonSmall: Knuth's product of uniforms (The Art of Computer
// Programming, vol. 2, 3.4.1): the count of factors before the running
// product falls to exp(-mean). Larger means: Hormann's transformed rejection
// with squeeze, PTRS ("The transformed rejection method for generating
// Poisson random variables", Insurance: Mathematics and Economics 12, 1993),
// which accepts about nine draws in ten. Both loops are bounded: past the
// bound (a probability far below 2^-60) the nearest integer to the mean is
// returned.
constexpr double kPoissonSmall = 10.0;
__device__ inline unsigned int AgentRandom::poisson(double mean) const {
    if (!(mean > 0.0)) return 0u;
    if (mean < kPoissonSmall) {
        const double limit = exp(-mean);
        double prod = 1.0;
        for (unsigned int k = 0; k < 1024u; ++k) {
            prod *= uniform<double>();
            if (prod <= limit) return k;
        }
        return static_cast<unsigned int>(floor(mean + 0.5));
    }
    const double slam = sqrt(mean), loglam = log(mean);
    const double b = 0.931 + 2.53 * slam;
    const double a = -0.059 + 0.02483 * b;
    const double inv_alpha = 1.1239 + 1.1328 / (b - 3.4);
    const double v_r = 0.9277 - 3.6224 / (b - 2.0);
    for (int it = 0; it < 64; ++it) {
        const double u = uniform<double>() - 0.5;
        const double v = uniform<double>();
        const double us = 0.5 - fabs(u);
        if (us <= 0.0) continue;
        const double k = floor((2.0 * a / us + b) * u + mean + 0.43);
        if (us >= 0.07 && v <= v_r) return static_cast<unsigned int>(k);
        if (k < 0.0 || (us < 0.013 && v > us)) continue;
        if (log(v) + log(inv_alpha) - log(a / (us * us) + b) <= -mean + k * loglam - lgamma(k + 1.0))
            return static_cast<unsigned int>(k);
    }
    return static_cast<unsigned int>(floor(mean + 0.5));
}
template <typename T>
__device__ inline T AgentRandom::uniform(T min, T max) const {
#if FLAMEGPU_SEATBELTS
    if (min > max) detail::device_error(P, detail::kDevRandomRange, 0, index);
#endif
    if constexpr (std::is_integral<T>::value) {
        const uint64_t span = static_cast<uint64_t>(static_cast<int64_t>(max) - static_cast<int64_t>(min)) + 1;
        return static_cast<T>(static_cast<int64_t>(min) + static_cast<int64_t>(next() % span));
    } else {
        return min + (max - min) * uniform<T>();
    }
}

// ------------------------------------------------------------------ DeviceAPI

/** The FLAMEGPU object of an agent function (DeviceAPI.cuh:163-401). */
template <typename MessageIn, typename MessageOut>
class DeviceAPI {
 public:
    /** agent_out: birth of at most one agent per agent function call (DeviceAPI.cuh:187-236). */
    class AgentOut {
     public:
        __device__ AgentOut(const detail::LaunchParams& p, uint32_t idx) : P(p), index(idx) {}
        template <typename T>
        __device__ void setVariable(detail::VarName name, T value) const {
            if (!start(name)) return;
            detail::write_var<T>(P, &P.T.birth, name.hash, index, value);
        }
        template <typename T, flamegpu::size_type N>
        __device__ void setVariable(detail::VarName name, unsigned int i, T value) const {
            if (!start(name)) return;
            detail::write_var<T>(P, &P.T.birth, name.hash, index, value, i);
        }
        /** The new agent's id (DeviceAPI.cuh:546-557 of the reference: an atomic
         * increment of the output agent's next id). A birth whose id is never
         * asked for gets it when the step appends the new agents (next id +
         * birth rank, deterministic); one that asks claims it here, and keeps it. */
        __device__ id_t getID() const {
            if (!start_row(0u)) return ID_NOT_SET;
            if (is_born != 2u) {
                // a batch keeps one next id per instance
                claimed = atomicAdd(P.birth_next_id + detail::ctx().inst, 1u);
                detail::write_var<id_t>(P, &P.T.birth, detail::VarName("_id").hash, index, claimed);
                is_born = 2u;
            }
            return claimed;
        }
        /** Claims the new agent's id now (DeviceAPI.cuh:548-557 of the reference); getID() returns it. */
        __device__ void genID() const { (void)getID(); }
        __device__ uint32_t born() const { return is_born; }

     private:
        // First write of a birth: fill the staging row with the defaults.
        __device__ bool start(const detail::VarName& name) const {
            if (name.reserved && P.birth_flags) {
                detail::device_error(P, detail::kDevReservedName, name.hash, index);
                return false;
            }
            return start_row(name.hash);
        }
        __device__ bool start_row(uint32_t hash) const {
            if (!P.birth_flags) {
                detail::device_error(P, detail::kDevBirthNotEnabled, hash, index);
                return false;
            }
            if (!is_born) {
                is_born = 1;
                const detail::VarTable* def = &P.T.birth_def;
                const detail::VarTable* dst = &P.T.birth;
                for (int s = 0; s < detail::kMaxVarSlots; ++s) {
                    const char* d = def->slot[s].ptr;
                    if (!d) continue;
                    char* o = dst->slot[s].ptr;
                    const uint32_t bytes = def->slot[s].stride;
                    o += static_cast<size_t>(index) * dst->slot[s].stride;
                    for (uint32_t b = 0; b < bytes; ++b) o[b] = d[b];
                }
            }
            return true;
        }
        const detail::LaunchParams& P;
        uint32_t index;
        mutable uint32_t is_born = 0;  // 1: born, 2: born and its id claimed
        mutable id_t claimed = ID_NOT_SET;
    };

    __device__ DeviceAPI(const detail::LaunchParams& p, uint32_t idx)
        : message_in(p), message_out(p, idx), agent_out(p, idx), environment(p), random(p, idx), P(p), index(idx) {}
    /** msg_row: the row this agent's output message takes (the agent's index
     *  among those running the function). */
    __device__ DeviceAPI(const detail::LaunchParams& p, uint32_t idx, uint32_t msg_row)
        : message_in(p), message_out(p, msg_row), agent_out(p, idx), environment(p), random(p, idx), P(p), index(idx) {}

    template <typename T>
    __device__ T getVariable(detail::VarName name) const {
        return detail::read_rw<T>(P, &P.T.agent, name.hash, index);
    }
    template <typename T, flamegpu::size_type N>
    __device__ T getVariable(detail::VarName name, unsigned int i) const {
        return detail::read_rw<T>(P, &P.T.agent, name.hash, index, i);
    }
    template <typename T>
    __device__ void setVariable(detail::VarName name, T value) {
#if FLAMEGPU_SEATBELTS
        if (name.reserved) {
            detail::device_error(P, detail::kDevReservedName, name.hash, index);
            return;
        }
#endif
        detail::write_var<T>(P, &P.T.agent, name.hash, index, value);
        if constexpr (std::is_same<T, float>::value) {  // the position, kept for the launch's epilogue
            if (name.hash == detail::VarName("x").hash) { pos[0] = value; pos_set |= 1u; }
            if (name.hash == detail::VarName("y").hash) { pos[1] = value; pos_set |= 2u; }
            if (name.hash == detail::VarName("z").hash) { pos[2] = value; pos_set |= 4u; }
        }
    }
    template <typename T, flamegpu::size_type N>
    __device__ void setVariable(detail::VarName name, unsigned int i, T value) {
        detail::write_var<T>(P, &P.T.agent, name.hash, index, value, i);
    }
    __device__ id_t getID() const { return detail::read_rw<id_t>(P, &P.T.agent, detail::VarName("_id").hash, index); }
    __device__ unsigned int getStepCounter() const { return detail::ctx().step; }
    __device__ unsigned int getIndex() const { return index - detail::ctx().row_begin; }
    /** Whether the function runs on agents of this name / in this state
     *  (DeviceAPI.cuh:366-380 of the reference; names compared by hash). */
    __device__ bool isAgent(const char* agent_name) const { return detail::fnv1a32(agent_name, ~0u) == P.agent_hash; }
    __device__ bool isState(const char* agent_state) const { return detail::fnv1a32(agent_state, ~0u) == P.state_hash; }

    typename MessageIn::In message_in;
    typename MessageOut::Out message_out;
    AgentOut agent_out;
    DeviceEnvironment environment;
    AgentRandom random;
    // float x, y, z this function set (bits 1, 2, 4 of pos_set), for the
    // launch's epilogue
    float pos[3] = {0.0f, 0.0f, 0.0f};
    uint32_t pos_set = 0;

 private:
    const detail::LaunchParams& P;
    uint32_t index;
};

/** ReadOnlyDeviceAPI (DeviceAPI.cuh:42-142 of the reference): what an agent
 *  function condition may use — the agent's variables and id, the step
 *  counter, environment properties and random numbers; nothing is written. */
class ReadOnlyDeviceAPI {
 public:
    __device__ ReadOnlyDeviceAPI(const detail::LaunchParams& p, uint32_t idx)
        : environment(p), random(p, idx), P(p), index(idx) {}
    template <typename T>
    __device__ T getVariable(detail::VarName name) const {
        return detail::read_rw<T>(P, &P.T.agent, name.hash, index);
    }
    template <typename T, flamegpu::size_type N>
    __device__ T getVariable(detail::VarName name, unsigned int i) const {
        return detail::read_rw<T>(P, &P.T.agent, name.hash, index, i);
    }
    __device__ id_t getID() const { return detail::read_rw<id_t>(P, &P.T.agent, detail::VarName("_id").hash, index); }
    __device__ unsigned int getStepCounter() const { return detail::ctx().step; }
    __device__ unsigned int getIndex() const { return index - detail::ctx().row_begin; }
    __device__ bool isAgent(const char* agent_name) const { return detail::fnv1a32(agent_name, ~0u) == P.agent_hash; }
    __device__ bool isState(const char* agent_state) const { return detail::fnv1a32(agent_state, ~0u) == P.state_hash; }

    DeviceEnvironment environment;
    AgentRandom random;

 private:
    const detail::LaunchParams& P;
    uint32_t index;
};

#endif  // __CUDACC__

}  // namespace flamegpu

#endif  // INCLUDE_FLAMEGPU_RUNTIME_DEVICEAPI_CUH_
