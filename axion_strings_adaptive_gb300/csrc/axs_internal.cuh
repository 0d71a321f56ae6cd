// Internal helpers shared by the axion-string CUDA sources (sm_103a).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>

#include "../../include/axs.h"

namespace axs {

// ---------------------------------------------------------------- errors
void set_error(const char *fmt, ...);  // thread-local message for axs_last_error()

#define AXS_REQUIRE(cond, code, ...)                                                    \
    do {                                                                               \
        if (!(cond)) {                                                                 \
            ::axs::set_error(__VA_ARGS__);                                             \
            return (code);                                                             \
        }                                                                              \
    } while (0)

#define AXS_CUDA_CHECK(expr)                                                            \
    do {                                                                               \
        cudaError_t e_ = (expr);                                                       \
        if (e_ != cudaSuccess) {                                                       \
            ::axs::set_error("%s failed: %s", #expr, cudaGetErrorString(e_));          \
            return AXS_ERR_CUDA;                                                       \
        }                                                                              \
    } while (0)

inline int launch_status(const char *what)
{
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("%s launch failed: %s", what, cudaGetErrorString(e));
        return AXS_ERR_CUDA;
    }
    return AXS_OK;
}

inline size_t dtype_size(int32_t dt) { return dt == AXS_F64 ? 8 : (dt == AXS_F32 ? 4 : 0); }

int device_sm_count();
int validate_fab(const axs_fab *f, const char *name, int min_comp, int min_ng);

// Geometry of the fused-RK4 level layout (see axs_level_layout in axs.h):
// element (x,y,z,c) at (x + ox) + (y + oy)*js + z*ks + c*cs. ox puts x = 0
// on a 128-byte boundary; js is a multiple of 128 bytes.
struct LevelGeom {
    int64_t js, ks, cs;
    int ox, oy;
};
int level_geom(int32_t dtype, int nx, int ny, int nz, LevelGeom &g);

// Background model (host), shared by the C ABI and the RK4 driver.
void background_values(const axs_background &bg, double tau, axs_background_values &v);
void rhs_coeffs(const axs_background &bg, double tau, axs_rhs_coeffs &c);

// Polls a bounded device-side wait may make before it gives up (library-wide,
// set by axs_set_device_wait_polls; read into each launch's arguments).
uint32_t device_wait_polls();

// ---------------------------------------------------------------- device status words
// Codes OR-ed into a device status word by kernels whose bounded waits expire.
constexpr unsigned kDevTimeout = 1u;

// ---------------------------------------------------------------- element-wise async copies
// cp.async of one element into shared memory; an invalid source fills zero
// (src-size 0 reads nothing; the dummy address is never dereferenced).
template <typename T>
__device__ __forceinline__ void cp_async_elem(T *dst_smem, const T *src, bool valid, const T *dummy)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst_smem);
    const int nbytes = valid ? (int)sizeof(T) : 0;
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;\n" ::"r"(d), "l"(valid ? src : dummy),
                 "n"((int)sizeof(T)), "r"(nbytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// ---------------------------------------------------------------- vector types
template <typename T> struct Vec;
template <> struct Vec<float> {
    using type = float4;
    static constexpr int N = 4;
};
template <> struct Vec<double> {
    using type = double2;
    static constexpr int N = 2;
};

// V consecutive elements of T moved as one vector access (4, 8 or 16 bytes).
template <typename T, int V> struct VecN;
template <> struct VecN<float, 1> { using type = float; };
template <> struct VecN<float, 2> { using type = float2; };
template <> struct VecN<float, 4> { using type = float4; };
template <> struct VecN<double, 1> { using type = double; };
template <> struct VecN<double, 2> { using type = double2; };

template <typename T, int V>
__device__ __forceinline__ void ldv(const T *p, T *out)
{
    using VT = typename VecN<T, V>::type;
    const VT v = *reinterpret_cast<const VT *>(p);
    const T *e = reinterpret_cast<const T *>(&v);
#pragma unroll
    for (int i = 0; i < V; ++i) out[i] = e[i];
}

template <typename T, int V>
__device__ __forceinline__ void ldv_nc(const T *p, T *out)
{
    using VT = typename VecN<T, V>::type;
    const VT v = __ldg(reinterpret_cast<const VT *>(p));
    const T *e = reinterpret_cast<const T *>(&v);
#pragma unroll
    for (int i = 0; i < V; ++i) out[i] = e[i];
}

template <typename T, int V>
__device__ __forceinline__ void stv(T *p, const T *in)
{
    using VT = typename VecN<T, V>::type;
    VT v;
    T *e = reinterpret_cast<T *>(&v);
#pragma unroll
    for (int i = 0; i < V; ++i) e[i] = in[i];
    *reinterpret_cast<VT *>(p) = v;
}

template <typename T>
__device__ __forceinline__ void load_vec(const T *p, T *out)
{
    using V = typename Vec<T>::type;
    const V v = *reinterpret_cast<const V *>(p);
    if constexpr (Vec<T>::N == 4) {
        out[0] = v.x; out[1] = v.y; out[2] = v.z; out[3] = v.w;
    } else {
        out[0] = v.x; out[1] = v.y;
    }
}

template <typename T>
__device__ __forceinline__ void load_vec_global_nc(const T *p, T *out)
{
    using V = typename Vec<T>::type;
    const V v = __ldg(reinterpret_cast<const V *>(p));
    if constexpr (Vec<T>::N == 4) {
        out[0] = v.x; out[1] = v.y; out[2] = v.z; out[3] = v.w;
    } else {
        out[0] = v.x; out[1] = v.y;
    }
}

template <typename T>
__device__ __forceinline__ void store_vec(T *p, const T *in)
{
    using V = typename Vec<T>::type;
    V v;
    if constexpr (Vec<T>::N == 4) {
        v.x = in[0]; v.y = in[1]; v.z = in[2]; v.w = in[3];
    } else {
        v.x = in[0]; v.y = in[1];
    }
    *reinterpret_cast<V *>(p) = v;
}

// ---------------------------------------------------------------- L2 cache policies
// 64-bit L2 access policies (createpolicy) for loads and stores that carry an
// .L2::cache_hint: evict_first for streams read or written once, evict_last
// for data other blocks re-read soon (stencil halos).
__device__ __forceinline__ uint64_t l2_policy_evict_first()
{
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}

__device__ __forceinline__ uint64_t l2_policy_evict_last()
{
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}

// V-wide vector store / non-coherent load with an L2 policy.
template <typename T, int V>
__device__ __forceinline__ void stv_hint(T *p, const T *in, uint64_t pol)
{
    if constexpr (sizeof(T) == 4 && V == 1) {
        asm volatile("st.global.L2::cache_hint.f32 [%0], %1, %2;" ::"l"(p), "f"(in[0]), "l"(pol) : "memory");
    } else if constexpr (sizeof(T) == 4 && V == 2) {
        asm volatile("st.global.L2::cache_hint.v2.f32 [%0], {%1, %2}, %3;" ::"l"(p), "f"(in[0]), "f"(in[1]),
                     "l"(pol)
                     : "memory");
    } else if constexpr (sizeof(T) == 4 && V == 4) {
        asm volatile("st.global.L2::cache_hint.v4.f32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(p), "f"(in[0]),
                     "f"(in[1]), "f"(in[2]), "f"(in[3]), "l"(pol)
                     : "memory");
    } else if constexpr (sizeof(T) == 8 && V == 1) {
        asm volatile("st.global.L2::cache_hint.f64 [%0], %1, %2;" ::"l"(p), "d"(in[0]), "l"(pol) : "memory");
    } else {
        static_assert(sizeof(T) == 8 && V == 2, "unsupported vector");
        asm volatile("st.global.L2::cache_hint.v2.f64 [%0], {%1, %2}, %3;" ::"l"(p), "d"(in[0]), "d"(in[1]),
                     "l"(pol)
                     : "memory");
    }
}

template <typename T, int V>
__device__ __forceinline__ void ldv_nc_hint(const T *p, T *out, uint64_t pol)
{
    if constexpr (sizeof(T) == 4 && V == 1) {
        asm volatile("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(out[0]) : "l"(p), "l"(pol));
    } else if constexpr (sizeof(T) == 4 && V == 2) {
        asm volatile("ld.global.nc.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;"
                     : "=f"(out[0]), "=f"(out[1])
                     : "l"(p), "l"(pol));
    } else if constexpr (sizeof(T) == 4 && V == 4) {
        asm volatile("ld.global.nc.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
                     : "=f"(out[0]), "=f"(out[1]), "=f"(out[2]), "=f"(out[3])
                     : "l"(p), "l"(pol));
    } else if constexpr (sizeof(T) == 8 && V == 1) {
        asm volatile("ld.global.nc.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(out[0]) : "l"(p), "l"(pol));
    } else {
        static_assert(sizeof(T) == 8 && V == 2, "unsupported vector");
        asm volatile("ld.global.nc.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;"
                     : "=d"(out[0]), "=d"(out[1])
                     : "l"(p), "l"(pol));
    }
}

// ---------------------------------------------------------------- PTX: mbarrier + TMA
__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait: returns false if the phase did not complete within the limit.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, uint32_t max_iters = (1u << 22))
{
    for (uint32_t it = 0; it < max_iters; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
    }
    return false;
}

__device__ __forceinline__ void tma_load_4d(void *dst, const CUtensorMap *map, int c0, int c1, int c2, int c3,
                                            uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_addr(bar))
        : "memory");
}

// A tensor map that lives in global memory and was written by a host copy must
// be acquired by the tensormap proxy before a TMA instruction reads it.
__device__ __forceinline__ void fence_tensormap_acquire(const CUtensorMap *map)
{
    asm volatile("fence.proxy.tensormap::generic.acquire.sys [%0], 128;" ::"l"(reinterpret_cast<uint64_t>(map))
                 : "memory");
}

__device__ __forceinline__ void tma_load_4d_hint(void *dst, const CUtensorMap *map, int c0, int c1, int c2, int c3,
                                                 uint64_t *bar, uint64_t pol)
{
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes.L2::cache_hint "
        "[%0], [%1, {%2, %3, %4, %5}], [%6], %7;" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_addr(bar)), "l"(pol)
        : "memory");
}

__device__ __forceinline__ void prefetch_tensormap(const CUtensorMap *map)
{
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// Host: build a 4D tiled tensor map {x, y, z, comp} over a padded level array.
int make_tensor_map_4d(CUtensorMap *map, const void *base, int32_t dtype, uint64_t dim0, uint64_t dim1,
                       uint64_t dim2, uint64_t dim3, uint64_t stride1_bytes, uint64_t stride2_bytes,
                       uint64_t stride3_bytes, uint32_t box0, uint32_t box1, uint32_t box2, uint32_t box3);

}  // namespace axs
