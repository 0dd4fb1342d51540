// Shared device/host helpers for the SPECTER GB300 library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "ff.cuh"

namespace sg {

template <typename T> struct cplx_t;
template <> struct cplx_t<double> { using type = double2; };
template <> struct cplx_t<float> { using type = float2; };
template <> struct cplx_t<ff> { using type = ffc; };
template <typename T> using C2 = typename cplx_t<T>::type;

// the three arithmetic types of the kernels: FP32, FP64 and float-float (ff.cuh)
template <typename T> constexpr bool is_f32 = std::is_same<T, float>::value;
template <typename T> constexpr bool is_f64 = std::is_same<T, double>::value;
template <typename T> constexpr bool is_ff = std::is_same<T, ff>::value;

// read-only global load of a complex element (float-float complex as one 16-byte load)
template <typename V> __device__ __forceinline__ V ldg_v(const V *p) { return __ldg(p); }
template <> __device__ __forceinline__ ffc ldg_v<ffc>(const ffc *p) {
    const float4 f = __ldg((const float4 *)p);
    ffc r;
    r.x = ff(f.x, f.y);
    r.y = ff(f.z, f.w);
    return r;
}
// a complex FP32 value in the kernel's type (exact)
template <typename T> __device__ __forceinline__ C2<T> from_f2(float2 v) {
    C2<T> r;
    r.x = v.x;
    r.y = v.y;
    return r;
}

template <typename T> __host__ __device__ __forceinline__ C2<T> mk(T r, T i) { C2<T> c; c.x = r; c.y = i; return c; }
template <typename V> __host__ __device__ __forceinline__ V cadd(V a, V b) { a.x += b.x; a.y += b.y; return a; }
template <typename V> __host__ __device__ __forceinline__ V csub(V a, V b) { a.x -= b.x; a.y -= b.y; return a; }
template <typename V> __host__ __device__ __forceinline__ V cmul(V a, V b) {
    V c; c.x = a.x * b.x - a.y * b.y; c.y = a.x * b.y + a.y * b.x; return c;
}
// a * conj(b)
template <typename V> __host__ __device__ __forceinline__ V cmulc(V a, V b) {
    V c; c.x = a.x * b.x + a.y * b.y; c.y = a.y * b.x - a.x * b.y; return c;
}
template <typename V, typename S> __host__ __device__ __forceinline__ V cscale(V a, S s) { a.x *= s; a.y *= s; return a; }
template <typename V> __host__ __device__ __forceinline__ V cconj(V a) { a.y = -a.y; return a; }
// i*k*a, written as the Fortran complex product (0,k)*(ar,ai)
template <typename V, typename S> __host__ __device__ __forceinline__ V cimk(S k, V a) {
    V c; c.x = -k * a.y; c.y = k * a.x; return c;
}
// multiply by i*s (s = +-1)
template <typename V> __device__ __forceinline__ V cmuli(V a, int s) {
    V c; c.x = -s * a.y; c.y = s * a.x; return c;
}

__host__ __device__ __forceinline__ int cdiv(int a, int b) { return (a + b - 1) / b; }
// log2 of a power of two.  Tile widths (kx columns per z/y tile, rows per x tile, FFT batch
// widths) are powers of two, so index splits use shifts and masks instead of divisions.
__device__ __forceinline__ int lg2(int pow2) { return __ffs(pow2) - 1; }

// ---- asynchronous global -> shared copies (cp.async): the copies of a whole tile are in
// flight together; async_wait() completes them for the calling thread (a barrier follows).
template <int BYTES>
__device__ __forceinline__ void cp_async(void *smem_dst, const void *gmem_src) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
    if constexpr (BYTES == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem_src) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(s), "l"(gmem_src), "n"(BYTES) : "memory");
}
__device__ __forceinline__ void async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void async_wait() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }
// wait until at most N of the calling thread's most recent copy groups are still in flight
template <int N>
__device__ __forceinline__ void async_wait_n() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Asynchronously copy a [rows][TK] complex column tile: element (k, c) comes from
// src[k*stride + c] for c < nv and is zero for nv <= c < TK.  Call async_wait() and
// __syncthreads() before reading the tile.
template <typename V>
__device__ __forceinline__ void tile_load_async(V *dst, const V *src, unsigned stride, int rows, int TK, int nv) {
    const int lgTK = lg2(TK);
    for (int idx = threadIdx.x; idx < rows * TK; idx += blockDim.x) {
        const int k = idx >> lgTK, c = idx & (TK - 1);
        if (c < nv) cp_async<sizeof(V)>(dst + idx, src + ((unsigned)k * stride + (unsigned)c));
        else { V z; z.x = 0; z.y = 0; dst[idx] = z; }
    }
    async_commit();
}

// Same for rows stored contiguously: element (k, c) of the [rows][TK] tile, held at
// dst[k*dstride + c], comes from src[c*cstride + k] (c < nv), so consecutive threads read
// consecutive k.  An odd dstride (TK + 1) keeps those shared-memory writes free of bank conflicts.
template <typename V>
__device__ __forceinline__ void rows_load_async(V *dst, const V *src, unsigned cstride, int rows, int TK, int nv,
                                                int dstride) {
    // (c, k) = divmod(idx, rows), advanced by blockDim.x without dividing per element
    const int sc = blockDim.x / rows, sk = blockDim.x - sc * rows;
    int c = threadIdx.x / rows, k = threadIdx.x - c * rows;
    for (int idx = threadIdx.x; idx < rows * TK; idx += blockDim.x) {
        if (c < nv) cp_async<sizeof(V)>(dst + k * dstride + c, src + ((unsigned)c * cstride + (unsigned)k));
        else { V z; z.x = 0; z.y = 0; dst[k * dstride + c] = z; }
        c += sc;
        k += sk;
        if (k >= rows) { k -= rows; c++; }
    }
    async_commit();
}

}  // namespace sg
