// Shared device/host helpers for the SPECTER GB300 library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace sg {

template <typename T> struct cplx_t;
template <> struct cplx_t<double> { using type = double2; };
template <> struct cplx_t<float> { using type = float2; };
template <typename T> using C2 = typename cplx_t<T>::type;

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

}  // namespace sg
