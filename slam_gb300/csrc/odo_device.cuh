// Device-side helpers shared by the kernels.  The float3 operators are
// written with the same expression trees as the reference's
// (src/cuda/operators.cuh:57-91): with the same nvcc flags
// (--ftz=true --prec-div=false --prec-sqrt=false, fmad on) the compiler then
// makes the same contraction and division choices, which keeps projective
// association indices and valid masks bit-identical.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "odo_internal.h"

namespace slamgb {

__device__ __forceinline__ float3 operator-(const float3 &a, const float3 &b) {
    return make_float3(a.x - b.x, a.y - b.y, a.z - b.z);
}
__device__ __forceinline__ float3 operator+(const float3 &a, const float3 &b) {
    return make_float3(a.x + b.x, a.y + b.y, a.z + b.z);
}
__device__ __forceinline__ float3 cross(const float3 &a, const float3 &b) {
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float dot(const float3 &a, const float3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float norm(const float3 &a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ float3 normalized(const float3 &a) {
    const float rn = rsqrtf(dot(a, a));
    return make_float3(a.x * rn, a.y * rn, a.z * rn);
}

struct M33 {
    float3 r[3];
};
__device__ __forceinline__ float3 operator*(const M33 &m, const float3 &a) {
    return make_float3(dot(m.r[0], a), dot(m.r[1], a), dot(m.r[2], a));
}
__device__ __forceinline__ M33 load_m33(const float *p) {
    M33 m;
    m.r[0] = make_float3(p[0], p[1], p[2]);
    m.r[1] = make_float3(p[3], p[4], p[5]);
    m.r[2] = make_float3(p[6], p[7], p[8]);
    return m;
}

__device__ __forceinline__ float qnan_f() { return __int_as_float(0x7fffffff); }

template <typename T>
__device__ __forceinline__ T *rowp(T *base, size_t pitch, int y) {
    return (T *)((char *)base + (size_t)y * pitch);
}
template <typename T>
__device__ __forceinline__ T &at(const Img<T> &im, int x, int y) {
    return rowp(im.data, im.pitch, y)[x];
}
__device__ __forceinline__ float *map_row(const Map3 &m, int c, int y) {
    return rowp(m.data, m.pitch, c * m.rows + y);
}

// The same addresses with a 32-bit byte offset (one 32-bit multiply-add and
// one 64-bit add instead of a 64-bit product), for the per-pixel loads and
// stores of the iteration passes.  Valid where the row index is not
// negative and every offset stays below 4 GiB: the library's own images and
// maps (frames of at most 8192 x 8192: the largest, the 16-byte
// correspondence records, spans 1 GiB) and caller maps whose 3 x rows x
// pitch the allocation-free entry point checks.
template <typename T>
__device__ __forceinline__ T &at32(T *base, size_t pitch, int x, int y) {
    return *(T *)((char *)base + ((unsigned)y * (unsigned)pitch + (unsigned)x * (unsigned)sizeof(T)));
}
template <typename T>
__device__ __forceinline__ T &at32(const Img<T> &im, int x, int y) {
    return at32(im.data, im.pitch, x, y);
}
__device__ __forceinline__ float &map_at32(const Map3 &m, int c, int x, int y) {
    return at32(m.data, m.pitch, x, c * m.rows + y);
}

}  // namespace slamgb
