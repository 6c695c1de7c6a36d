// Depth pre-filter of the tracking input, as CUDA kernels: the reference
// computes it with GL fragment shaders before every initICP(depth) (the
// FILTER and METRIC compute packs, src/apps/elastic_fusion_file.cpp:310-312,
// 349-351).
//
//  depth_bilateral.frag (src/gl/shaders/depth_bilateral.frag:30-76): raw u16
//  depth in mm; a pixel outside [300, uint(maxD * 1000)] becomes 0; any other
//  becomes round(sum1 / sum2) over the 13x13 window clipped to the image,
//  sum1 = sum tmp * w, sum2 = sum w, w = exp(-(space2 * 0.024691358 + color2
//  * 0.000555556)) with space2 the squared pixel distance and color2 the
//  squared difference of raw values (neighbours are raw values, zeros and
//  out-of-range ones included).  Taps are visited row by row, as the shader's
//  loops do; the products and sums are rounded one operation at a time (no
//  contraction), the exponential is expf, the division IEEE, and the final
//  rounding is to nearest with ties to even (GLSL leaves the tie direction
//  and the accuracy of exp to the implementation).  The shader reads each
//  neighbour at the texel's corner coordinate (cx / cols); exactly that texel
//  is read here.
//
//  depth_metric.frag (src/gl/shaders/depth_metric.frag:28-40): metres as
//  float, 0 outside [300, uint(maxD * 1000)].
//
// One 32 x 16 output tile per block of 32 x 8 threads (two rows per thread);
// the tile and its 6-pixel halo are staged in shared memory once.  The
// exponentials dominate (169 per pixel): the kernel is bound by the special
// function units, not by memory (4 B per pixel).
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/slam_gb300.h"

namespace slamgb {
namespace {

constexpr int kR = 6;               // window radius (D = 13)
constexpr int kTW = 32, kTH = 16;   // output tile
constexpr int kBY = 8;              // thread rows (2 output rows each)
constexpr int kSW = kTW + 2 * kR, kSH = kTH + 2 * kR;
constexpr float kSpace = 0.024691358f;  // 0.5 / sigma_space^2
constexpr float kColor = 0.000555556f;  // 0.5 / sigma_color^2

__device__ __forceinline__ const uint16_t *row16(const uint16_t *p, size_t pitch, int y) {
    return reinterpret_cast<const uint16_t *>(reinterpret_cast<const uint8_t *>(p) + (size_t)y * pitch);
}

__global__ void __launch_bounds__(kTW *kBY) k_depth_bilateral(const uint16_t *src, size_t sp, uint16_t *dst, size_t dp,
                                                              int cols, int rows, unsigned max_mm) {
    __shared__ float t[kSH][kSW];
    const int X0 = blockIdx.x * kTW, Y0 = blockIdx.y * kTH;
    const int tid = threadIdx.y * kTW + threadIdx.x;
    for (int k = tid; k < kSH * kSW; k += kTW * kBY) {
        const int ty = k / kSW, tx = k - ty * kSW;
        const int gx = X0 - kR + tx, gy = Y0 - kR + ty;
        t[ty][tx] = (gx >= 0 && gy >= 0 && gx < cols && gy < rows) ? (float)row16(src, sp, gy)[gx] : 0.f;
    }
    __syncthreads();
    for (int r = 0; r < kTH / kBY; ++r) {
        const int x = X0 + threadIdx.x, y = Y0 + threadIdx.y + kBY * r;
        if (x >= cols || y >= rows) continue;
        const unsigned value = row16(src, sp, y)[x];
        uint16_t out = 0;
        if (!(value > max_mm || value < 300u)) {
            const float v = (float)value;
            const int cy0 = max(y - kR, 0), cy1 = min(y - kR + 2 * kR + 1, rows);
            const int cx0 = max(x - kR, 0), cx1 = min(x - kR + 2 * kR + 1, cols);
            float sum1 = 0.f, sum2 = 0.f;
            for (int cy = cy0; cy < cy1; ++cy) {
                const float *trow = t[cy - Y0 + kR];
                const float dy = __fsub_rn((float)y, (float)cy);
                const float dy2 = __fmul_rn(dy, dy);
                for (int cx = cx0; cx < cx1; ++cx) {
                    const float tmp = trow[cx - X0 + kR];
                    const float dx = __fsub_rn((float)x, (float)cx);
                    const float space2 = __fadd_rn(__fmul_rn(dx, dx), dy2);
                    const float dc = __fsub_rn(v, tmp);
                    const float color2 = __fmul_rn(dc, dc);
                    const float arg = __fadd_rn(__fmul_rn(space2, kSpace), __fmul_rn(color2, kColor));
                    const float w = expf(-arg);
                    sum1 = __fadd_rn(sum1, __fmul_rn(tmp, w));
                    sum2 = __fadd_rn(sum2, w);
                }
            }
            out = (uint16_t)__float2uint_rn(__fdiv_rn(sum1, sum2));
        }
        reinterpret_cast<uint16_t *>(reinterpret_cast<uint8_t *>(dst) + (size_t)y * dp)[x] = out;
    }
}

__global__ void k_depth_metric(const uint16_t *src, size_t sp, float *dst, size_t dp, int cols, int rows,
                               unsigned max_mm) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= cols || y >= rows) return;
    const unsigned value = row16(src, sp, y)[x];
    reinterpret_cast<float *>(reinterpret_cast<uint8_t *>(dst) + (size_t)y * dp)[x] =
        (value > max_mm || value < 300u) ? 0.f : __fdiv_rn((float)value, 1000.0f);
}

}  // namespace

// uint(maxD * 1000.0f) of the shaders
unsigned depth_filter_max_mm(float maxD) {
    const float m = maxD * 1000.0f;
    return m <= 0.f ? 0u : (m >= 4294967040.f ? 0xffffffffu : (unsigned)m);
}

cudaError_t launch_depth_bilateral(const uint16_t *src, size_t sp, uint16_t *dst, size_t dp, int cols, int rows,
                                   float maxD, cudaStream_t s) {
    dim3 grid((cols + kTW - 1) / kTW, (rows + kTH - 1) / kTH);
    k_depth_bilateral<<<grid, dim3(kTW, kBY), 0, s>>>(src, sp, dst, dp, cols, rows, depth_filter_max_mm(maxD));
    return cudaGetLastError();
}

cudaError_t launch_depth_metric(const uint16_t *src, size_t sp, float *dst, size_t dp, int cols, int rows, float maxD,
                                cudaStream_t s) {
    dim3 grid((cols + 127) / 128, rows);
    k_depth_metric<<<grid, 128, 0, s>>>(src, sp, dst, dp, cols, rows, depth_filter_max_mm(maxD));
    return cudaGetLastError();
}

}  // namespace slamgb

extern "C" int odo_filter_depth(const uint16_t *raw, size_t raw_pitch, uint16_t *out, size_t out_pitch, int width,
                                int height, float maxD, void *stream) {
    if (!raw || !out || width < 1 || height < 1 || width > 16384 || height > 16384 ||
        raw_pitch < (size_t)width * 2 || out_pitch < (size_t)width * 2 || (raw_pitch % 2) || (out_pitch % 2) ||
        ((uintptr_t)raw % 2) || ((uintptr_t)out % 2) || !(maxD == maxD) || (const void *)raw == (const void *)out)
        return ODO_ERR_ARG;
    if (slamgb::launch_depth_bilateral(raw, raw_pitch, out, out_pitch, width, height, maxD, (cudaStream_t)stream) !=
        cudaSuccess)
        return ODO_ERR_CUDA;
    return ODO_OK;
}

extern "C" int odo_depth_metric(const uint16_t *raw, size_t raw_pitch, float *out, size_t out_pitch, int width,
                                int height, float maxD, void *stream) {
    if (!raw || !out || width < 1 || height < 1 || width > 16384 || height > 16384 ||
        raw_pitch < (size_t)width * 2 || out_pitch < (size_t)width * 4 || (raw_pitch % 2) || (out_pitch % 4) ||
        ((uintptr_t)raw % 2) || ((uintptr_t)out % 4) || !(maxD == maxD))
        return ODO_ERR_ARG;
    if (slamgb::launch_depth_metric(raw, raw_pitch, out, out_pitch, width, height, maxD, (cudaStream_t)stream) !=
        cudaSuccess)
        return ODO_ERR_CUDA;
    return ODO_OK;
}
