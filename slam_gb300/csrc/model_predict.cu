// Model prediction and fill-in: the maps initICPModel / initRGBModel consume,
// computed from the surfel map by CUDA splatting instead of the reference's
// GL pipeline.
//
// Prediction (IndexMap::combinedPredict, src/model/IndexMap.cpp:243-345, with
// src/model/shaders/splat.vert and combo_splat.frag): every surfel is moved
// into the camera by t_inv = pose^-1 and culled (z > maxDepth, z < 0,
// confidence < confThreshold, time - lastSeen > timeDelta, lastSeen >
// maxTime); its disk (normal, radius) is bounded on screen by the projections
// of centre +- x1, +- y1 (x1 = normalize(n.y - n.z, -n.x, n.x) * r * sqrt 2,
// y1 = n x x1), which sets the point-sprite size; each pixel whose centre lies
// in that square is a candidate fragment: the ray through the pixel centre
// meets the surfel's plane at dot(p, n) / dot(l, n) * l, outside the radius
// it is discarded, otherwise its depth z / (2 maxDepth) + 0.5 is tested
// (GL_LESS against a buffer cleared to 1) and the nearest fragment writes the
// colour (decoded from the packed float), the vertex ((u - cx) z / fx,
// (v - cy) z / fy, z, confidence) at the pixel centre (u, v) = (x + 0.5,
// y + 0.5), the normal and radius, and the surfel's initialisation time.
//
// Kernels: k_splat (one thread per surfel: vertex stage, then every
// candidate pixel of its square; a 64-bit atomicMin of (depth bits << 32 |
// surfel index) per pixel is the depth test -- equal depths keep the lower
// index, the surfel the GL draw order would keep), k_splat_resolve (one
// thread per pixel: the winner's outputs, zeros where nothing was drawn).
// Arithmetic is single-operation rounded (no contraction) with IEEE division
// and square root, evaluated in the shaders' order; GL leaves the precision
// of its rasteriser and of normalize() to the implementation, so these are
// the definitions the oracle restates.  Point sizes are clamped to
// [1, 2047] (the usual implementation range); a pixel is in a point's square
// when xw - s/2 <= x + 0.5 < xw + s/2 (likewise for y).
//
// Fill-in (FillIn::vertex / normal / image, src/gl/FillIn.cpp, with
// src/gl/shaders/fill_vertex.frag:37-53, fill_normal.frag:34-50,
// fill_rgb.frag:29-37): where the prediction has a hole (vertex / normal
// z == 0, or rgb sum 0) or passthrough is set, the raw frame's value: the
// vertex from the filtered depth at integer pixel coordinates, the normal
// from forward differences of those vertices (neighbours clamped at the
// image edge), the raw colour.  One kernel, one thread per pixel.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/slam_gb300.h"

namespace slamgb {
namespace {

struct PredictK {
    float t[12];  // rows 0..2 of t_inv (row-major)
    float cx, cy, fx, fy;
    int cols, rows;
    float maxDepth, confThreshold;
    int time, maxTime, timeDelta;
    float ifx, ify;  // 1 / fx, 1 / fy (IEEE)
};

__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fd(float a, float b) { return __fdiv_rn(a, b); }

__device__ __forceinline__ float dot3(float ax, float ay, float az, float bx, float by, float bz) {
    return fa(fa(fm(ax, bx), fm(ay, by)), fm(az, bz));
}
// normalize(v) = v / sqrt(dot(v, v))
__device__ __forceinline__ void normalize3(float &x, float &y, float &z) {
    const float l = __fsqrt_rn(dot3(x, y, z, x, y, z));
    x = fd(x, l);
    y = fd(y, l);
    z = fd(z, l);
}

struct Splat {
    float px, py, pz, conf;  // position in the camera frame, confidence
    float nx, ny, nz, rad;   // normal (camera frame), radius
    float xw, yw, size;      // window position, point size
};

// splat.vert for one surfel; false when culled.
__device__ __forceinline__ bool vertex_stage(const PredictK &k, const float4 &P, const float4 &C, const float4 &N,
                                             Splat &s) {
    const float *t = k.t;
    const float hx = fa(fa(fa(fm(t[0], P.x), fm(t[1], P.y)), fm(t[2], P.z)), t[3]);
    const float hy = fa(fa(fa(fm(t[4], P.x), fm(t[5], P.y)), fm(t[6], P.z)), t[7]);
    const float hz = fa(fa(fa(fm(t[8], P.x), fm(t[9], P.y)), fm(t[10], P.z)), t[11]);
    if (hz > k.maxDepth || hz < 0.f || P.w < k.confThreshold || fs((float)k.time, C.w) > (float)k.timeDelta ||
        C.w > (float)k.maxTime)
        return false;
    s.px = hx;
    s.py = hy;
    s.pz = hz;
    s.conf = P.w;
    float nx = fa(fa(fm(t[0], N.x), fm(t[1], N.y)), fm(t[2], N.z));
    float ny = fa(fa(fm(t[4], N.x), fm(t[5], N.y)), fm(t[6], N.z));
    float nz = fa(fa(fm(t[8], N.x), fm(t[9], N.y)), fm(t[10], N.z));
    normalize3(nx, ny, nz);
    s.nx = nx;
    s.ny = ny;
    s.nz = nz;
    s.rad = N.w;
    // projectPoint, then the viewport transform
    const float hc = fm((float)k.cols, 0.5f), hr = fm((float)k.rows, 0.5f);
    const float ndx = fd(fs(fa(fd(fm(k.fx, hx), hz), k.cx), hc), hc);
    const float ndy = fd(fs(fa(fd(fm(k.fy, hy), hz), k.cy), hr), hr);
    s.xw = fm(fa(ndx, 1.f), hc);
    s.yw = fm(fa(ndy, 1.f), hr);
    // disk axes and their projections
    float ax = fs(ny, nz), ay = -nx, az = nx;
    normalize3(ax, ay, az);
    const float sc = N.w;
    ax = fm(fm(ax, sc), 1.41421356f);
    ay = fm(fm(ay, sc), 1.41421356f);
    az = fm(fm(az, sc), 1.41421356f);
    const float bx = fs(fm(ny, az), fm(nz, ay)), by = fs(fm(nz, ax), fm(nx, az)), bz = fs(fm(nx, ay), fm(ny, ax));
    float xmin = 3.4e38f, xmax = -3.4e38f, ymin = 3.4e38f, ymax = -3.4e38f;
    const float ox[4] = {ax, bx, -bx, -ax}, oy[4] = {ay, by, -by, -ay}, oz[4] = {az, bz, -bz, -az};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const float qx = fa(hx, ox[q]), qy = fa(hy, oy[q]), qz = fa(hz, oz[q]);
        const float u = fa(fd(fm(k.fx, qx), qz), k.cx), v = fa(fd(fm(k.fy, qy), qz), k.cy);
        xmin = fminf(xmin, u);
        xmax = fmaxf(xmax, u);
        ymin = fminf(ymin, v);
        ymax = fmaxf(ymax, v);
    }
    float size = fmaxf(0.f, fmaxf(fabsf(fs(xmax, xmin)), fabsf(fs(ymax, ymin))));
    size = fminf(fmaxf(size, 1.f), 2047.f);
    s.size = size;
    return true;
}

// combo_splat.frag for pixel (x, y): the corrected z, or false if discarded.
__device__ __forceinline__ bool fragment_stage(const PredictK &k, const Splat &s, int x, int y, float &z) {
    const float u = fa((float)x, 0.5f), v = fa((float)y, 0.5f);
    float lx = fd(fs(u, k.cx), k.fx), ly = fd(fs(v, k.cy), k.fy), lz = 1.f;
    normalize3(lx, ly, lz);
    const float f = fd(dot3(s.px, s.py, s.pz, s.nx, s.ny, s.nz), dot3(lx, ly, lz, s.nx, s.ny, s.nz));
    const float cxp = fm(f, lx), cyp = fm(f, ly), czp = fm(f, lz);
    const float dx = fs(cxp, s.px), dy = fs(cyp, s.py), dz = fs(czp, s.pz);
    if (dot3(dx, dy, dz, dx, dy, dz) > fm(s.rad, s.rad)) return false;
    z = czp;
    return true;
}

__device__ __forceinline__ void load_surfel(const float4 *S, int i, float4 &P, float4 &C, float4 &N) {
    P = S[3 * (size_t)i];
    C = S[3 * (size_t)i + 1];
    N = S[3 * (size_t)i + 2];
}

__global__ void __launch_bounds__(256) k_splat(const float4 *surfels, int n, PredictK k, unsigned long long *zbuf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 P, C, N;
    load_surfel(surfels, i, P, C, N);
    Splat s;
    if (!vertex_stage(k, P, C, N, s)) return;
    if (!isfinite(s.xw) || !isfinite(s.yw)) return;  // a point at z = 0 projects to infinity: no fragment
    const float h = fm(s.size, 0.5f);
    // pixels whose centre x + 0.5 lies in [xw - h, xw + h) (clamped to the
    // image before the conversion to int)
    const float lo_x = fs(fs(s.xw, h), 0.5f), hi_x = fs(fa(s.xw, h), 0.5f);
    const float lo_y = fs(fs(s.yw, h), 0.5f), hi_y = fs(fa(s.yw, h), 0.5f);
    const int x0 = (int)ceilf(fmaxf(lo_x, 0.f)), y0 = (int)ceilf(fmaxf(lo_y, 0.f));
    const int x1 = (int)ceilf(fminf(hi_x, (float)k.cols)) - 1, y1 = (int)ceilf(fminf(hi_y, (float)k.rows)) - 1;
    for (int y = y0; y <= y1; ++y)
        for (int x = x0; x <= x1; ++x) {
            float z;
            if (!fragment_stage(k, s, x, y, z)) continue;
            float depth = fa(fd(z, fm(2.f, k.maxDepth)), 0.5f);
            depth = fminf(fmaxf(depth, 0.f), 1.f);  // gl_FragDepth is clamped to [0, 1]
            if (!(depth < 1.f)) continue;            // GL_LESS against the cleared depth 1
            const unsigned long long key = ((unsigned long long)__float_as_uint(depth) << 32) | (unsigned)i;
            atomicMin(&zbuf[(size_t)y * k.cols + x], key);
        }
}

__global__ void k_splat_resolve(const float4 *surfels, PredictK k, const unsigned long long *zbuf, uchar4 *image,
                                size_t ip, float4 *vertex, float4 *normal, size_t fp, uint16_t *time, size_t tp) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= k.cols) return;
    const unsigned long long key = zbuf[(size_t)y * k.cols + x];
    uchar4 img = make_uchar4(0, 0, 0, 0);
    float4 vo = make_float4(0.f, 0.f, 0.f, 0.f), no = vo;
    unsigned tm = 0;
    if (key != ~0ull) {
        float4 P, C, N;
        load_surfel(surfels, (int)(unsigned)(key & 0xffffffffu), P, C, N);
        Splat s;
        float z = 0.f;
        vertex_stage(k, P, C, N, s);
        fragment_stage(k, s, x, y, z);
        const int c = (int)C.x;  // decodeColor (src/model/shaders/color.glsl)
        img = make_uchar4((unsigned char)((c >> 16) & 0xff), (unsigned char)((c >> 8) & 0xff),
                          (unsigned char)(c & 0xff), 255);
        vo = make_float4(fm(fm(fs(fa((float)x, 0.5f), k.cx), z), k.ifx), fm(fm(fs(fa((float)y, 0.5f), k.cy), z), k.ify),
                         z, s.conf);
        no = make_float4(s.nx, s.ny, s.nz, s.rad);
        const float tf = C.z;
        tm = tf <= 0.f ? 0u : (tf >= 65535.f ? 65535u : (unsigned)tf);
    }
    if (image) reinterpret_cast<uchar4 *>(reinterpret_cast<uint8_t *>(image) + (size_t)y * ip)[x] = img;
    if (vertex) reinterpret_cast<float4 *>(reinterpret_cast<uint8_t *>(vertex) + (size_t)y * fp)[x] = vo;
    if (normal) reinterpret_cast<float4 *>(reinterpret_cast<uint8_t *>(normal) + (size_t)y * fp)[x] = no;
    if (time) reinterpret_cast<uint16_t *>(reinterpret_cast<uint8_t *>(time) + (size_t)y * tp)[x] = (uint16_t)tm;
}

struct FillK {
    float cx, cy, ifx, ify;  // cam of the fill shaders: cx, cy, 1 / fx, 1 / fy
    int cols, rows, passthrough;
};

// getVertex of geometry.glsl (raw u16 mm depth, integer pixel coordinates),
// neighbours clamped at the image edge
__device__ __forceinline__ float3 raw_vertex(const FillK &k, const uint16_t *d, size_t dp, int x, int y) {
    x = min(max(x, 0), k.cols - 1);
    y = min(max(y, 0), k.rows - 1);
    const float z =
        fd((float)reinterpret_cast<const uint16_t *>(reinterpret_cast<const uint8_t *>(d) + (size_t)y * dp)[x],
           1000.0f);
    return make_float3(fm(fm(fs((float)x, k.cx), z), k.ifx), fm(fm(fs((float)y, k.cy), z), k.ify), z);
}

__global__ void k_fill_in(FillK k, const float4 *pv, const float4 *pn, size_t pfp, const uchar4 *pi, size_t pip,
                          const uint16_t *raw_d, size_t rdp, const uchar4 *raw_rgb, size_t rrp, float4 *ov, float4 *on,
                          size_t ofp, uchar4 *oi, size_t oip) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= k.cols) return;
    auto rowf = [](const float4 *p, size_t pitch, int r) {
        return reinterpret_cast<const float4 *>(reinterpret_cast<const uint8_t *>(p) + (size_t)r * pitch);
    };
    // fill_vertex.frag
    if (ov) {
        float4 s = rowf(pv, pfp, y)[x];
        if (s.z == 0.f || k.passthrough) {
            const float3 v = raw_vertex(k, raw_d, rdp, x, y);
            s = make_float4(v.x, v.y, v.z, 1.f);
        }
        reinterpret_cast<float4 *>(reinterpret_cast<uint8_t *>(ov) + (size_t)y * ofp)[x] = s;
    }
    // fill_normal.frag: forward differences of the raw vertices
    if (on) {
        float4 s = rowf(pn, pfp, y)[x];
        if (s.z == 0.f || k.passthrough) {
            const float3 v = raw_vertex(k, raw_d, rdp, x, y);
            const float3 vx = raw_vertex(k, raw_d, rdp, x + 1, y), vy = raw_vertex(k, raw_d, rdp, x, y + 1);
            const float ax = fs(vx.x, v.x), ay = fs(vx.y, v.y), az = fs(vx.z, v.z);
            const float bx = fs(vy.x, v.x), by = fs(vy.y, v.y), bz = fs(vy.z, v.z);
            float cx = fs(fm(ay, bz), fm(az, by)), cy = fs(fm(az, bx), fm(ax, bz)), cz = fs(fm(ax, by), fm(ay, bx));
            normalize3(cx, cy, cz);
            s = make_float4(cx, cy, cz, 1.f);
        }
        reinterpret_cast<float4 *>(reinterpret_cast<uint8_t *>(on) + (size_t)y * ofp)[x] = s;
    }
    // fill_rgb.frag
    if (oi) {
        uchar4 s = reinterpret_cast<const uchar4 *>(reinterpret_cast<const uint8_t *>(pi) + (size_t)y * pip)[x];
        if ((int)s.x + (int)s.y + (int)s.z == 0 || k.passthrough) {
            const uchar4 r =
                reinterpret_cast<const uchar4 *>(reinterpret_cast<const uint8_t *>(raw_rgb) + (size_t)y * rrp)[x];
            s = make_uchar4(r.x, r.y, r.z, 255);
        }
        reinterpret_cast<uchar4 *>(reinterpret_cast<uint8_t *>(oi) + (size_t)y * oip)[x] = s;
    }
}

}  // namespace
}  // namespace slamgb

using namespace slamgb;

extern "C" size_t odo_model_predict_scratch_bytes(int width, int height) {
    return width > 0 && height > 0 ? (size_t)width * height * sizeof(unsigned long long) : 0;
}

extern "C" int odo_model_predict(const float *surfels, int nsurfels, const float t_inv[16],
                                 const odo_predict_params *p, void *scratch, uint8_t *image, size_t image_pitch,
                                 float *vertex, float *normal, size_t map_pitch, uint16_t *time, size_t time_pitch,
                                 void *stream) {
    if (!p || !t_inv || !scratch || nsurfels < 0 || (nsurfels > 0 && !surfels) || p->width < 1 || p->height < 1 ||
        p->width > 16384 || p->height > 16384 || !(p->fx != 0) || !(p->fy != 0) || ((uintptr_t)surfels % 16) ||
        ((uintptr_t)scratch % 8))
        return ODO_ERR_ARG;
    if ((image && (image_pitch < (size_t)p->width * 4 || (image_pitch % 4) || ((uintptr_t)image % 4))) ||
        ((vertex || normal) && (map_pitch < (size_t)p->width * 16 || (map_pitch % 16))) ||
        (vertex && ((uintptr_t)vertex % 16)) || (normal && ((uintptr_t)normal % 16)) ||
        (time && (time_pitch < (size_t)p->width * 2 || (time_pitch % 2) || ((uintptr_t)time % 2))))
        return ODO_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    PredictK k{};
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 4; ++c) k.t[r * 4 + c] = t_inv[r * 4 + c];
    k.cx = p->cx;
    k.cy = p->cy;
    k.fx = p->fx;
    k.fy = p->fy;
    k.cols = p->width;
    k.rows = p->height;
    k.maxDepth = p->maxDepth;
    k.confThreshold = p->confThreshold;
    k.time = p->time;
    k.maxTime = p->maxTime;
    k.timeDelta = p->timeDelta;
    k.ifx = 1.f / p->fx;
    k.ify = 1.f / p->fy;
    unsigned long long *z = (unsigned long long *)scratch;
    if (cudaMemsetAsync(z, 0xff, odo_model_predict_scratch_bytes(p->width, p->height), s) != cudaSuccess)
        return ODO_ERR_CUDA;
    if (nsurfels > 0) k_splat<<<(nsurfels + 255) / 256, 256, 0, s>>>((const float4 *)surfels, nsurfels, k, z);
    k_splat_resolve<<<dim3((p->width + 127) / 128, p->height), 128, 0, s>>>(
        (const float4 *)surfels, k, z, (uchar4 *)image, image_pitch, (float4 *)vertex, (float4 *)normal, map_pitch,
        time, time_pitch);
    return cudaGetLastError() == cudaSuccess ? ODO_OK : ODO_ERR_CUDA;
}

extern "C" int odo_fill_in(const float *pred_vertex, const float *pred_normal, size_t pred_map_pitch,
                           const uint8_t *pred_image, size_t pred_image_pitch, const uint16_t *raw_depth,
                           size_t raw_depth_pitch, const uint8_t *raw_rgba, size_t raw_rgba_pitch, int width,
                           int height, float cx, float cy, float fx, float fy, int passthrough, float *out_vertex,
                           float *out_normal, size_t out_map_pitch, uint8_t *out_image, size_t out_image_pitch,
                           void *stream) {
    if (width < 1 || height < 1 || width > 16384 || height > 16384 || !(fx != 0) || !(fy != 0)) return ODO_ERR_ARG;
    if ((out_vertex && !pred_vertex) || (out_normal && !pred_normal) || (out_image && (!pred_image || !raw_rgba)) ||
        ((out_vertex || out_normal) && !raw_depth))
        return ODO_ERR_ARG;
    if ((out_vertex || out_normal) &&
        (pred_map_pitch < (size_t)width * 16 || out_map_pitch < (size_t)width * 16 || (pred_map_pitch % 16) ||
         (out_map_pitch % 16) || raw_depth_pitch < (size_t)width * 2 || (raw_depth_pitch % 2)))
        return ODO_ERR_ARG;
    if (out_image && (pred_image_pitch < (size_t)width * 4 || raw_rgba_pitch < (size_t)width * 4 ||
                      out_image_pitch < (size_t)width * 4 || (pred_image_pitch % 4) || (raw_rgba_pitch % 4) ||
                      (out_image_pitch % 4)))
        return ODO_ERR_ARG;
    FillK k{cx, cy, 1.f / fx, 1.f / fy, width, height, passthrough ? 1 : 0};
    k_fill_in<<<dim3((width + 127) / 128, height), 128, 0, (cudaStream_t)stream>>>(
        k, (const float4 *)pred_vertex, (const float4 *)pred_normal, pred_map_pitch, (const uchar4 *)pred_image,
        pred_image_pitch, raw_depth, raw_depth_pitch, (const uchar4 *)raw_rgba, raw_rgba_pitch, (float4 *)out_vertex,
        (float4 *)out_normal, out_map_pitch, (uchar4 *)out_image, out_image_pitch);
    return cudaGetLastError() == cudaSuccess ? ODO_OK : ODO_ERR_CUDA;
}
