// Per-frame preprocessing kernels: depth pyramid, vertex/normal maps, model
// map import (RGBA32F -> planar pyramid, rigid transform), photometric
// depth/intensity pyramids and derivative images.
//
// Each kernel restates the arithmetic of the reference kernel it replaces
// (cited per kernel) so results are identical, but several reference
// launches are fused into one: vertex+normal maps for all levels, the whole
// model-map pyramid with its transform, and one launch per pyramid step for
// depth and intensity together.  Blocks of 32x8 threads; the window kernels
// stage their source tile in shared memory and compute 32 x 8 (one frame) or
// 32 x 32 (batches) outputs per block; the model-map kernel imports one
// 32x32 input tile per block for all three levels.
#include "odo_device.cuh"

namespace slamgb {

namespace {

constexpr int BX = 32, BY = 8;

// Output rows per block of the per-pixel preprocessing kernels: 32 for
// batches (a block's memory round trip shared by 1024 outputs), 8 for a
// single frame (enough blocks to fill the GPU from one 640x480 image).
constexpr int kTileRowsBatch = 32, kTileRowsSingle = 8;
// The Gaussian pyramid's batched tiles are 16 rows high: its staged tiles
// and horizontal sums for 32 rows would exceed 48 KB of static shared memory.
constexpr int kGaussRowsBatch = 16;

// Linear enumeration of the 32 x th tiles of all pyramid levels (level l is
// (cols >> l) x (rows >> l)), so that a multi-level launch has no blocks for
// pixels outside a level; a 32x8 block covers a tile in th / 8 passes.
struct LevelTiles {
    int tx[kLevels];     // tiles per row of each level
    int start[kLevels];  // first linear tile of each level
    int total;
    int th;              // tile rows
};
inline LevelTiles level_tiles(int cols, int rows, int nlevels, int th) {
    LevelTiles t{};
    t.th = th;
    int s = 0;
    for (int l = 0; l < kLevels; ++l) {
        const int c = l < nlevels ? cols >> l : 0, r = l < nlevels ? rows >> l : 0;
        t.tx[l] = (c + BX - 1) / BX;
        t.start[l] = s;
        s += t.tx[l] * ((r + th - 1) / th);
    }
    t.total = s;
    return t;
}
// Level and first pixel (X0, Y0) of linear tile b.
// (Selects, not an indexed read: a dynamically indexed kernel-parameter
// array is copied to local memory.)
__device__ __forceinline__ void tile_origin(const LevelTiles &t, int b, int &l, int &X0, int &Y0) {
    l = b >= t.start[2] ? 2 : (b >= t.start[1] ? 1 : 0);
    const int k = b - (l == 2 ? t.start[2] : (l == 1 ? t.start[1] : t.start[0]));
    const int tx = l == 2 ? t.tx[2] : (l == 1 ? t.tx[1] : t.tx[0]);
    X0 = (k % tx) * BX;
    Y0 = (k / tx) * t.th;
}

// The window kernels stage the source pixels of their block in shared
// memory (coalesced loads, each source pixel read once) and then evaluate
// the reference's windows on the tile.  A block of 32x8 threads computes
// 32 x TR outputs (TR / 8 per thread, rows 8 apart).  A 2x downsampling 5x5
// window of those outputs covers source columns [2 X0 - 2, 2 X0 + 65) and
// rows [2 Y0 - 2, 2 Y0 + 2 TR + 1); the same-level 3x3 / 4x4 windows of the
// derivative kernel cover [X0 - 2, X0 + 33) x [Y0 - 2, Y0 + TR + 1).  The
// Gaussian and derivative tiles start at a multiple of 4 columns and are a
// few columns wider, so 4-pixel loads fill them.  Tile entries outside the
// image are never read by the border loops (they clamp to the image).
constexpr int kDownTW = 2 * BX + 4;

// The batched kernels read their pair's argument block from a device array.
// Read there directly, every field would be re-loaded from global memory
// after each global store of the kernel (the compiler cannot rule out that a
// store changes it); a copy in shared memory (which global stores cannot
// touch) is loaded once.  All threads of the block take part.
template <typename T>
__device__ __forceinline__ const T &stage_args(T &dst, const T &src) {
    static_assert(sizeof(T) % 4 == 0, "word copy");
    unsigned *d = reinterpret_cast<unsigned *>(&dst);
    const unsigned *s = reinterpret_cast<const unsigned *>(&src);
    const int tid = (threadIdx.z * blockDim.y + threadIdx.y) * blockDim.x + threadIdx.x;
    const int nt = blockDim.x * blockDim.y * blockDim.z;
    for (int k = tid; k < (int)(sizeof(T) / 4); k += nt) d[k] = s[k];
    __syncthreads();
    return dst;
}
template <int TR>
__host__ __device__ constexpr int down_th() { return 2 * TR + 4; }
template <int TR>
__host__ __device__ constexpr int der_th() { return TR + 4; }
// All loads of a thread are issued before the first store to shared memory
// (a register array of compile-time size), so a block waits for one memory
// round trip, not one per element.  Blocks are BX x BY threads.
template <typename T, typename S, int TH, int TW>
__device__ __forceinline__ void load_tile(const Img<const T> &src, int ox, int oy, S (&tile)[TH][TW]) {
    constexpr int N = TH * TW, NT = BX * BY, IT = (N + NT - 1) / NT;
    const int tid = threadIdx.y * BX + threadIdx.x;
    T v[IT];
#pragma unroll
    for (int k = 0; k < IT; ++k) {
        const int i = tid + k * NT;
        const int ty = i / TW, tx = i - ty * TW;
        const int gx = ox + tx, gy = oy + ty;
        v[k] = T{};
        if (i < N && gx >= 0 && gy >= 0 && gx < src.cols && gy < src.rows) v[k] = at(src, gx, gy);
    }
    S *flat = &tile[0][0];
#pragma unroll
    for (int k = 0; k < IT; ++k)
        if (tid + k * NT < N) flat[tid + k * NT] = (S)v[k];
}

// pyrDownGaussKernel, src/odom/utils.cu:57-94 (sigma_color = 30, :103), on
// a shared-memory tile of the source; (X0, Y0) = the block's first output.
template <int TR>
__device__ __forceinline__ void pyr_out(const PyrArgs &a, const uint16_t (&t)[down_th<TR>()][kDownTW], int ox, int oy,
                                        int x, int y) {
    const Img<const uint16_t> src = a.src;
    const Img<uint16_t> dst = a.dst;
    if (x >= dst.cols || y >= dst.rows) return;
    const int D = 5;
    const float sigma_color = 30.f;
    int center = t[2 * y - oy][2 * x - ox];
    int x_mi = max(0, 2 * x - D / 2) - 2 * x;
    int y_mi = max(0, 2 * y - D / 2) - 2 * y;
    int x_ma = min(src.cols, 2 * x - D / 2 + D) - 2 * x;
    int y_ma = min(src.rows, 2 * y - D / 2 + D) - 2 * y;
    float sum = 0, wall = 0;
    const float weights[] = {0.375f, 0.25f, 0.0625f};
    if (x_mi == -2 && x_ma == 3 && y_mi == -2 && y_ma == 3) {
        // interior, in fixed point: the weights are 6/16, 4/16, 1/16, so every
        // term is val * W / 256 (W integer <= 36) and every partial sum of the
        // reference's float loop is an exact float (numerator < 65536 * 256 =
        // 2^24); the integer sums scaled by 2^-8 are those same floats
        int isum = 0, iwall = 0;
#pragma unroll
        for (int yi = -2; yi < 3; ++yi) {
            const uint16_t *r = t[2 * y + yi - oy] - ox;
#pragma unroll
            for (int xi = -2; xi < 3; ++xi) {
                const int val = r[2 * x + xi];
                const int w = (xi == 0 ? 6 : (xi == 1 || xi == -1 ? 4 : 1)) * (yi == 0 ? 6 : (yi == 1 || yi == -1 ? 4 : 1));
                const bool ok = abs(val - center) < 90;  // 3 * sigma_color = 90.0f exactly
                isum += ok ? val * w : 0;
                iwall += ok ? w : 0;
            }
        }
        sum = (float)isum * 0.00390625f;
        wall = (float)iwall * 0.00390625f;
    } else {
        for (int yi = y_mi; yi < y_ma; ++yi) {
            const uint16_t *r = t[2 * y + yi - oy] - ox;
            for (int xi = x_mi; xi < x_ma; ++xi) {
                int val = r[2 * x + xi];
                if (abs(val - center) < 3 * sigma_color) {
                    sum += val * weights[abs(xi)] * weights[abs(yi)];
                    wall += weights[abs(xi)] * weights[abs(yi)];
                }
            }
        }
    }
    at(dst, x, y) = static_cast<int>(sum / wall);
}
template <int TR>
__device__ __forceinline__ void pyr_tile(const PyrArgs &a, int X0, int Y0) {
    __shared__ uint16_t t[down_th<TR>()][kDownTW];
    const int ox = 2 * X0 - 2, oy = 2 * Y0 - 2;
    load_tile(a.src, ox, oy, t);
    __syncthreads();
#pragma unroll 1
    for (int r = 0; r < TR / BY; ++r) pyr_out<TR>(a, t, ox, oy, X0 + threadIdx.x, Y0 + threadIdx.y + BY * r);
}
__global__ void k_pyr_down_depth(PyrArgs a) {
    pyr_tile<kTileRowsSingle>(a, blockIdx.x * BX, blockIdx.y * kTileRowsSingle);
}
__global__ void k_pyr_down_depth_b(const PyrArgs *A) {
    __shared__ PyrArgs sa;
    pyr_tile<kTileRowsBatch>(stage_args(sa, A[blockIdx.z]), blockIdx.x * BX, blockIdx.y * kTileRowsBatch);
}

// computeVmapKernel, src/odom/utils.cu:109-133, for one pixel.
__device__ __forceinline__ float3 vertex_at(const Img<const uint16_t> &depth, int u, int v, float fx_inv,
                                            float fy_inv, float cx, float cy, float depthCutoff) {
    float z = at(depth, u, v) / 1000.f;  // mm -> m
    if (z != 0 && z < depthCutoff) {
        float vx = z * (u - cx) * fx_inv;
        float vy = z * (v - cy) * fy_inv;
        return make_float3(vx, vy, z);
    }
    return make_float3(qnan_f(), qnan_f(), qnan_f());
}

// createVMap + createNMap (src/odom/utils.cu:109-204) fused, all levels in
// one launch (blockIdx.z = level).  The normal needs the vertices right and
// below; they are recomputed from depth with the same arithmetic instead of
// being re-read, so the result is bit-identical to the two-pass version.
__device__ __forceinline__ void vnmap_px(const VNArgs &a, int l, int u, int v) {
    const Img<const uint16_t> depth = a.depth[l];
    if (u >= depth.cols || v >= depth.rows) return;
    const float fxi = a.fx_inv[l], fyi = a.fy_inv[l], cx = a.cx[l], cy = a.cy[l];
    const Map3 vm = a.vmap[l], nm = a.nmap[l];
    float3 v00 = vertex_at(depth, u, v, fxi, fyi, cx, cy, a.cutoff);
    map_row(vm, 0, v)[u] = v00.x;
    map_row(vm, 1, v)[u] = v00.y;
    map_row(vm, 2, v)[u] = v00.z;
    // computeNmapKernel, src/odom/utils.cu:151-188
    float3 n = make_float3(qnan_f(), qnan_f(), qnan_f());
    if (!(u == depth.cols - 1 || v == depth.rows - 1)) {
        float3 v01 = vertex_at(depth, u + 1, v, fxi, fyi, cx, cy, a.cutoff);
        float3 v10 = vertex_at(depth, u, v + 1, fxi, fyi, cx, cy, a.cutoff);
        if (!isnan(v00.x) && !isnan(v01.x) && !isnan(v10.x)) n = normalized(cross(v01 - v00, v10 - v00));
    }
    map_row(nm, 0, v)[u] = n.x;
    map_row(nm, 1, v)[u] = n.y;
    map_row(nm, 2, v)[u] = n.z;
}
__device__ __forceinline__ void vnmap_tile(const VNArgs &a, const LevelTiles &t) {
    int l, X0, Y0;
    tile_origin(t, blockIdx.x, l, X0, Y0);
#pragma unroll 1
    for (int r = 0; r < t.th / BY; ++r) vnmap_px(a, l, X0 + threadIdx.x, Y0 + threadIdx.y + BY * r);
}
__global__ void k_vmap_nmap(VNArgs a, LevelTiles t) { vnmap_tile(a, t); }
__global__ void k_vmap_nmap_b(const VNArgs *A, LevelTiles t) {
    __shared__ VNArgs sa;
    vnmap_tile(stage_args(sa, A[blockIdx.z]), t);
}

// verticesToDepthKernel (src/odom/utils.cu:526-537): the photometric depth
// of a vertex, cut at maxDepthRGB = 6.0 (src/odom/RGBDOdometryef.cpp:37).
__device__ __forceinline__ float model_depth(float z) {
    const float cutOff = 6.0f;
    return z > cutOff || z <= 0 ? qnan_f() : z;
}

// copyMapsKernel (src/odom/utils.cu:270-310): a pixel is valid iff the
// vertex z != 0.
__device__ __forceinline__ void copy_px(const ModelArgs &a, int x, int y, float3 &v, float3 &n) {
    const float *vr = rowp(a.v4, a.pitch4, y) + 4 * x;
    const float *nr = rowp(a.n4, a.pitch4, y) + 4 * x;
    float4 vs = *reinterpret_cast<const float4 *>(vr);
    float4 ns = *reinterpret_cast<const float4 *>(nr);
    const float q = qnan_f();
    v = make_float3(q, q, q);
    n = make_float3(q, q, q);
    if (!(vs.z == 0)) {
        v = make_float3(vs.x, vs.y, vs.z);
        n = make_float3(ns.x, ns.y, ns.z);
    }
}

// resizeMapKernel<normalize>, src/odom/utils.cu:365-416: 2x2 mean, NaN if
// any x tap is NaN.
template <bool normalize>
__device__ __forceinline__ float3 resize4(const float3 &a00, const float3 &a01, const float3 &a10, const float3 &a11) {
    if (isnan(a00.x) || isnan(a01.x) || isnan(a10.x) || isnan(a11.x)) return make_float3(qnan_f(), qnan_f(), qnan_f());
    float3 n;
    n.x = (a00.x + a01.x + a10.x + a11.x) / 4;
    n.y = (a00.y + a01.y + a10.y + a11.y) / 4;
    n.z = (a00.z + a01.z + a10.z + a11.z) / 4;
    if (normalize) n = normalized(n);
    return n;
}


// tranformMapsKernel (src/odom/utils.cu:206-248) and the planar store of one
// model-map pixel.
__device__ __forceinline__ void store_model_px(const ModelArgs &a, const Map3 &vm, const Map3 &nm, int x, int y,
                                               float3 v, float3 n) {
    if (a.do_transform) {
        const float q = qnan_f();
        float3 vd = make_float3(q, q, q), nd = make_float3(q, q, q);
        const M33 R = load_m33(a.R);
        const float3 t = make_float3(a.t[0], a.t[1], a.t[2]);
        if (!isnan(v.x)) vd = R * v + t;
        if (!isnan(n.x)) nd = R * n;
        v = vd;
        n = nd;
    }
    map_row(vm, 0, y)[x] = v.x;
    map_row(vm, 1, y)[x] = v.y;
    map_row(vm, 2, y)[x] = v.z;
    map_row(nm, 0, y)[x] = n.x;
    map_row(nm, 1, y)[x] = n.y;
    map_row(nm, 2, y)[x] = n.z;
}

__device__ __forceinline__ float3 shfl_xor3(float3 v, int m) {
    return make_float3(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m),
                       __shfl_xor_sync(0xffffffffu, v.z, m));
}

// initICPModel / initICP(maps) (src/odom/RGBDOdometryef.cpp:144-206):
// copyMaps, resizeVMap/NMap x2 and tranformMaps for every level, one 32x32
// tile of the RGBA32F input per block of 16x16 threads, read once: thread
// (tx, ty) imports the 2x2 level-0 pixels of its level-1 pixel and resizes
// them; the level-2 pixel of a 2x2 thread quad (lanes l, l^1, l^16, l^17 of
// one warp) is resized from the quad's untransformed level-1 values.  The
// operations and their order are the reference's (copy, resize of the
// untransformed level above, then the transform).
constexpr int kModelTile = 32;  // level-0 pixels per tile side; block = 16 x 16 threads
__device__ __forceinline__ void model_tile(const ModelArgs &a, int tile) {
    const int tiles_x = (a.cols0 + kModelTile - 1) / kModelTile;
    const int X1 = (tile % tiles_x) * (kModelTile / 2) + threadIdx.x;
    const int Y1 = (tile / tiles_x) * (kModelTile / 2) + threadIdx.y;
    const float q = qnan_f();
    float3 v0[4], n0[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int x = 2 * X1 + (k & 1), y = 2 * Y1 + (k >> 1);
        v0[k] = n0[k] = make_float3(q, q, q);
        if (x < a.cols0 && y < a.rows0 && a.vmap[0].cols > 0) {
            copy_px(a, x, y, v0[k], n0[k]);
            rowp(a.vz, a.vz_pitch, y)[x] = model_depth(rowp(a.v4, a.pitch4, y)[4 * x + 2]);
            store_model_px(a, a.vmap[0], a.nmap[0], x, y, v0[k], n0[k]);
        }
    }
    const Map3 vm1 = a.vmap[1], nm1 = a.nmap[1];
    const bool in1 = X1 < vm1.cols && Y1 < vm1.rows;
    float3 v1 = make_float3(q, q, q), n1 = v1;
    if (in1) {
        v1 = resize4<false>(v0[0], v0[1], v0[2], v0[3]);
        n1 = resize4<true>(n0[0], n0[1], n0[2], n0[3]);
        store_model_px(a, vm1, nm1, X1, Y1, v1, n1);
    }
    const float3 v1x = shfl_xor3(v1, 1), v1y = shfl_xor3(v1, 16), v1xy = shfl_xor3(v1, 17);
    const float3 n1x = shfl_xor3(n1, 1), n1y = shfl_xor3(n1, 16), n1xy = shfl_xor3(n1, 17);
    const Map3 vm2 = a.vmap[2], nm2 = a.nmap[2];
    const int X2 = X1 >> 1, Y2 = Y1 >> 1;
    if (!(threadIdx.x & 1) && !(threadIdx.y & 1) && X2 < vm2.cols && Y2 < vm2.rows)
        store_model_px(a, vm2, nm2, X2, Y2, resize4<false>(v1, v1x, v1y, v1xy), resize4<true>(n1, n1x, n1y, n1xy));
}
__global__ void __launch_bounds__(256) k_model_maps(ModelArgs a) { model_tile(a, blockIdx.x); }
__global__ void __launch_bounds__(256) k_model_maps_b(const ModelArgs *A) {
    __shared__ ModelArgs sa;
    model_tile(stage_args(sa, A[blockIdx.z]), blockIdx.x);
}

// The level-0 photometric images: the depth that the map import wrote
// (verticesToDepthKernel's cut vertex z, see model_depth), copied, and
// bgr2IntensityKernel (src/odom/utils.cu:550-563; RGBA input, so R is
// weighted 0.114).
__device__ __forceinline__ void rgbd_px(const RgbdArgs &a, int x, int y) {
    if (x >= a.img0.cols || y >= a.img0.rows) return;
    if (a.do_depth) at(a.depth0, x, y) = rowp(a.vz, a.vz_pitch, y)[x];
    uchar4 src = *reinterpret_cast<const uchar4 *>(rowp(a.rgba, a.rgba_pitch, y) + 4 * x);
    int value = (float)src.x * 0.114f + (float)src.y * 0.299f + (float)src.z * 0.587f;
    at(a.img0, x, y) = value;
}
// Four consecutive pixels per thread: 16-byte loads of the vertex z and the
// RGBA bytes and 16 / 4-byte stores when the rows allow it (the library's
// buffers always do; the caller's RGBA image needs a 16-byte aligned base and
// pitch), else the same pixels one by one.
__device__ __forceinline__ void rgbd_px4(const RgbdArgs &a, int x0, int y) {
    const int cols = a.img0.cols;
    if (x0 >= cols || y >= a.img0.rows) return;
    const bool vec = x0 + 3 < cols &&
                     !(((uintptr_t)a.rgba | (uintptr_t)a.rgba_pitch | (uintptr_t)a.vz | (uintptr_t)a.vz_pitch) & 15);
    if (!vec) {
        for (int k = 0; k < 4 && x0 + k < cols; ++k) rgbd_px(a, x0 + k, y);
        return;
    }
    const uint4 c4 = *reinterpret_cast<const uint4 *>(rowp(a.rgba, a.rgba_pitch, y) + 4 * x0);
    const unsigned cw[4] = {c4.x, c4.y, c4.z, c4.w};
    unsigned packed = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float r = (float)(cw[k] & 0xff), g = (float)((cw[k] >> 8) & 0xff), b = (float)((cw[k] >> 16) & 0xff);
        int value = r * 0.114f + g * 0.299f + b * 0.587f;
        packed |= ((unsigned)value & 0xffu) << (8 * k);
    }
    *reinterpret_cast<unsigned *>(&at(a.img0, x0, y)) = packed;
    if (a.do_depth)
        *reinterpret_cast<float4 *>(&at(a.depth0, x0, y)) =
            *reinterpret_cast<const float4 *>(rowp(a.vz, a.vz_pitch, y) + x0);
}
__global__ void k_rgbd_level0(RgbdArgs a) {
    rgbd_px4(a, 4 * (blockIdx.x * blockDim.x + threadIdx.x), blockIdx.y * blockDim.y + threadIdx.y);
}
__global__ void k_rgbd_level0_b(const RgbdArgs *A) {
    __shared__ RgbdArgs sa;
    rgbd_px4(stage_args(sa, A[blockIdx.z]), 4 * (blockIdx.x * blockDim.x + threadIdx.x),
             blockIdx.y * blockDim.y + threadIdx.y);
}

__constant__ float c_gauss5x5[25] = {1, 4, 6, 4, 1, 4, 16, 24, 16, 4, 6, 24, 36, 24, 6, 4, 16, 24, 16, 4, 1, 4, 6, 4, 1};
// The same weights as compile-time integers for the unrolled interior loops
// (the reference's `count += weight` on an int: all weights and partial
// counts are small integers, so integer addition gives the same value).
__host__ __device__ constexpr int gauss_w(int i, int j) {
    return (i == 0 || i == 4 ? 1 : (i == 2 ? 6 : 4)) * (j == 0 || j == 4 ? 1 : (j == 2 ? 6 : 4));
}

// pyrDownKernelGaussF (src/odom/utils.cu:332-363) and
// pyrDownKernelIntensityGauss (src/odom/utils.cu:470-500) in one launch:
// masked 5x5 Gaussian, window clamped at cols-1/rows-1 (exclusive), reversed
// kernel index, int count.
//
// The block's source pixels are staged once per tile as
//   d[r][c]  the depth, a NaN stored as +0, and
//   w[r][c]  intensity | (intensity > 0) << 12 | (depth not NaN) << 20.
// Interior outputs (the full 5x5 window inside the image, where the
// reversed index equals the forward one: the weights are symmetric):
//  * intensity sum and both counts are integers (weights 1 4 6 4 1 per
//    axis, products <= 36), and every partial sum of the reference's float
//    intensity loop is an integer below 2^24, hence exact; so they are sums
//    in any order, and separable: a horizontal pass computes, for every
//    staged row and output column, the three 5-tap sums at once on the
//    packed word (fields <= 16 * 255 < 2^12, <= 16 < 2^8, <= 16 < 2^12), and
//    each output adds five of them with the vertical weights (intensity sum
//    <= 65280 and the counts <= 256 each in 16-bit fields);
//  * the depth sum is the reference's chain of 25 fused multiply-adds in its
//    order, over the zeroed tile: a NaN tap contributes fma(+0, w, s) = s
//    (s is never -0: it starts at +0 and no round-to-nearest sum of these
//    terms is -0), the same value as skipping it.
// Border outputs run the reference's loops on the same tiles.
// The staged tile starts 4 source columns left of the block's first
// window column pair (2 X0 - 4, a multiple of 4) and is 2 BX + 8 wide, so
// that it is filled by aligned 4-pixel loads.
constexpr int kGaussTW = 2 * BX + 8;
template <int TR>
struct GaussTile {
    static constexpr int TH = down_th<TR>();
    __align__(16) float d[TH][kGaussTW];
    __align__(16) unsigned w[TH][kGaussTW];
    unsigned hs[TH][BX];  // horizontal weighted intensity sums
    unsigned hc[TH][BX];  // horizontal weighted counts: intensity | depth << 16
};
constexpr unsigned kGaussNz = 1u << 12, kGaussValid = 1u << 20;

// Stages source columns [ox, ox + kGaussTW) x rows [oy, oy + TH), ox a
// multiple of 4: one 4-byte intensity load and one 16-byte depth load per
// 4 pixels where the 4 pixels lie inside the image and the rows are
// aligned, pixel by pixel at the image's edges.  All loads of a thread are
// issued before its first shared-memory store.
template <int TR>
__device__ __forceinline__ void gauss_stage(const GaussArgs &a, int ox, int oy, GaussTile<TR> &g) {
    constexpr int Q = kGaussTW / 4, N = GaussTile<TR>::TH * Q, NT = BX * BY, IT = (N + NT - 1) / NT;
    const int tid = threadIdx.y * BX + threadIdx.x;
    const Img<const uint8_t> isrc = a.isrc;
    const Img<const float> dsrc = a.dsrc;
    const bool dep = a.do_depth != 0;
    const bool aligned = !(((uintptr_t)isrc.data | isrc.pitch) & 3) &&
                         (!dep || !(((uintptr_t)dsrc.data | dsrc.pitch) & 15));
    unsigned iv[IT];
    float4 dv[IT];
#pragma unroll
    for (int k = 0; k < IT; ++k) {
        const int i = tid + k * NT;
        const int ty = i / Q, gx = ox + 4 * (i - ty * Q), gy = oy + ty;
        const float q = qnan_f();
        iv[k] = 0;
        dv[k] = make_float4(q, q, q, q);
        if (i < N && gy >= 0 && gy < isrc.rows) {
            if (aligned && gx >= 0 && gx + 3 < isrc.cols) {
                iv[k] = *reinterpret_cast<const unsigned *>(&at(isrc, gx, gy));
                if (dep) dv[k] = *reinterpret_cast<const float4 *>(&at(dsrc, gx, gy));
            } else {
                float d4[4] = {q, q, q, q};
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (gx + e >= 0 && gx + e < isrc.cols) {
                        iv[k] |= (unsigned)at(isrc, gx + e, gy) << (8 * e);
                        if (dep) d4[e] = at(dsrc, gx + e, gy);
                    }
                dv[k] = make_float4(d4[0], d4[1], d4[2], d4[3]);
            }
        }
    }
#pragma unroll
    for (int k = 0; k < IT; ++k) {
        const int i = tid + k * NT;
        if (i < N) {
            const int ty = i / Q, tx = 4 * (i - ty * Q);
            const float d4[4] = {dv[k].x, dv[k].y, dv[k].z, dv[k].w};
            float o[4];
            unsigned w[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const unsigned v = (iv[k] >> (8 * e)) & 0xffu;
                const bool ok = !isnan(d4[e]);
                o[e] = ok ? d4[e] : 0.f;
                w[e] = v | (v > 0 ? kGaussNz : 0u) | (ok ? kGaussValid : 0u);
            }
            *reinterpret_cast<float4 *>(&g.d[ty][tx]) = make_float4(o[0], o[1], o[2], o[3]);
            *reinterpret_cast<uint4 *>(&g.w[ty][tx]) = make_uint4(w[0], w[1], w[2], w[3]);
        }
    }
}

// Horizontal 5-tap sums of every staged row at the 32 output columns
// (output column X0 + j reads staged columns 2 j + 2 .. 2 j + 6).
template <int TR>
__device__ __forceinline__ void gauss_rows(GaussTile<TR> &g) {
    const int tid = threadIdx.y * BX + threadIdx.x, lane = threadIdx.x;
    for (int r = tid >> 5; r < GaussTile<TR>::TH; r += BY) {
        const unsigned *p = &g.w[r][2 * lane + 2];
        const uint2 w01 = *reinterpret_cast<const uint2 *>(p), w23 = *reinterpret_cast<const uint2 *>(p + 2);
        const unsigned h = (w01.x + p[4]) + 4u * (w01.y + w23.y) + 6u * w23.x;
        g.hs[r][lane] = h & 0xfffu;
        g.hc[r][lane] = ((h >> 12) & 0xffu) | ((h >> 20) << 16);
    }
}

template <int TR>
__device__ __forceinline__ void gauss_out(const GaussArgs &a, const GaussTile<TR> &g, int ox, int oy, int x, int y) {
    const Img<float> ddst = a.ddst;
    const Img<const uint8_t> isrc = a.isrc;
    const Img<uint8_t> idst = a.idst;
    const int do_depth = a.do_depth;
    if (x >= idst.cols || y >= idst.rows) return;
    const int D = 5;
    int tx = min(2 * x - D / 2 + D, isrc.cols - 1);
    int ty = min(2 * y - D / 2 + D, isrc.rows - 1);
    const int cy0 = max(0, 2 * y - D / 2), cx0 = max(0, 2 * x - D / 2);
    const bool interior = cx0 == 2 * x - 2 && tx == 2 * x + 3 && cy0 == 2 * y - 2 && ty == 2 * y + 3;
    if (interior) {
        const int r0 = cy0 - oy, c0 = cx0 - ox;  // even: 2 (y - Y0), 2 (x - X0) + 2
        constexpr unsigned wv[5] = {1, 4, 6, 4, 1};
        unsigned isum = 0, cnt = 0;
#pragma unroll
        for (int i = 0; i < 5; ++i) {
            isum += wv[i] * g.hs[r0 + i][(c0 - 2) >> 1];
            cnt += wv[i] * g.hc[r0 + i][(c0 - 2) >> 1];
        }
        if (do_depth) {
            float sum = 0;
#pragma unroll
            for (int i = 0; i < 5; ++i) {
                const float *r = &g.d[r0 + i][c0];
                const float2 d01 = *reinterpret_cast<const float2 *>(r), d23 = *reinterpret_cast<const float2 *>(r + 2);
                const float v[5] = {d01.x, d01.y, d23.x, d23.y, r[4]};
#pragma unroll
                for (int j = 0; j < 5; ++j) sum = __fmaf_rn(v[j], (float)gauss_w(4 - i, 4 - j), sum);
            }
            at(ddst, x, y) = (float)(sum / (float)(int)(cnt >> 16));
        }
        at(idst, x, y) = ((float)isum / (float)(int)(cnt & 0xffffu));
        return;
    }
    if (do_depth) {
        float sum = 0;
        int count = 0;
        for (int cy = cy0; cy < ty; ++cy) {
            const float *r = g.d[cy - oy] - ox;
            const unsigned *m = g.w[cy - oy] - ox;
            for (int cx = cx0; cx < tx; ++cx) {
                if (m[cx] & kGaussValid) {
                    sum += r[cx] * c_gauss5x5[(ty - cy - 1) * 5 + (tx - cx - 1)];
                    count += c_gauss5x5[(ty - cy - 1) * 5 + (tx - cx - 1)];
                }
            }
        }
        at(ddst, x, y) = (float)(sum / (float)count);
    }
    {
        float sum = 0;
        int count = 0;
        for (int cy = cy0; cy < ty; ++cy) {
            const unsigned *r = g.w[cy - oy] - ox;
            for (int cx = cx0; cx < tx; ++cx) {
                const int v = r[cx] & 0xffu;
                if (v > 0) {
                    sum += v * c_gauss5x5[(ty - cy - 1) * 5 + (tx - cx - 1)];
                    count += c_gauss5x5[(ty - cy - 1) * 5 + (tx - cx - 1)];
                }
            }
        }
        at(idst, x, y) = (sum / (float)count);
    }
}
template <int TR>
__device__ __forceinline__ void gauss_tile(const GaussArgs &a, int X0, int Y0) {
    __shared__ GaussTile<TR> g;
    const int ox = 2 * X0 - 4, oy = 2 * Y0 - 2;
    gauss_stage<TR>(a, ox, oy, g);
    __syncthreads();
    gauss_rows<TR>(g);
    __syncthreads();
#pragma unroll 1
    for (int r = 0; r < TR / BY; ++r) gauss_out<TR>(a, g, ox, oy, X0 + threadIdx.x, Y0 + threadIdx.y + BY * r);
}
__global__ void k_gauss_down(GaussArgs a) {
    gauss_tile<kTileRowsSingle>(a, blockIdx.x * BX, blockIdx.y * kTileRowsSingle);
}
__global__ void k_gauss_down_b(const GaussArgs *A) {
    __shared__ GaussArgs sa;
    gauss_tile<kGaussRowsBatch>(stage_args(sa, A[blockIdx.z]), blockIdx.x * BX, blockIdx.y * kGaussRowsBatch);
}

__constant__ float c_sobel_x[9] = {0.52201f, 0.00000f, -0.52201f, 0.79451f, -0.00000f,
                                   -0.79451f, 0.52201f, 0.00000f, -0.52201f};
__constant__ float c_sobel_y[9] = {0.52201f, 0.79451f, 0.52201f, 0.00000f, 0.00000f,
                                   0.00000f, -0.52201f, -0.79451f, -0.52201f};

// applyKernel (src/odom/utils.cu:582-606), all levels in one launch.  Also
// evaluates, once per frame, the pose-independent preconditions of a
// photometric correspondence (RGBResidual::getProducts,
// src/odom/reduce.cu:782-810: j0 < cols-5, i < rows-1, no zero intensity in
// the [i-2, i+2) x [j0-2, j0+2) window, |grad|^2 >= minScale, depth not NaN)
// into a byte mask, so the per-iteration pass reads one byte per pixel.
//
// The block's source intensities are staged as floats (the values the
// reference's taps convert them to), and each staged row's non-zero bits
// over its 36 columns as one 64-bit mask (two ballots per row), so that a
// pixel tests its 4x4 window with four broadcast loads and shifts.  Tile
// entries outside the image read 0; the masks are used for pixels whose
// window lies inside the image only.
//
// Interior Sobel sums: the reference accumulates all nine taps in order,
// three of them with weight +-0 in each sum.  Those are no-ops: the taps are
// intensities >= 0, so a zero-weight term is +-0, and the running sum is
// never -0 (it starts at +0 and a round-to-nearest sum is -0 only when both
// terms are), so adding +-0 returns it unchanged.  The six others are added
// in the reference's order.
// The staged tile starts 4 columns left of the block's first pixel (X0 - 4,
// a multiple of 4) and is BX + 8 wide, filled by aligned 4-pixel loads.
constexpr int kDerTW4 = BX + 8;
template <int TR>
struct DerivTile {
    __align__(16) float f[der_th<TR>()][kDerTW4];
    unsigned long long nz[der_th<TR>()];
};
template <int TR>
__device__ __forceinline__ void deriv_stage(const Img<const uint8_t> &src, int ox, int oy, DerivTile<TR> &t) {
    constexpr int Q = kDerTW4 / 4, N = der_th<TR>() * Q, NT = BX * BY, IT = (N + NT - 1) / NT;
    const int tid = threadIdx.y * BX + threadIdx.x;
    const bool aligned = !(((uintptr_t)src.data | src.pitch) & 3);
    unsigned v[IT];
#pragma unroll
    for (int k = 0; k < IT; ++k) {
        const int i = tid + k * NT;
        const int ty = i / Q, gx = ox + 4 * (i - ty * Q), gy = oy + ty;
        v[k] = 0;
        if (i < N && gy >= 0 && gy < src.rows) {
            if (aligned && gx >= 0 && gx + 3 < src.cols) {
                v[k] = *reinterpret_cast<const unsigned *>(&at(src, gx, gy));
            } else {
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (gx + e >= 0 && gx + e < src.cols) v[k] |= (unsigned)at(src, gx + e, gy) << (8 * e);
            }
        }
    }
#pragma unroll
    for (int k = 0; k < IT; ++k) {
        const int i = tid + k * NT;
        if (i < N) {
            const int ty = i / Q, tx = 4 * (i - ty * Q);
            *reinterpret_cast<float4 *>(&t.f[ty][tx]) =
                make_float4((float)(v[k] & 0xffu), (float)((v[k] >> 8) & 0xffu), (float)((v[k] >> 16) & 0xffu),
                            (float)(v[k] >> 24));
        }
    }
}

template <int TR>
__device__ __forceinline__ void deriv_px(const DerivArgs &a, int l, const DerivTile<TR> &t, int ox, int oy, int x,
                                         int y) {
    const Img<const uint8_t> src = a.src[l];
    if (x >= src.cols || y >= src.rows) return;
    // the depth the candidate test reads, loaded before the arithmetic
    const float depth = at(a.depth[l], x, y);
    float dxVal = 0, dyVal = 0;
    if (x >= 1 && x <= src.cols - 2 && y >= 1 && y <= src.rows - 2) {
        const float *r0 = &t.f[y - 1 - oy][x - 1 - ox], *r1 = r0 + kDerTW4, *r2 = r1 + kDerTW4;
        // weights c_sobel_x[8 - k], c_sobel_y[8 - k] of tap k = 3 row + column
        dxVal += r0[0] * -0.52201f;
        dyVal += r0[0] * -0.52201f;
        dyVal += r0[1] * -0.79451f;
        dxVal += r0[2] * 0.52201f;
        dyVal += r0[2] * -0.52201f;
        dxVal += r1[0] * -0.79451f;
        dxVal += r1[2] * 0.79451f;
        dxVal += r2[0] * -0.52201f;
        dyVal += r2[0] * 0.52201f;
        dyVal += r2[1] * 0.79451f;
        dxVal += r2[2] * 0.52201f;
        dyVal += r2[2] * 0.52201f;
    } else {
        int kernelIndex = 8;
        for (int j = max(y - 1, 0); j <= min(y + 1, src.rows - 1); j++) {
            const float *r = t.f[j - oy] - ox;
            for (int i = max(x - 1, 0); i <= min(x + 1, src.cols - 1); i++) {
                dxVal += r[i] * c_sobel_x[kernelIndex];
                dyVal += r[i] * c_sobel_y[kernelIndex];
                --kernelIndex;
            }
        }
    }
    const short sx = dxVal, sy = dyVal;
    at(a.dx[l], x, y) = sx;
    at(a.dy[l], x, y) = sy;
    const int cols = src.cols, rows = src.rows, i = y, j0 = x;
    bool c = false;
    if (j0 < cols - 5 && i < rows - 1) {
        bool valid = true;
        if (i >= 2 && j0 >= 2) {  // interior (i + 2 <= rows, j0 + 2 <= cols hold here)
            const int r = y - 2 - oy;
            const unsigned long long m = t.nz[r] & t.nz[r + 1] & t.nz[r + 2] & t.nz[r + 3];
            valid = ((m >> (x - 2 - ox)) & 0xFull) == 0xFull;
        } else {
            for (int u = max(i - 2, 0); u < min(i + 2, rows); u++) {
                const float *r = t.f[u - oy] - ox;
                for (int v = max(j0 - 2, 0); v < min(j0 + 2, cols); v++) valid = valid && (r[v] > 0);
            }
        }
        if (valid) {
            float mTwo = (sx * sx) + (sy * sy);
            c = mTwo >= a.minScale[l] && !isnan(depth);
        }
    }
    at(a.cand[l], x, y) = c ? 1 : 0;
}
template <int TR>
__device__ __forceinline__ void deriv_tile(const DerivArgs &a, const LevelTiles &lt) {
    __shared__ DerivTile<TR> t;
    int l, X0, Y0;
    tile_origin(lt, blockIdx.x, l, X0, Y0);
    const int ox = X0 - 4, oy = Y0 - 2;
    deriv_stage<TR>(a.src[l], ox, oy, t);
    __syncthreads();
    const int lane = threadIdx.x;
    for (int r = threadIdx.y; r < der_th<TR>(); r += BY) {
        const unsigned lo = __ballot_sync(0xffffffffu, t.f[r][lane] > 0);
        const unsigned hi = __ballot_sync(0xffffffffu, lane < kDerTW4 - 32 && t.f[r][32 + (lane & 7)] > 0);
        if (lane == 0) t.nz[r] = ((unsigned long long)hi << 32) | lo;
    }
    __syncthreads();
#pragma unroll 1
    for (int r = 0; r < TR / BY; ++r) deriv_px<TR>(a, l, t, ox, oy, X0 + threadIdx.x, Y0 + threadIdx.y + BY * r);
}
__global__ void k_derivatives(DerivArgs a, LevelTiles t) { deriv_tile<kTileRowsSingle>(a, t); }
__global__ void k_derivatives_b(const DerivArgs *A, LevelTiles t) {
    __shared__ DerivArgs sa;
    deriv_tile<kTileRowsBatch>(stage_args(sa, A[blockIdx.z]), t);
}

inline dim3 grid2(int cols, int rows, int z = 1) { return dim3((cols + BX - 1) / BX, (rows + BY - 1) / BY, z); }
// grid of the window kernels: 32 x th outputs per block
inline dim3 grid_tall(int cols, int rows, int z, int th) { return dim3((cols + BX - 1) / BX, (rows + th - 1) / th, z); }

}  // namespace

cudaError_t launch_pyr_down_depth(Img<const uint16_t> src, Img<uint16_t> dst, cudaStream_t s) {
    k_pyr_down_depth<<<grid_tall(dst.cols, dst.rows, 1, kTileRowsSingle), dim3(BX, BY), 0, s>>>(PyrArgs{src, dst});
    return cudaGetLastError();
}

cudaError_t launch_vmap_nmap(const Img<const uint16_t> *depth, const Map3 *vmap, const Map3 *nmap, const Intr *K,
                             float cutoff, int nlevels, cudaStream_t s) {
    VNArgs a;
    for (int l = 0; l < nlevels; ++l) {
        a.depth[l] = depth[l];
        a.vmap[l] = vmap[l];
        a.nmap[l] = nmap[l];
        a.fx_inv[l] = 1.f / K[l].fx;  // createVMap passes 1.f / fx (src/odom/utils.cu:147)
        a.fy_inv[l] = 1.f / K[l].fy;
        a.cx[l] = K[l].cx;
        a.cy[l] = K[l].cy;
    }
    a.cutoff = cutoff;
    const LevelTiles t = level_tiles(depth[0].cols, depth[0].rows, nlevels, kTileRowsSingle);
    k_vmap_nmap<<<t.total, dim3(BX, BY), 0, s>>>(a, t);
    return cudaGetLastError();
}

cudaError_t launch_model_maps(const float *v4, const float *n4, size_t pitch4, int cols, int rows, const Map3 *vmap,
                              const Map3 *nmap, int nlevels, int do_transform, const float R[9], const float t[3],
                              float *vz, size_t vz_pitch, cudaStream_t s) {
    ModelArgs a{};
    a.v4 = v4;
    a.n4 = n4;
    a.pitch4 = pitch4;
    a.cols0 = cols;
    a.rows0 = rows;
    for (int l = 0; l < nlevels; ++l) {
        a.vmap[l] = vmap[l];
        a.nmap[l] = nmap[l];
    }
    a.do_transform = do_transform;
    for (int i = 0; i < 9; ++i) a.R[i] = R[i];
    for (int i = 0; i < 3; ++i) a.t[i] = t[i];
    a.vz = vz;
    a.vz_pitch = vz_pitch;
    const int tiles = ((cols + kModelTile - 1) / kModelTile) * ((rows + kModelTile - 1) / kModelTile);
    k_model_maps<<<tiles, dim3(kModelTile / 2, kModelTile / 2), 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_rgbd_level0(const float *vz, size_t vz_pitch, const uint8_t *rgba, size_t rgba_pitch, int cols,
                               int rows, Img<float> depth0, Img<uint8_t> img0, int do_depth, cudaStream_t s) {
    k_rgbd_level0<<<grid2((cols + 3) / 4, rows), dim3(BX, BY), 0, s>>>(
        RgbdArgs{vz, vz_pitch, rgba, rgba_pitch, depth0, img0, do_depth});
    return cudaGetLastError();
}

cudaError_t launch_gauss_down(Img<const float> dsrc, Img<float> ddst, Img<const uint8_t> isrc, Img<uint8_t> idst,
                              int do_depth, cudaStream_t s) {
    k_gauss_down<<<grid_tall(idst.cols, idst.rows, 1, kTileRowsSingle), dim3(BX, BY), 0, s>>>(GaussArgs{dsrc, ddst, isrc, idst, do_depth});
    return cudaGetLastError();
}

cudaError_t launch_derivatives(const Img<const uint8_t> *src, const Img<int16_t> *dx, const Img<int16_t> *dy,
                               const Img<const float> *nextDepth, const Img<uint8_t> *cand, const float *minScale,
                               int nlevels, cudaStream_t s) {
    DerivArgs a;
    for (int l = 0; l < nlevels; ++l) {
        a.src[l] = src[l];
        a.dx[l] = dx[l];
        a.dy[l] = dy[l];
        a.depth[l] = nextDepth[l];
        a.cand[l] = cand[l];
        a.minScale[l] = minScale[l];
    }
    const LevelTiles t = level_tiles(src[0].cols, src[0].rows, nlevels, kTileRowsSingle);
    k_derivatives<<<t.total, dim3(BX, BY), 0, s>>>(a, t);
    return cudaGetLastError();
}

cudaError_t launch_pyr_down_depth_batch(const PyrArgs *args, int npairs, int max_cols, int max_rows, cudaStream_t s) {
    k_pyr_down_depth_b<<<grid_tall(max_cols, max_rows, npairs, kTileRowsBatch), dim3(BX, BY), 0, s>>>(args);
    return cudaGetLastError();
}
cudaError_t launch_vmap_nmap_batch(const VNArgs *args, int npairs, int max_cols, int max_rows, cudaStream_t s) {
    const LevelTiles t = level_tiles(max_cols, max_rows, kLevels, kTileRowsBatch);
    k_vmap_nmap_b<<<dim3(t.total, 1, npairs), dim3(BX, BY), 0, s>>>(args, t);
    return cudaGetLastError();
}
cudaError_t launch_model_maps_batch(const ModelArgs *args, int npairs, int max_cols, int max_rows, cudaStream_t s) {
    const int tiles = ((max_cols + kModelTile - 1) / kModelTile) * ((max_rows + kModelTile - 1) / kModelTile);
    k_model_maps_b<<<dim3(tiles, 1, npairs), dim3(kModelTile / 2, kModelTile / 2), 0, s>>>(args);
    return cudaGetLastError();
}
cudaError_t launch_rgbd_level0_batch(const RgbdArgs *args, int npairs, int max_cols, int max_rows, cudaStream_t s) {
    k_rgbd_level0_b<<<grid2((max_cols + 3) / 4, max_rows, npairs), dim3(BX, BY), 0, s>>>(args);
    return cudaGetLastError();
}
cudaError_t launch_gauss_down_batch(const GaussArgs *args, int npairs, int max_cols, int max_rows, cudaStream_t s) {
    k_gauss_down_b<<<grid_tall(max_cols, max_rows, npairs, kGaussRowsBatch), dim3(BX, BY), 0, s>>>(args);
    return cudaGetLastError();
}
cudaError_t launch_derivatives_batch(const DerivArgs *args, int npairs, int max_cols, int max_rows, cudaStream_t s) {
    const LevelTiles t = level_tiles(max_cols, max_rows, kLevels, kTileRowsBatch);
    k_derivatives_b<<<dim3(t.total, 1, npairs), dim3(BX, BY), 0, s>>>(args, t);
    return cudaGetLastError();
}

}  // namespace slamgb
