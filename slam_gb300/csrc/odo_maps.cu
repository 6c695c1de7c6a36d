// Per-frame preprocessing kernels: depth pyramid, vertex/normal maps, model
// map import (RGBA32F -> planar pyramid, rigid transform), photometric
// depth/intensity pyramids and derivative images.
//
// Each kernel restates the arithmetic of the reference kernel it replaces
// (cited per kernel) so results are identical, but several reference
// launches are fused into one: vertex+normal maps for all levels, the whole
// model-map pyramid with its transform, and one launch per pyramid step for
// depth and intensity together.  Memory-bound, 32x8 thread blocks, one thread
// per output pixel.
#include "odo_device.cuh"

namespace slamgb {

namespace {

constexpr int BX = 32, BY = 8;

// pyrDownGaussKernel, src/odom/utils.cu:57-94 (sigma_color = 30, :103).
__device__ __forceinline__ void pyr_px(const PyrArgs &a, int x, int y) {
    const Img<const uint16_t> src = a.src;
    const Img<uint16_t> dst = a.dst;
    if (x >= dst.cols || y >= dst.rows) return;
    const int D = 5;
    const float sigma_color = 30.f;
    int center = at(src, 2 * x, 2 * y);
    int x_mi = max(0, 2 * x - D / 2) - 2 * x;
    int y_mi = max(0, 2 * y - D / 2) - 2 * y;
    int x_ma = min(src.cols, 2 * x - D / 2 + D) - 2 * x;
    int y_ma = min(src.rows, 2 * y - D / 2 + D) - 2 * y;
    float sum = 0, wall = 0;
    const float weights[] = {0.375f, 0.25f, 0.0625f};
    for (int yi = y_mi; yi < y_ma; ++yi) {
        const uint16_t *r = rowp(src.data, src.pitch, 2 * y + yi);
        for (int xi = x_mi; xi < x_ma; ++xi) {
            int val = r[2 * x + xi];
            if (abs(val - center) < 3 * sigma_color) {
                sum += val * weights[abs(xi)] * weights[abs(yi)];
                wall += weights[abs(xi)] * weights[abs(yi)];
            }
        }
    }
    at(dst, x, y) = static_cast<int>(sum / wall);
}
__global__ void k_pyr_down_depth(PyrArgs a) {
    pyr_px(a, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y * blockDim.y + threadIdx.y);
}
__global__ void k_pyr_down_depth_b(const PyrArgs *A) {
    pyr_px(A[blockIdx.z], blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y * blockDim.y + threadIdx.y);
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
__global__ void k_vmap_nmap(VNArgs a) {
    vnmap_px(a, blockIdx.z, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y * blockDim.y + threadIdx.y);
}
__global__ void k_vmap_nmap_b(const VNArgs *A) {
    vnmap_px(A[blockIdx.z / kLevels], blockIdx.z % kLevels, blockIdx.x * blockDim.x + threadIdx.x,
             blockIdx.y * blockDim.y + threadIdx.y);
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

__device__ __forceinline__ void level1_px(const ModelArgs &a, int x, int y, float3 &v, float3 &n) {
    float3 v00, v01, v10, v11, n00, n01, n10, n11;
    copy_px(a, 2 * x, 2 * y, v00, n00);
    copy_px(a, 2 * x + 1, 2 * y, v01, n01);
    copy_px(a, 2 * x, 2 * y + 1, v10, n10);
    copy_px(a, 2 * x + 1, 2 * y + 1, v11, n11);
    v = resize4<false>(v00, v01, v10, v11);
    n = resize4<true>(n00, n01, n10, n11);
}

// initICPModel / initICP(maps) (src/odom/RGBDOdometryef.cpp:144-206):
// copyMaps, resizeVMap/NMap x2 and tranformMaps for every level in one
// launch (blockIdx.z = level); level l re-derives its 2^l x 2^l block from
// the RGBA32F input with the reference's order of operations.
__device__ __forceinline__ void model_px(const ModelArgs &a, int l, int x, int y) {
    const Map3 vm = a.vmap[l], nm = a.nmap[l];
    if (x >= vm.cols || y >= vm.rows) return;
    float3 v, n;
    if (l == 0) {
        copy_px(a, x, y, v, n);
        rowp(a.vz, a.vz_pitch, y)[x] = rowp(a.v4, a.pitch4, y)[4 * x + 2];
    } else if (l == 1) {
        level1_px(a, x, y, v, n);
    } else {
        float3 v00, v01, v10, v11, n00, n01, n10, n11;
        level1_px(a, 2 * x, 2 * y, v00, n00);
        level1_px(a, 2 * x + 1, 2 * y, v01, n01);
        level1_px(a, 2 * x, 2 * y + 1, v10, n10);
        level1_px(a, 2 * x + 1, 2 * y + 1, v11, n11);
        v = resize4<false>(v00, v01, v10, v11);
        n = resize4<true>(n00, n01, n10, n11);
    }
    if (a.do_transform) {
        // tranformMapsKernel, src/odom/utils.cu:206-248
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
__global__ void k_model_maps(ModelArgs a) {
    model_px(a, blockIdx.z, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y * blockDim.y + threadIdx.y);
}
__global__ void k_model_maps_b(const ModelArgs *A) {
    model_px(A[blockIdx.z / kLevels], blockIdx.z % kLevels, blockIdx.x * blockDim.x + threadIdx.x,
             blockIdx.y * blockDim.y + threadIdx.y);
}

// verticesToDepthKernel (src/odom/utils.cu:526-537, cut at maxDepthRGB =
// 6.0, src/odom/RGBDOdometryef.cpp:37) and bgr2IntensityKernel
// (src/odom/utils.cu:550-563; RGBA input, so R is weighted 0.114).
__device__ __forceinline__ void rgbd_px(const RgbdArgs &a, int x, int y) {
    if (x >= a.img0.cols || y >= a.img0.rows) return;
    if (a.do_depth) {
        const float cutOff = 6.0f;
        float z = rowp(a.vz, a.vz_pitch, y)[x];
        at(a.depth0, x, y) = z > cutOff || z <= 0 ? qnan_f() : z;
    }
    uchar4 src = *reinterpret_cast<const uchar4 *>(rowp(a.rgba, a.rgba_pitch, y) + 4 * x);
    int value = (float)src.x * 0.114f + (float)src.y * 0.299f + (float)src.z * 0.587f;
    at(a.img0, x, y) = value;
}
__global__ void k_rgbd_level0(RgbdArgs a) {
    rgbd_px(a, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y * blockDim.y + threadIdx.y);
}
__global__ void k_rgbd_level0_b(const RgbdArgs *A) {
    rgbd_px(A[blockIdx.z], blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y * blockDim.y + threadIdx.y);
}

__constant__ float c_gauss5x5[25] = {1, 4, 6, 4, 1, 4, 16, 24, 16, 4, 6, 24, 36, 24, 6, 4, 16, 24, 16, 4, 1, 4, 6, 4, 1};

// pyrDownKernelGaussF (src/odom/utils.cu:332-363) and
// pyrDownKernelIntensityGauss (src/odom/utils.cu:470-500) in one launch:
// masked 5x5 Gaussian, window clamped at cols-1/rows-1 (exclusive), reversed
// kernel index, int count.
__device__ __forceinline__ void gauss_px(const GaussArgs &a, int x, int y) {
    const Img<const float> dsrc = a.dsrc;
    const Img<float> ddst = a.ddst;
    const Img<const uint8_t> isrc = a.isrc;
    const Img<uint8_t> idst = a.idst;
    const int do_depth = a.do_depth;
    if (x >= idst.cols || y >= idst.rows) return;
    const int D = 5;
    int tx = min(2 * x - D / 2 + D, isrc.cols - 1);
    int ty = min(2 * y - D / 2 + D, isrc.rows - 1);
    const int cy0 = max(0, 2 * y - D / 2), cx0 = max(0, 2 * x - D / 2);
    if (do_depth) {
        float sum = 0;
        int count = 0;
        for (int cy = cy0; cy < ty; ++cy) {
            const float *r = rowp(dsrc.data, dsrc.pitch, cy);
            for (int cx = cx0; cx < tx; ++cx) {
                if (!isnan(r[cx])) {
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
            const uint8_t *r = rowp(isrc.data, isrc.pitch, cy);
            for (int cx = cx0; cx < tx; ++cx) {
                if (r[cx] > 0) {
                    sum += r[cx] * c_gauss5x5[(ty - cy - 1) * 5 + (tx - cx - 1)];
                    count += c_gauss5x5[(ty - cy - 1) * 5 + (tx - cx - 1)];
                }
            }
        }
        at(idst, x, y) = (sum / (float)count);
    }
}
__global__ void k_gauss_down(GaussArgs a) {
    gauss_px(a, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y * blockDim.y + threadIdx.y);
}
__global__ void k_gauss_down_b(const GaussArgs *A) {
    gauss_px(A[blockIdx.z], blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y * blockDim.y + threadIdx.y);
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
__device__ __forceinline__ void deriv_px(const DerivArgs &a, int l, int x, int y) {
    const Img<const uint8_t> src = a.src[l];
    if (x >= src.cols || y >= src.rows) return;
    float dxVal = 0, dyVal = 0;
    int kernelIndex = 8;
    for (int j = max(y - 1, 0); j <= min(y + 1, src.rows - 1); j++) {
        const uint8_t *r = rowp(src.data, src.pitch, j);
        for (int i = max(x - 1, 0); i <= min(x + 1, src.cols - 1); i++) {
            dxVal += (float)r[i] * c_sobel_x[kernelIndex];
            dyVal += (float)r[i] * c_sobel_y[kernelIndex];
            --kernelIndex;
        }
    }
    const short sx = dxVal, sy = dyVal;
    at(a.dx[l], x, y) = sx;
    at(a.dy[l], x, y) = sy;
    const int cols = src.cols, rows = src.rows, i = y, j0 = x;
    bool c = false;
    if (j0 < cols - 5 && i < rows - 1) {
        bool valid = true;
        for (int u = max(i - 2, 0); u < min(i + 2, rows); u++) {
            const uint8_t *r = rowp(src.data, src.pitch, u);
            for (int v = max(j0 - 2, 0); v < min(j0 + 2, cols); v++) valid = valid && (r[v] > 0);
        }
        if (valid) {
            float mTwo = (sx * sx) + (sy * sy);
            c = mTwo >= a.minScale[l] && !isnan(at(a.depth[l], x, y));
        }
    }
    at(a.cand[l], x, y) = c ? 1 : 0;
}
__global__ void k_derivatives(DerivArgs a) {
    deriv_px(a, blockIdx.z, threadIdx.x + blockIdx.x * blockDim.x, threadIdx.y + blockIdx.y * blockDim.y);
}
__global__ void k_derivatives_b(const DerivArgs *A) {
    deriv_px(A[blockIdx.z / kLevels], blockIdx.z % kLevels, threadIdx.x + blockIdx.x * blockDim.x,
             threadIdx.y + blockIdx.y * blockDim.y);
}

inline dim3 grid2(int cols, int rows, int z = 1) { return dim3((cols + BX - 1) / BX, (rows + BY - 1) / BY, z); }

}  // namespace

cudaError_t launch_pyr_down_depth(Img<const uint16_t> src, Img<uint16_t> dst, cudaStream_t s) {
    k_pyr_down_depth<<<grid2(dst.cols, dst.rows), dim3(BX, BY), 0, s>>>(PyrArgs{src, dst});
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
    k_vmap_nmap<<<grid2(depth[0].cols, depth[0].rows, nlevels), dim3(BX, BY), 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_model_maps(const float *v4, const float *n4, size_t pitch4, int cols, int rows, const Map3 *vmap,
                              const Map3 *nmap, int nlevels, int do_transform, const float R[9], const float t[3],
                              float *vz, size_t vz_pitch, cudaStream_t s) {
    ModelArgs a;
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
    k_model_maps<<<grid2(cols, rows, nlevels), dim3(BX, BY), 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_rgbd_level0(const float *vz, size_t vz_pitch, const uint8_t *rgba, size_t rgba_pitch, int cols,
                               int rows, Img<float> depth0, Img<uint8_t> img0, int do_depth, cudaStream_t s) {
    k_rgbd_level0<<<grid2(cols, rows), dim3(BX, BY), 0, s>>>(
        RgbdArgs{vz, vz_pitch, rgba, rgba_pitch, depth0, img0, do_depth});
    return cudaGetLastError();
}

cudaError_t launch_gauss_down(Img<const float> dsrc, Img<float> ddst, Img<const uint8_t> isrc, Img<uint8_t> idst,
                              int do_depth, cudaStream_t s) {
    k_gauss_down<<<grid2(idst.cols, idst.rows), dim3(BX, BY), 0, s>>>(GaussArgs{dsrc, ddst, isrc, idst, do_depth});
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
    k_derivatives<<<grid2(src[0].cols, src[0].rows, nlevels), dim3(BX, BY), 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_pyr_down_depth_batch(const PyrArgs *args, int npairs, int max_cols, int max_rows, cudaStream_t s) {
    k_pyr_down_depth_b<<<grid2(max_cols, max_rows, npairs), dim3(BX, BY), 0, s>>>(args);
    return cudaGetLastError();
}
cudaError_t launch_vmap_nmap_batch(const VNArgs *args, int npairs, int max_cols, int max_rows, cudaStream_t s) {
    k_vmap_nmap_b<<<grid2(max_cols, max_rows, npairs * kLevels), dim3(BX, BY), 0, s>>>(args);
    return cudaGetLastError();
}
cudaError_t launch_model_maps_batch(const ModelArgs *args, int npairs, int max_cols, int max_rows, cudaStream_t s) {
    k_model_maps_b<<<grid2(max_cols, max_rows, npairs * kLevels), dim3(BX, BY), 0, s>>>(args);
    return cudaGetLastError();
}
cudaError_t launch_rgbd_level0_batch(const RgbdArgs *args, int npairs, int max_cols, int max_rows, cudaStream_t s) {
    k_rgbd_level0_b<<<grid2(max_cols, max_rows, npairs), dim3(BX, BY), 0, s>>>(args);
    return cudaGetLastError();
}
cudaError_t launch_gauss_down_batch(const GaussArgs *args, int npairs, int max_cols, int max_rows, cudaStream_t s) {
    k_gauss_down_b<<<grid2(max_cols, max_rows, npairs), dim3(BX, BY), 0, s>>>(args);
    return cudaGetLastError();
}
cudaError_t launch_derivatives_batch(const DerivArgs *args, int npairs, int max_cols, int max_rows, cudaStream_t s) {
    k_derivatives_b<<<grid2(max_cols, max_rows, npairs * kLevels), dim3(BX, BY), 0, s>>>(args);
    return cudaGetLastError();
}

}  // namespace slamgb
