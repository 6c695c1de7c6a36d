// Build-time shim that compiles the REFERENCE's own odometry kernels
// (src/odom/reduce.cu, src/odom/utils.cu, included from the reference tree at
// build time; nothing is copied into this repository) into a device-only
// cubin, so the tests can run the reference's arithmetic on the GPU as the
// bit-exact oracle for association indices, valid masks and integer images.
//
// TEST INFRASTRUCTURE ONLY (built by oracle/build_ref.py into oracle/_ref/).
//
// Two source-level adaptations are needed for CUDA 13, neither touching the
// arithmetic:
//  - the non-sync warp shuffle __shfl_down (removed in CUDA 12) maps to
//    __shfl_down_sync over the full warp (every call site is warp-uniform);
//  - the legacy texture reference used by bgr2IntensityKernel
//    (src/odom/utils.cu:548-563, removed in CUDA 12) becomes a pitched
//    global-memory read of the same RGBA texel (point sampling at integer
//    coordinates returns texel (x, y)).
// Compiled with the reference's numeric flags
// (--ftz=true --prec-div=false --prec-sqrt=false, src/CMakeLists.txt:116).

#include <cuda_runtime.h>

#define __shfl_down(v, o) __shfl_down_sync(0xffffffffu, (v), (o))

template <class T, int dim, enum cudaTextureReadMode mode>
struct texture {};

__device__ const unsigned char *g_shim_rgba;
__device__ unsigned long long g_shim_rgba_pitch;

template <class T, int dim, enum cudaTextureReadMode mode>
__device__ T tex2D(texture<T, dim, mode>, int x, int y) {
    return *reinterpret_cast<const T *>(g_shim_rgba + (unsigned long long)y * g_shim_rgba_pitch + x * sizeof(T));
}

#define cudaBindTextureToArray(tex, arr) cudaSuccess
#define cudaUnbindTexture(tex) cudaSuccess

#include "odom/reduce.cu"
#include "odom/utils.cu"

// ---------------------------------------------------------------------------
// Per-pixel probes of the reference's reduction functors.  Each writes the
// functor's own per-pixel output (before any summation).
// ---------------------------------------------------------------------------
// The reference's mat33 / CameraModel constructors are host-only; the
// functors are therefore built in raw storage and their members set in place.
static __device__ __forceinline__ void shim_m33(mat33 &m, const float *p) {
    m.data[0] = make_float3(p[0], p[1], p[2]);
    m.data[1] = make_float3(p[3], p[4], p[5]);
    m.data[2] = make_float3(p[6], p[7], p[8]);
}
template <class T>
struct Raw {
    alignas(T) unsigned char bytes[sizeof(T)];
    __device__ T &get() { return *reinterpret_cast<T *>(bytes); }
};

// ICPReduction::search / getProducts (src/odom/reduce.cu:282-387).
// out_found[i]: 1 if a correspondence was accepted; out_d[3*i..]: the gathered
// model vertex (identifies the gathered pixel); out_prod[29*i..]: products.
extern "C" __global__ void shim_icp_pixels(const float *pose /*Rcurr9 tcurr3 Rprev_inv9 tprev3*/, const float *vc,
                                           const float *nc, const float *vp, const float *np_, unsigned long long pitch,
                                           int cols, int rows, float fx, float fy, float cx, float cy, float dist,
                                           float angle, int *out_found, float *out_d, float *out_prod) {
    Raw<ICPReduction> raw;
    ICPReduction &icp = raw.get();
    shim_m33(icp.Rcurr, pose);
    icp.tcurr = make_float3(pose[9], pose[10], pose[11]);
    shim_m33(icp.Rprev_inv, pose + 12);
    icp.tprev = make_float3(pose[21], pose[22], pose[23]);
    icp.vmap_curr = PtrStep<float>(const_cast<float *>(vc), pitch);
    icp.nmap_curr = PtrStep<float>(const_cast<float *>(nc), pitch);
    icp.vmap_g_prev = PtrStep<float>(const_cast<float *>(vp), pitch);
    icp.nmap_g_prev = PtrStep<float>(const_cast<float *>(np_), pitch);
    icp.intr.fx = fx;
    icp.intr.fy = fy;
    icp.intr.cx = cx;
    icp.intr.cy = cy;
    icp.intr.width = (float)cols;
    icp.intr.height = (float)rows;
    icp.distThres = dist;
    icp.angleThres = angle;
    icp.cols = cols;
    icp.rows = rows;
    icp.N = cols * rows;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < icp.N; i += blockDim.x * gridDim.x) {
        int y = i / cols, x = i - y * cols;
        float3 n, d, s;
        bool f = icp.search(x, y, n, d, s);
        out_found[i] = f ? 1 : 0;
        out_d[3 * i] = f ? d.x : 0.f;
        out_d[3 * i + 1] = f ? d.y : 0.f;
        out_d[3 * i + 2] = f ? d.z : 0.f;
        JtJJtrSE3 v = icp.getProducts(i);
        const float *pv = reinterpret_cast<const float *>(&v);
        for (int k = 0; k < 29; ++k) out_prod[29 * (size_t)i + k] = pv[k];
    }
}

// RGBResidual::getProducts (src/odom/reduce.cu:768-841): DataTerm map and the
// per-pixel int2.
extern "C" __global__ void shim_rgb_residual(float minScale, const short *dIdx, const short *dIdy,
                                             unsigned long long spitch, const float *lastDepth,
                                             const float *nextDepth, unsigned long long fpitch,
                                             const unsigned char *lastImage, const unsigned char *nextImage,
                                             unsigned long long ipitch, int cols, int rows, float maxDepthDelta,
                                             const float *kt_krk /*kt3 krkinv9*/, DataTerm *corres, int2 *out) {
    Raw<RGBResidual> raw;
    RGBResidual &r = raw.get();
    r.minScale = minScale;
    r.dIdx = PtrStepSz<short>(rows, cols, const_cast<short *>(dIdx), spitch);
    r.dIdy = PtrStepSz<short>(rows, cols, const_cast<short *>(dIdy), spitch);
    r.lastDepth = PtrStepSz<float>(rows, cols, const_cast<float *>(lastDepth), fpitch);
    r.nextDepth = PtrStepSz<float>(rows, cols, const_cast<float *>(nextDepth), fpitch);
    r.lastImage = PtrStepSz<unsigned char>(rows, cols, const_cast<unsigned char *>(lastImage), ipitch);
    r.nextImage = PtrStepSz<unsigned char>(rows, cols, const_cast<unsigned char *>(nextImage), ipitch);
    r.corresImg = PtrStepSz<DataTerm>(rows, cols, corres, cols * sizeof(DataTerm));
    r.maxDepthDelta = maxDepthDelta;
    r.kt = make_float3(kt_krk[0], kt_krk[1], kt_krk[2]);
    shim_m33(r.krkinv, kt_krk + 3);
    r.cols = cols;
    r.rows = rows;
    r.N = cols * rows;
    r.pitch = (int)spitch;
    r.imgPitch = (int)ipitch;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < r.N; k += blockDim.x * gridDim.x) out[k] = r.getProducts(k);
}

// RGBReduction::getProducts (src/odom/reduce.cu:512-595).
extern "C" __global__ void shim_rgb_step(const DataTerm *corres, float sigma, const float3 *cloud,
                                         unsigned long long cpitch, float fx, float fy, const short *dIdx,
                                         const short *dIdy, unsigned long long spitch, int cols, int rows,
                                         float *out_prod) {
    Raw<RGBReduction> raw;
    RGBReduction &r = raw.get();
    r.corresImg = PtrStepSz<DataTerm>(rows, cols, const_cast<DataTerm *>(corres), cols * sizeof(DataTerm));
    r.sigma = sigma;
    r.cloud = PtrStepSz<float3>(rows, cols, const_cast<float3 *>(cloud), cpitch);
    r.fx = fx;
    r.fy = fy;
    r.dIdx = PtrStepSz<short>(rows, cols, const_cast<short *>(dIdx), spitch);
    r.dIdy = PtrStepSz<short>(rows, cols, const_cast<short *>(dIdy), spitch);
    r.sobelScale = 0.125f;
    r.cols = cols;
    r.rows = rows;
    r.N = cols * rows;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < r.N; i += blockDim.x * gridDim.x) {
        JtJJtrSE3 v = r.getProducts(i);
        const float *pv = reinterpret_cast<const float *>(&v);
        for (int k = 0; k < 29; ++k) out_prod[29 * (size_t)i + k] = pv[k];
    }
}

// SO3Reduction::getProducts (src/odom/reduce.cu:971-1054).
extern "C" __global__ void shim_so3_pixels(const unsigned char *lastImage, const unsigned char *nextImage,
                                           unsigned long long ipitch, int cols, int rows, const float *mats,
                                           float *out_prod) {
    Raw<SO3Reduction> raw;
    SO3Reduction &r = raw.get();
    r.lastImage = PtrStepSz<unsigned char>(rows, cols, const_cast<unsigned char *>(lastImage), ipitch);
    r.nextImage = PtrStepSz<unsigned char>(rows, cols, const_cast<unsigned char *>(nextImage), ipitch);
    shim_m33(r.imageBasis, mats);
    shim_m33(r.kinv, mats + 9);
    shim_m33(r.krlr, mats + 18);
    r.cols = cols;
    r.rows = rows;
    r.N = cols * rows;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < r.N; k += blockDim.x * gridDim.x) {
        JtJJtrSO3 v = r.getProducts(k);
        const float *pv = reinterpret_cast<const float *>(&v);
        for (int c = 0; c < 11; ++c) out_prod[11 * (size_t)k + c] = pv[c];
    }
}

// Sets the RGBA source that the texture replacement reads.
extern "C" __global__ void shim_set_rgba(const unsigned char *p, unsigned long long pitch) {
    g_shim_rgba = p;
    g_shim_rgba_pitch = pitch;
}

// Rounding-pattern probe for the photometric warp of RGBResidual
// (src/odom/reduce.cu:812-814): evaluates
//   num = d1 * (k0 * x + k1 * y + k2) + t
// for each row of krkinv under every fused/unfused evaluation order the
// expression allows (inner: fma(k1,y,k0*x)+k2 | fma(k0,x,k1*y)+k2 |
// (k0*x+k1*y)+k2; outer: fma(d1,inner,t) | d1*inner+t), then the rounded
// quotients u = rn(num_u / td) and v = rn(num_v / td) for every pairing,
// with this file's division flags.  The tests pick the pairing that the
// reference kernel's own outputs follow.
static __device__ __forceinline__ float shim_inner(int v, float k0, float k1, float k2, float x, float y) {
    if (v == 0) return __fadd_rn(__fmaf_rn(k1, y, __fmul_rn(k0, x)), k2);
    if (v == 1) return __fadd_rn(__fmaf_rn(k0, x, __fmul_rn(k1, y)), k2);
    return __fadd_rn(__fadd_rn(__fmul_rn(k0, x), __fmul_rn(k1, y)), k2);
}
static __device__ __forceinline__ float shim_outer(int v, float d1, float in, float t) {
    return v == 0 ? __fmaf_rn(d1, in, t) : __fadd_rn(__fmul_rn(d1, in), t);
}
extern "C" __global__ void shim_warp_variants(const float *nextDepth, int cols, int rows, const float *kt_krk,
                                              int *out /* [pixel][6 num][6 td][2] */) {
    const float *kr = kt_krk + 3;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < cols * rows; k += blockDim.x * gridDim.x) {
        int y = k / cols, x = k - y * cols;
        float d1 = nextDepth[k];
        float fx = (float)x, fy = (float)y;
        for (int a = 0; a < 6; ++a) {
            float nu = shim_outer(a / 3, d1, shim_inner(a % 3, kr[0], kr[1], kr[2], fx, fy), kt_krk[0]);
            float nv = shim_outer(a / 3, d1, shim_inner(a % 3, kr[3], kr[4], kr[5], fx, fy), kt_krk[1]);
            for (int b = 0; b < 6; ++b) {
                float td = shim_outer(b / 3, d1, shim_inner(b % 3, kr[6], kr[7], kr[8], fx, fy), kt_krk[2]);
                out[((size_t)k * 36 + a * 6 + b) * 2] = __float2int_rn(nu / td);
                out[((size_t)k * 36 + a * 6 + b) * 2 + 1] = __float2int_rn(nv / td);
            }
        }
    }
}
