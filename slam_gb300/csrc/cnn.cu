// Warm-start network kernels: forward, loss, backward and Adam, every
// product on the tcgen05 tensor-core GEMM of umma_gemm.cuh (BF16 operands,
// FP32 accumulation).  Layer l's GEMMs:
//   forward      act[l+1][m][co] = relu(sum_k im2col(act[l])[m][k] W[co][k] + b[co])
//   weight grad  dW[co][k]      = sum_m dpre[m][co] im2col(act[l])[m][k]     (split over m)
//   data grad    dcol[m][k]     = sum_co dpre[m][co] W[co][k]
//                dpre_prev      = col2im(dcol) * (act[l] > 0)
// Rounding points (mirrored by the CPU oracle of this network): weights and
// activations are BF16, the output and the loss gradient FP32 (rounded to
// BF16 where they enter a product), dcol and all gradients FP32.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "cnn_internal.h"
#include "umma_gemm.cuh"

namespace slamgb {
namespace cnn {
namespace {

using bf16 = __nv_bfloat16;

__device__ __forceinline__ uint16_t f2bf(float f) {
    bf16 h = __float2bfloat16_rn(f);
    return *reinterpret_cast<uint16_t *>(&h);
}
__device__ __forceinline__ float bf2f(uint16_t u) { return __uint_as_float((uint32_t)u << 16); }
__device__ __forceinline__ uint16_t h2bf(uint16_t h) {
    __half x = *reinterpret_cast<__half *>(&h);
    return f2bf(__half2float(x));
}
__device__ __forceinline__ uint4 pack8(const uint16_t (&v)[8]) {
    uint4 r;
    r.x = v[0] | ((uint32_t)v[1] << 16);
    r.y = v[2] | ((uint32_t)v[3] << 16);
    r.z = v[4] | ((uint32_t)v[5] << 16);
    r.w = v[6] | ((uint32_t)v[7] << 16);
    return r;
}
__device__ __forceinline__ uint4 zero4() { return make_uint4(0, 0, 0, 0); }

// ---------------------------------------------------------------- loaders
// (interface: umma_gemm.cuh -- Row once per CTA row, Col once per K group)
constexpr uint16_t kBf16One = 0x3F80;

// Row-major BF16 [rows][ld], K columns used (ld % 8 == 0, 16-byte aligned base).
struct LdDense {
    const uint16_t *p;
    int rows, K, ld;
    using Row = const uint16_t *;
    using Col = int;
    __device__ Row row(int r) const { return r < rows ? p + (size_t)r * ld : nullptr; }
    __device__ Col col(int k8) const { return k8 * 8; }
    __device__ uint4 load(Row q, int k) const {
        if (!q || k >= K) return zero4();
        if (k + 8 <= K) return __ldg(reinterpret_cast<const uint4 *>(q + k));
        uint16_t v[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) v[j] = (k + j < K) ? q[k + j] : 0;
        return pack8(v);
    }
    // the same slot for the asynchronously fed GEMM (a partial last K group
    // copies its valid bytes and zero-fills the rest)
    __device__ const void *src(Row q, int k, int &bytes) const {
        const int n = (q && k < K) ? min(8, K - k) : 0;
        bytes = 2 * n;
        return n ? static_cast<const void *>(q + k) : static_cast<const void *>(p);
    }
};
// Row-major FP32 [rows][ld] rounded to BF16.
struct LdDenseF32 {
    const float *p;
    int rows, K, ld;
    using Row = const float *;
    using Col = int;
    __device__ Row row(int r) const { return r < rows ? p + (size_t)r * ld : nullptr; }
    __device__ Col col(int k8) const { return k8 * 8; }
    __device__ uint4 load(Row q, int k) const {
        uint16_t v[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) v[j] = (q && k + j < K) ? f2bf(q[k + j]) : 0;
        return pack8(v);
    }
};
// Transposed view of a row-major matrix G[K][ld]: A(r, k) = G[k][r] (BF16,
// or FP32 rounded to BF16).  ones_row >= 0: that row reads 1 for every
// k < K (a bias column of a weight-gradient product).
template <typename T>
struct LdTransT {
    const T *p;
    int rows, K, ld, ones_row;
    using Row = int;
    using Col = int;
    __device__ Row row(int r) const { return r == ones_row ? -2 : (r < rows ? r : -1); }
    __device__ Col col(int k8) const { return k8 * 8; }
    __device__ uint4 load(int r, int k0) const {
        uint16_t v[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int k = k0 + j;
            uint16_t u = 0;
            if (k < K) {
                if (r == -2) u = kBf16One;
                else if (r >= 0) {
                    if constexpr (sizeof(T) == 4) u = f2bf(p[(size_t)k * ld + r]);
                    else u = p[(size_t)k * ld + r];
                }
            }
            v[j] = u;
        }
        return pack8(v);
    }
};
using LdTrans = LdTransT<uint16_t>;
using LdTransF32 = LdTransT<float>;

// Geometry of one ks x ks / stride 2 / pad (ks - 1) / 2 convolution over NHWC input.
struct ConvGeo {
    int B, H, W, C, Ho, Wo, ks;
    __device__ int pad() const { return (ks - 1) >> 1; }
    __device__ int K() const { return ks * ks * C; }
    __device__ int M() const { return B * Ho * Wo; }
    // output position m -> {pixel index of image b's origin, 2 oy - 1, 2 ox - 1, valid}
    __device__ int4 pos(int m) const {
        if (m >= M()) return make_int4(0, 0, 0, 0);
        const int ox = m % Wo, t = m / Wo, oy = t % Ho, b = t / Ho;
        return make_int4(b * H * W, 2 * oy - pad(), 2 * ox - pad(), 1);
    }
    // im2col column k -> {ky, kx, ci, valid}
    __device__ int4 tap(int k) const {
        if (k >= K()) return make_int4(0, 0, 0, 0);
        const int t = k / C, ci = k - t * C, ky = t / ks;
        return make_int4(ky, t - ks * ky, ci, 1);
    }
    // input element of (position, tap), or -1 for the zero padding
    __device__ long long src(const int4 &p, const int4 &t) const {
        if (!p.w || !t.w) return -1;
        const int iy = p.y + t.x, ix = p.z + t.y;
        if (iy < 0 || iy >= H || ix < 0 || ix >= W) return -1;
        return ((long long)p.x + (long long)iy * W + ix) * C + t.z;
    }
};
// Implicit im2col A(m, k) of an NHWC input; C % 8 == 0 so the 8 values of a
// K group share one tap.  F16: the input is FP16 and is converted to BF16.
// (With F16 false the 16-bit values pass through unchanged: BF16 for the BF16
// GEMM, or FP16 for the FP16 GEMM of the first layer.)
template <bool F16>
struct LdIm2col {
    const uint16_t *x;
    ConvGeo g;
    using Row = int4;
    using Col = int4;
    __device__ Row row(int m) const { return g.pos(m); }
    __device__ Col col(int k8) const { return g.tap(k8 * 8); }
    __device__ const void *src(const int4 &p, const int4 &t, int &bytes) const {
        static_assert(!F16, "the asynchronously fed GEMM copies the 16-bit values unconverted");
        const long long o = g.src(p, t);
        bytes = o < 0 ? 0 : 16;
        return o < 0 ? static_cast<const void *>(x) : static_cast<const void *>(x + o);
    }
    __device__ uint4 load(const int4 &p, const int4 &t) const {
        const long long o = g.src(p, t);
        if (o < 0) return zero4();
        uint4 v = __ldg(reinterpret_cast<const uint4 *>(x + o));
        if (!F16) return v;
        const uint16_t *h = reinterpret_cast<const uint16_t *>(&v);
        uint16_t b[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) b[j] = h2bf(h[j]);
        return pack8(b);
    }
};
// Transposed im2col: B(k, m) = im2col(m, k) for 8 consecutive positions m;
// row k = K reads 1 for every valid position (the bias column).
template <bool F16>
struct LdIm2colT {
    const uint16_t *x;
    ConvGeo g;
    struct Col {
        int4 p[8];
    };
    using Row = int4;  // tap; w = 0 invalid, 1 tap, 2 the ones row
    __device__ Row row(int k) const {
        if (k == g.K()) return make_int4(0, 0, 0, 2);
        return g.tap(k);
    }
    __device__ Col col(int m8) const {
        Col c;
#pragma unroll
        for (int j = 0; j < 8; ++j) c.p[j] = g.pos(m8 * 8 + j);
        return c;
    }
    __device__ uint4 load(const int4 &t, const Col &c) const {
        uint16_t v[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            uint16_t u = 0;
            if (t.w == 2) u = c.p[j].w ? kBf16One : 0;
            else {
                const long long o = g.src(c.p[j], t);
                if (o >= 0) u = F16 ? h2bf(x[o]) : x[o];
            }
            v[j] = u;
        }
        return pack8(v);
    }
};

// -------------------------------------------------------------- epilogues
__device__ __forceinline__ uint16_t f2h(float f) {
    __half h = __float2half_rn(f);
    return *reinterpret_cast<uint16_t *>(&h);
}

struct EpBiasAct {  // y = act(v + bias) as BF16
    uint16_t *y;
    const float *bias;
    int N, ld, relu;
    __device__ void operator()(int m, int n0, const float (&v)[8]) const {
        if (n0 + 8 <= N && (ld & 7) == 0) {  // one 16-byte store (bias 32-byte aligned)
            const float4 b0 = *reinterpret_cast<const float4 *>(bias + n0);
            const float4 b1 = *reinterpret_cast<const float4 *>(bias + n0 + 4);
            const float bb[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
            uint16_t o[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                float f = v[j] + bb[j];
                if (relu) f = fmaxf(f, 0.f);
                o[j] = f2bf(f);
            }
            *reinterpret_cast<uint4 *>(y + (size_t)m * ld + n0) = pack8(o);
            return;
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int n = n0 + j;
            if (n < N) {
                float f = v[j] + bias[n];
                if (relu) f = fmaxf(f, 0.f);
                y[(size_t)m * ld + n] = f2bf(f);
            }
        }
    }
};
struct EpBiasF32 {
    float *y;
    const float *bias;
    int N, ld;
    __device__ void operator()(int m, int n0, const float (&v)[8]) const {
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (n0 + j < N) y[(size_t)m * ld + n0 + j] = v[j] + bias[n0 + j];
    }
};
struct EpStore {
    float *y;
    int N, ld;
    __device__ void operator()(int m, int n0, const float (&v)[8]) const {
        if (n0 + 8 <= N && (ld & 3) == 0) {
            float4 *q = reinterpret_cast<float4 *>(y + (size_t)m * ld + n0);
            q[0] = make_float4(v[0], v[1], v[2], v[3]);
            q[1] = make_float4(v[4], v[5], v[6], v[7]);
            return;
        }
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (n0 + j < N) y[(size_t)m * ld + n0 + j] = v[j];
    }
};
// Weight gradient [rows][K] and, from column K, the bias gradient [rows];
// atomic when the product is split over K.
template <bool ATOMIC>
struct EpWeightBias {
    float *w, *bias;
    int K;
    __device__ void operator()(int m, int n0, const float (&v)[8]) const {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int n = n0 + j;
            float *dst = n < K ? w + (size_t)m * K + n : (n == K && bias ? bias + m : nullptr);
            if (!dst) continue;
            if (ATOMIC) atomicAdd(dst, v[j]);
            else *dst = v[j];
        }
    }
};
struct EpMask {  // dst = BF16(v) where the activation is positive, else 0
    uint16_t *dst;
    const uint16_t *act;
    int N, ld;
    __device__ void operator()(int m, int n0, const float (&v)[8]) const {
        if (n0 + 8 <= N && (ld & 7) == 0) {
            const size_t o = (size_t)m * ld + n0;
            const uint4 a4 = *reinterpret_cast<const uint4 *>(act + o);
            const uint16_t *a = reinterpret_cast<const uint16_t *>(&a4);
            uint16_t r[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) r[j] = bf2f(a[j]) > 0.f ? f2bf(v[j]) : (uint16_t)0;
            *reinterpret_cast<uint4 *>(dst + o) = pack8(r);
            return;
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int n = n0 + j;
            if (n < N) {
                const size_t o = (size_t)m * ld + n;
                dst[o] = bf2f(act[o]) > 0.f ? f2bf(v[j]) : (uint16_t)0;
            }
        }
    }
};

// ---------------------------------------------------------------- kernels
// Data gradient of a 3x3 / stride 2 / pad 1 layer (conv2..6; the first
// layer needs none) gathered from dcol in the tap order (ky, kx).
__global__ void k_col2im_mask(const float *dcol, const uint16_t *act, uint16_t *dpre, int B, int H, int W, int C,
                              int Ho, int Wo) {
    const long long n = (long long)B * H * W * C;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int ci = (int)(i % C);
        long long t = i / C;
        const int ix = (int)(t % W);
        t /= W;
        const int iy = (int)(t % H);
        const int b = (int)(t / H);
        float s = 0.f;
        for (int ky = 0; ky < 3; ++ky) {
            const int ty = iy + 1 - ky;
            if (ty < 0 || (ty & 1)) continue;
            const int oy = ty >> 1;
            if (oy >= Ho) continue;
            for (int kx = 0; kx < 3; ++kx) {
                const int tx = ix + 1 - kx;
                if (tx < 0 || (tx & 1)) continue;
                const int ox = tx >> 1;
                if (ox >= Wo) continue;
                s += dcol[(((long long)b * Ho + oy) * Wo + ox) * 9 * C + (ky * 3 + kx) * C + ci];
            }
        }
        dpre[i] = bf2f(act[i]) > 0.f ? f2bf(s) : (uint16_t)0;
    }
}

// loss = mean_b e_b^T M e_b with e = out - label and a symmetric 6x6 metric
// M; dout = d loss / d out = 2 M e / B
__global__ void k_loss(const float *out, const float *label, const float *metric, int B, float *dout, float *loss) {
    __shared__ float red[256];
    float acc = 0.f;
    for (int b = threadIdx.x; b < B; b += blockDim.x) {
        float e[kOut];
        for (int i = 0; i < kOut; ++i) e[i] = out[b * kOut + i] - label[b * kOut + i];
        for (int i = 0; i < kOut; ++i) {
            float me = 0.f;
            for (int j = 0; j < kOut; ++j) me += metric[i * kOut + j] * e[j];
            acc += e[i] * me;
            dout[b * kOut + i] = 2.f * me / (float)B;
        }
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *loss = red[0] / (float)B;
}

__global__ void k_adam(float *p, const float *g, float *m, float *v, size_t n, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

__global__ void k_to_bf16(const float *p, uint16_t *q, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        q[i] = f2bf(p[i]);
}
__global__ void k_to_f16(const float *p, uint16_t *q, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        q[i] = f2h(p[i]);
}
// wt[c][r] = w[r][c] (BF16), rows padded with zeros up to ldt
__global__ void k_transpose_bf16(const uint16_t *w, int rows, int cols, uint16_t *wt, int ldt) {
    const long long n = (long long)cols * ldt;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i / ldt), r = (int)(i % ldt);
        wt[i] = r < rows ? w[(size_t)r * cols + c] : (uint16_t)0;
    }
}

// Network input of pair blockIdx.z: s x s block means of the valid depths
// (metres; 0 where no pixel is valid) and of the intensities (the tracker's
// weighting of the RGBA bytes, 0..1) of both frames, FP16; channels 4-7 are
// derived from them in FP32 before rounding: live - model intensity, live -
// model depth (0 unless both are valid), and the valid-depth fractions of the
// two blocks (the differences keep the precision that FP16 depth loses).
__global__ void k_pack(const PackArgs *args, uint16_t *out) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= kInW || y >= kInH) return;
    const PackArgs a = args[blockIdx.z];
    float md = 0.f, mg = 0.f, ld = 0.f, lg = 0.f;
    int nm = 0, nl = 0;
    for (int dy = 0; dy < a.s; ++dy) {
        const int yy = y * a.s + dy;
        const float4 *mv = reinterpret_cast<const float4 *>(reinterpret_cast<const char *>(a.model_verts) +
                                                            (size_t)yy * a.model_pitch);
        const uchar4 *mc = reinterpret_cast<const uchar4 *>(a.model_rgba + (size_t)yy * a.model_rgba_pitch);
        const uint16_t *dd = reinterpret_cast<const uint16_t *>(reinterpret_cast<const char *>(a.depth) +
                                                                (size_t)yy * a.depth_pitch);
        const uchar4 *lc = reinterpret_cast<const uchar4 *>(a.rgba + (size_t)yy * a.rgba_pitch);
        for (int dx = 0; dx < a.s; ++dx) {
            const int xx = x * a.s + dx;
            const float z = mv[xx].z;
            if (z > 0.f) {
                md += z;
                ++nm;
            }
            const uchar4 c = mc[xx];
            mg += (float)c.x * 0.114f + (float)c.y * 0.299f + (float)c.z * 0.587f;
            const uint16_t d = dd[xx];
            if (d) {
                ld += (float)d * 1e-3f;
                ++nl;
            }
            const uchar4 e = lc[xx];
            lg += (float)e.x * 0.114f + (float)e.y * 0.299f + (float)e.z * 0.587f;
        }
    }
    const float inv = 1.f / (255.f * a.s * a.s), invn = 1.f / (a.s * a.s);
    const float dm = nm ? md / nm : 0.f, dl = nl ? ld / nl : 0.f, gm = mg * inv, gl = lg * inv;
    __align__(16) __half h[8];
    h[0] = __float2half_rn(dm);
    h[1] = __float2half_rn(gm);
    h[2] = __float2half_rn(dl);
    h[3] = __float2half_rn(gl);
    // unscaled and unclamped: the metre-sized depth differences at occlusion
    // edges are part of the signal (clamping them to +-0.25 m, or dropping
    // the derived channels, left the network unable to learn)
    h[4] = __float2half_rn(gl - gm);
    h[5] = __float2half_rn((nm && nl) ? dl - dm : 0.f);
    h[6] = __float2half_rn(nm * invn);
    h[7] = __float2half_rn(nl * invn);
    uint16_t *o = out + (((size_t)blockIdx.z * kInH + y) * kInW + x) * kInC;
    *reinterpret_cast<uint4 *>(o) = *reinterpret_cast<const uint4 *>(h);
}

int grid_for(long long n, int threads) {
    long long b = (n + threads - 1) / threads;
    if (b > 152 * 16) b = 152 * 16;
    return (int)(b < 1 ? 1 : b);
}

// Conv layer l geometry for batch B.
ConvGeo conv_geo(int l, int B) { return ConvGeo{B, kH[l], kW[l], kCin[l], kH[l + 1], kW[l + 1], kKs[l]}; }

template <bool F16 = false, class LA, class LB, class EP>
cudaError_t gemm(const LA &a, const LB &b, const EP &e, int M, int N, int K, int splits, int *err, cudaStream_t s) {
    if (N <= 32) return launch_umma_gemm<32, LA, LB, EP, F16>(a, b, e, M, N, K, splits, 0, err, s);
    if (N <= 64) return launch_umma_gemm<64, LA, LB, EP, F16>(a, b, e, M, N, K, splits, 0, err, s);
    return launch_umma_gemm<128, LA, LB, EP, F16>(a, b, e, M, N, K, splits, 0, err, s);
}

// Forward products (k_umma_gemm_async): the activations' implicit im2col
// rows copied into shared memory by cp.async, the weights by TMA, a few K
// chunks in flight per CTA.
inline int gemm_bn(int N) { return N <= 32 ? 32 : (N <= 64 ? 64 : 128); }
template <bool F16 = false, class LA, class LB, class EP>
cudaError_t gemm_async(const LA &a, const LB &b, const EP &e, int M, int N, int K, int *err, cudaStream_t s,
                       const CUtensorMap *tmb = nullptr) {
    if (N <= 32) return launch_umma_gemm_async<32, LA, LB, EP, F16>(a, b, e, M, N, K, err, s, tmb);
    if (N <= 64) return launch_umma_gemm_async<64, LA, LB, EP, F16>(a, b, e, M, N, K, err, s, tmb);
    return launch_umma_gemm_async<128, LA, LB, EP, F16>(a, b, e, M, N, K, err, s, tmb);
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library).
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

// TMA descriptor of a row-major 16-bit weight matrix [N][K] (K % 8 == 0,
// 16-byte aligned rows): boxes of box_rows (default gemm_bn(N)) rows x 8 K
// values, zero fill outside the matrix.
bool weight_map(CUtensorMap *m, const uint16_t *w, int N, int K, int box_rows = 0) {
    EncodeTiledFn fn = encode_tiled();
    if (!fn || (K % 8) != 0 || (reinterpret_cast<uintptr_t>(w) & 15) != 0) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)N};
    const cuuint64_t strides[1] = {(cuuint64_t)K * 2};
    const cuuint32_t box[2] = {8, (cuuint32_t)(box_rows > 0 ? box_rows : gemm_bn(N))};
    const cuuint32_t estr[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, const_cast<uint16_t *>(w), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

#define CNN_CK(x)                              \
    do {                                       \
        cudaError_t e_ = (x);                  \
        if (e_ != cudaSuccess) return e_;      \
    } while (0)

cudaError_t cnn_forward(Net &n, const uint16_t *input, int B, cudaStream_t s) {
    const ParamLayout &P = n.L;
    const int l1 = kConv, l2 = kConv + 1;
    if (n.tm_state == 0) {  // the weights never move: their TMA descriptors are built once
        bool ok = weight_map(&n.tmw[0], n.wh, kCout[0], w_cols(0));
        for (int l = 1; l < kConv && ok; ++l) ok = weight_map(&n.tmw[l], n.wbf + P.w[l], kCout[l], w_cols(l));
        ok = ok && weight_map(&n.tmw[l1], n.wbf + P.w[l1], kHidden, kFlat);
        ok = ok && weight_map(&n.tmw[l2], n.wbf + P.w[l2], kOut, kHidden);
        n.tm_state = ok ? 1 : -1;
    }
    auto tm = [&](int l) { return n.tm_state == 1 ? &n.tmw[l] : nullptr; };
    for (int l = 0; l < kConv; ++l) {
        const ConvGeo g = conv_geo(l, B);
        const int M = B * g.Ho * g.Wo, N = kCout[l], K = w_cols(l);
        const EpBiasAct ep{n.act[l + 1], n.master + P.b[l], N, N, 1};
        // the first layer in FP16 (the FP16 depth keeps 11 significant bits)
        if (l == 0)
            CNN_CK(gemm_async<true>(LdIm2col<false>{input, g}, LdDense{n.wh, N, K, K}, ep, M, N, K, n.err, s, tm(0)));
        else
            CNN_CK(gemm_async(LdIm2col<false>{n.act[l], g}, LdDense{n.wbf + P.w[l], N, K, K}, ep, M, N, K, n.err, s,
                              tm(l)));
    }
    CNN_CK(gemm_async(LdDense{n.act[kConv], B, kFlat, kFlat}, LdDense{n.wbf + P.w[l1], kHidden, kFlat, kFlat},
                      EpBiasAct{n.hid, n.master + P.b[l1], kHidden, kHidden, 1}, B, kHidden, kFlat, n.err, s, tm(l1)));
    CNN_CK(gemm_async(LdDense{n.hid, B, kHidden, kHidden}, LdDense{n.wbf + P.w[l2], kOut, kHidden, kHidden},
                      EpBiasF32{n.out, n.master + P.b[l2], kOut, kOut}, B, kOut, kHidden, n.err, s, tm(l2)));
    return cudaSuccess;
}

cudaError_t cnn_pack(const PackArgs *args_dev, int n, uint16_t *out, cudaStream_t s) {
    dim3 blk(32, 8), grid((kInW + 31) / 32, (kInH + 7) / 8, n);
    k_pack<<<grid, blk, 0, s>>>(args_dev, out);
    return cudaGetLastError();
}

cudaError_t cnn_loss(Net &n, const float *labels, int B, cudaStream_t s) {
    k_loss<<<1, 256, 0, s>>>(n.out, labels, n.metric, B, n.dout, n.loss);
    return cudaGetLastError();
}

cudaError_t cnn_backward(Net &n, const uint16_t *input, int B, cudaStream_t s) {
    const ParamLayout &P = n.L;
    CNN_CK(cudaMemsetAsync(n.grad, 0, P.total * sizeof(float), s));
    const int l1 = kConv, l2 = kConv + 1;
    // fc2: weight gradient and, from the ones row of B, the bias gradient
    CNN_CK(gemm(LdTransF32{n.dout, kOut, B, kOut, -1}, LdTrans{n.hid, kHidden, B, kHidden, kHidden},
                EpWeightBias<false>{n.grad + P.w[l2], n.grad + P.b[l2], kHidden}, kOut, kHidden + 1, B, 1, n.err,
                s));
    CNN_CK(gemm(LdDenseF32{n.dout, B, kOut, kOut}, LdDense{n.wt + P.wt[l2], kHidden, kOut, P.wt_ld[l2]},
                EpMask{n.dpre_hid, n.hid, kHidden, kHidden}, B, kHidden, kOut, 1, n.err, s));
    // fc1
    CNN_CK(gemm(LdTrans{n.dpre_hid, kHidden, B, kHidden, -1}, LdTrans{n.act[kConv], kFlat, B, kFlat, kFlat},
                EpWeightBias<false>{n.grad + P.w[l1], n.grad + P.b[l1], kFlat}, kHidden, kFlat + 1, B, 1, n.err, s));
    CNN_CK(gemm(LdDense{n.dpre_hid, B, kHidden, kHidden}, LdDense{n.wt + P.wt[l1], kFlat, kHidden, P.wt_ld[l1]},
                EpMask{n.dpre[kConv], n.act[kConv], kFlat, kFlat}, B, kFlat, kHidden, 1, n.err, s));
    CNN_CK(cudaGetLastError());
    // conv layers, last to first
    for (int l = kConv - 1; l >= 0; --l) {
        const ConvGeo g = conv_geo(l, B);
        const int Mpos = B * g.Ho * g.Wo, Co = kCout[l], K = w_cols(l);
        const uint16_t *dp = n.dpre[l + 1];
        // weight gradient (columns 0..K-1) and bias gradient (column K, the
        // ones row of the transposed im2col), split over positions
        const int kchunks = (Mpos + kGemmKChunk - 1) / kGemmKChunk;
        const int tiles = (K + 1 + 127) / 128;
        int splits = 2 * 152 / tiles;
        if (splits > kchunks) splits = kchunks;
        if (splits < 1) splits = 1;
        const LdTrans da{dp, Co, Mpos, Co, -1};
        const EpWeightBias<true> ew{n.grad + P.w[l], n.grad + P.b[l], K};
        if (l == 0)
            CNN_CK(launch_umma_gemm<128>(da, LdIm2colT<true>{input, g}, ew, Co, K + 1, Mpos, splits, 0, n.err, s));
        else
            CNN_CK(launch_umma_gemm<128>(da, LdIm2colT<false>{n.act[l], g}, ew, Co, K + 1, Mpos, splits, 0, n.err, s));
        if (l == 0) break;
        // data gradient
        CNN_CK(gemm(LdDense{dp, Mpos, Co, Co}, LdDense{n.wt + P.wt[l], K, Co, P.wt_ld[l]}, EpStore{n.dcol, K, K},
                    Mpos, K, Co, 1, n.err, s));
        const long long ne = (long long)B * g.H * g.W * g.C;
        k_col2im_mask<<<grid_for(ne, 256), 256, 0, s>>>(n.dcol, n.act[l], n.dpre[l], B, g.H, g.W, g.C, g.Ho, g.Wo);
        CNN_CK(cudaGetLastError());
    }
    return cudaSuccess;
}

cudaError_t cnn_adam(Net &n, float lr, float beta1, float beta2, float eps, cudaStream_t s) {
    n.step += 1;
    const float c1 = 1.f - powf(beta1, (float)n.step), c2 = 1.f - powf(beta2, (float)n.step);
    k_adam<<<grid_for((long long)n.L.total, 256), 256, 0, s>>>(n.master, n.grad, n.adam_m, n.adam_v, n.L.total, lr,
                                                                 beta1, beta2, eps, c1, c2);
    CNN_CK(cudaGetLastError());
    return cnn_refresh_weights(n, s);
}

cudaError_t cnn_refresh_weights(Net &n, cudaStream_t s) {
    k_to_bf16<<<grid_for((long long)n.L.total, 256), 256, 0, s>>>(n.master, n.wbf, n.L.total);
    CNN_CK(cudaGetLastError());
    const size_t n0 = (size_t)w_rows(0) * w_cols(0);
    k_to_f16<<<grid_for((long long)n0, 256), 256, 0, s>>>(n.master + n.L.w[0], n.wh, n0);
    CNN_CK(cudaGetLastError());
    for (int l = 0; l < kLayers; ++l) {
        const long long ne = (long long)w_cols(l) * n.L.wt_ld[l];
        k_transpose_bf16<<<grid_for(ne, 256), 256, 0, s>>>(n.wbf + n.L.w[l], w_rows(l), w_cols(l), n.wt + n.L.wt[l],
                                                          n.L.wt_ld[l]);
        CNN_CK(cudaGetLastError());
    }
    return cudaSuccess;
}

cudaError_t cnn_debug_gemm(const uint16_t *A, const uint16_t *B, float *C, int M, int N, int K, int bn, int layout,
                           int *err, cudaStream_t s) {
    const LdDense la{A, M, K, (K + 7) & ~7}, lb{B, N, K, (K + 7) & ~7};
    const EpStore ep{C, N, N};
    if (layout == 8 || layout == 9) {  // the asynchronously fed kernel (BF16); 9: B by TMA
        CUtensorMap map;
        const CUtensorMap *tmb = nullptr;
        if (layout == 9) {
            if (!weight_map(&map, B, N, K, bn)) return cudaErrorNotSupported;
            tmb = &map;
        }
        if (bn == 32) return launch_umma_gemm_async<32>(la, lb, ep, M, N, K, err, s, tmb);
        if (bn == 64) return launch_umma_gemm_async<64>(la, lb, ep, M, N, K, err, s, tmb);
        if (bn == 128) return launch_umma_gemm_async<128>(la, lb, ep, M, N, K, err, s, tmb);
        return launch_umma_gemm_async<256>(la, lb, ep, M, N, K, err, s, tmb);
    }
    if ((layout & 3) == 2) {  // FP16 operands
        const int lay = layout & 4;
        if (bn == 32) return launch_umma_gemm<32, LdDense, LdDense, EpStore, true>(la, lb, ep, M, N, K, 1, lay, err, s);
        if (bn == 64) return launch_umma_gemm<64, LdDense, LdDense, EpStore, true>(la, lb, ep, M, N, K, 1, lay, err, s);
        if (bn == 128)
            return launch_umma_gemm<128, LdDense, LdDense, EpStore, true>(la, lb, ep, M, N, K, 1, lay, err, s);
        return launch_umma_gemm<256, LdDense, LdDense, EpStore, true>(la, lb, ep, M, N, K, 1, lay, err, s);
    }
    if (bn == 32) return launch_umma_gemm<32>(la, lb, ep, M, N, K, 1, layout, err, s);
    if (bn == 64) return launch_umma_gemm<64>(la, lb, ep, M, N, K, 1, layout, err, s);
    if (bn == 128) return launch_umma_gemm<128>(la, lb, ep, M, N, K, 1, layout, err, s);
    if (bn == 256) return launch_umma_gemm<256>(la, lb, ep, M, N, K, 1, layout, err, s);
    return cudaErrorInvalidValue;
}

}  // namespace cnn
}  // namespace slamgb
