// Warm-start network: architecture constants and device launchers shared by
// cnn.cu (kernels) and cnn_host.cpp (C ABI, training driver).
//
// Input  [B, 120, 160, 8] FP16 NHWC: model depth (m), model gray (0..1),
//        live depth (m), live gray, four zero channels (16-byte rows).
// conv1..6  3x3, stride 2, pad 1, ReLU: 8->32->64->128->128->128->128
//           (a 7x7 first layer was tried: with Adam's scale-free steps its
//           392-wide fan-in over metre-valued depth made training unstable)
//           (120x160 -> 60x80 -> 30x40 -> 15x20 -> 8x10 -> 4x5 -> 2x3)
// fc1       768 -> 768, ReLU;  fc2  768 -> 6 (translation m, rotation vector rad)
// Weights are stored [out][in] with the conv input index (ky * 3 + kx) * Cin + ci;
// activations are BF16 NHWC after the ReLU, the output FP32.
#pragma once
#include <cuda.h>
#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

namespace slamgb {
namespace cnn {

constexpr int kInH = 120, kInW = 160, kInC = 8;
constexpr int kConv = 6;
constexpr int kCin[kConv] = {8, 32, 64, 128, 128, 128};
constexpr int kCout[kConv] = {32, 64, 128, 128, 128, 128};
constexpr int kKs[kConv] = {3, 3, 3, 3, 3, 3};  // square kernel size (pad (k - 1) / 2, stride 2)
constexpr int kH[kConv + 1] = {120, 60, 30, 15, 8, 4, 2};
constexpr int kW[kConv + 1] = {160, 80, 40, 20, 10, 5, 3};
constexpr int kFlat = 2 * 3 * 128;
constexpr int kHidden = 768;
constexpr int kOut = 6;
constexpr int kLayers = kConv + 2;  // 6 conv + fc1 + fc2

// rows x cols of layer l's weight matrix
constexpr int w_rows(int l) { return l < kConv ? kCout[l] : (l == kConv ? kHidden : kOut); }
constexpr int w_cols(int l) { return l < kConv ? kKs[l] * kKs[l] * kCin[l] : (l == kConv ? kFlat : kHidden); }

struct ParamLayout {
    size_t w[kLayers], b[kLayers];  // float offsets into the parameter vector
    size_t wt[kLayers];             // offsets into the transposed BF16 buffer
    int wt_ld[kLayers];             // row length of each transposed matrix (rows padded to 8)
    size_t total, wt_total;
};

inline ParamLayout param_layout() {
    ParamLayout p{};
    size_t o = 0, t = 0;
    for (int l = 0; l < kLayers; ++l) {
        p.w[l] = o;
        o += (size_t)w_rows(l) * w_cols(l);
        p.b[l] = o;
        o += (size_t)w_rows(l);
        o = (o + 7) & ~size_t(7);  // 16-byte aligned BF16 rows
        p.wt[l] = t;
        p.wt_ld[l] = (w_rows(l) + 7) & ~7;
        t += (size_t)w_cols(l) * p.wt_ld[l];
    }
    p.total = o;
    p.wt_total = t;
    return p;
}

// Device buffers of one network instance for batches of up to max_batch.
struct Net {
    int max_batch = 0;
    ParamLayout L{};
    float *master = nullptr;      // FP32 parameters
    uint16_t *wbf = nullptr;      // BF16 copy (same offsets)
    uint16_t *wt = nullptr;       // BF16 transposed weights (backward data products)
    uint16_t *wh = nullptr;       // FP16 copy of the first layer's weights (FP16 forward product)
    float *grad = nullptr;        // FP32 gradients (same offsets)
    float *adam_m = nullptr, *adam_v = nullptr;
    uint16_t *act[kConv + 1] = {}; // act[0] unused (input is FP16), act[l] = conv l output
    uint16_t *hid = nullptr;      // fc1 output
    float *out = nullptr;         // [B][6]
    float *dout = nullptr;        // d loss / d out
    uint16_t *dpre_hid = nullptr; // d loss / d fc1 pre-activation
    uint16_t *dpre[kConv + 1] = {}; // dpre[l]: d loss / d conv l pre-activation (l = 1..6)
    float *dcol = nullptr;        // backward im2col scratch
    float *loss = nullptr;        // device scalar
    float *metric = nullptr;      // loss metric, 6x6 row-major
    int *err = nullptr;           // tensor-core wait time-out flag
    int step = 0;
    // TMA descriptors of the forward weights ([N][K] BF16 / FP16, boxes of
    // BN rows x 8 K values): 0 not built yet, 1 built, -1 unavailable
    CUtensorMap tmw[kLayers];
    int tm_state = 0;
};

// One frame pair's inputs for the network input packer: level-0 images of
// size (160 s) x (120 s), reduced by s x s block means.
struct PackArgs {
    const float *model_verts;  // RGBA32F camera-frame vertices (z = depth)
    size_t model_pitch;
    const uint8_t *model_rgba;
    size_t model_rgba_pitch;
    const uint16_t *depth;     // live depth, mm
    size_t depth_pitch;
    const uint8_t *rgba;       // live RGBA
    size_t rgba_pitch;
    int s;
};

// kernels (cnn.cu)
cudaError_t cnn_pack(const PackArgs *args_dev, int n, uint16_t *out, cudaStream_t s);
cudaError_t cnn_forward(Net &n, const uint16_t *input, int B, cudaStream_t s);
cudaError_t cnn_loss(Net &n, const float *labels, int B, cudaStream_t s);
cudaError_t cnn_backward(Net &n, const uint16_t *input, int B, cudaStream_t s);
cudaError_t cnn_adam(Net &n, float lr, float beta1, float beta2, float eps, cudaStream_t s);
cudaError_t cnn_refresh_weights(Net &n, cudaStream_t s);  // master -> BF16 copies (plain and transposed)
cudaError_t cnn_debug_gemm(const uint16_t *A, const uint16_t *B, float *C, int M, int N, int K, int bn, int layout,
                           int *err, cudaStream_t s);

}  // namespace cnn
}  // namespace slamgb
