// C ABI of the warm-start network (odo_cnn_*): parameter handling, forward,
// one training step (forward, loss, backward, Adam) and gradients for the
// gradient check.  All device work runs on the network's stream; every entry
// point returns a status and never exits.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/slam_gb300.h"
#include "cnn_internal.h"

using namespace slamgb::cnn;

namespace slamgb {
// transfer.cu: pinned host <-> device copy by a kernel (not the copy engines)
cudaError_t launch_host_copy(void *dst, const void *src, size_t bytes, cudaStream_t s);
}  // namespace slamgb
using slamgb::launch_host_copy;

struct odo_cnn {
    Net net;
    int device = 0;
    cudaStream_t stream = nullptr, own_stream = nullptr;
    std::string err;
    void *arena = nullptr;
    PackArgs *pack_host = nullptr;  // pinned staging of the packer's per-pair arguments
    PackArgs *pack_dev = nullptr;
    cudaEvent_t pack_done = nullptr;  // the staging buffer is free again once this has fired
    uint16_t *in_buf = nullptr;       // network inputs of odo_cnn_propose (max_batch pairs)
    int *flag_host = nullptr;         // pinned copy of the time-out flag of the last proposal
    cudaEvent_t done = nullptr;       // end of the last proposal
};

namespace {

int cfail(odo_cnn_t *n, cudaError_t e, const char *what) {
    if (n) {
        char buf[256];
        std::snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
        n->err = buf;
    }
    if (e == cudaErrorMemoryAllocation) return ODO_ERR_OOM;
    return ODO_ERR_CUDA;
}

#define CCK(call)                                          \
    do {                                                   \
        cudaError_t e_ = (call);                           \
        if (e_ != cudaSuccess) return cfail(n, e_, #call); \
    } while (0)

inline size_t up256(size_t v) { return (v + 255) & ~size_t(255); }

// The tensor cores' bounded waits report through n.err; a time-out leaves
// the outputs undefined and is returned as ODO_ERR_TIMEOUT.
int check_timeout(odo_cnn_t *n) {
    int flag = 0;
    CCK(cudaMemcpyAsync(&flag, n->net.err, sizeof(int), cudaMemcpyDeviceToHost, n->stream));
    CCK(cudaStreamSynchronize(n->stream));
    if (flag) {
        n->err = "tensor-core pipeline wait timed out";
        CCK(cudaMemsetAsync(n->net.err, 0, sizeof(int), n->stream));
        CCK(cudaStreamSynchronize(n->stream));
        return ODO_ERR_TIMEOUT;
    }
    return ODO_OK;
}

// splitmix64 + Box-Muller: He-normal weights, zero biases.
void he_init(const ParamLayout &L, uint64_t seed, std::vector<float> &p) {
    p.assign(L.total, 0.f);
    uint64_t s = seed ^ 0x9E3779B97F4A7C15ull;
    auto next = [&]() {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return ((z >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    };
    for (int l = 0; l < kLayers; ++l) {
        const int rows = w_rows(l), cols = w_cols(l);
        const double fan_in = (double)cols;
        const double sd = (l == kLayers - 1) ? 0.1 * std::sqrt(1.0 / fan_in) : std::sqrt(2.0 / fan_in);
        for (int r = 0; r < rows; ++r)
            for (int c = 0; c < cols; ++c) {
                const double u1 = next(), u2 = next();
                const double v = sd * std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
                p[L.w[l] + (size_t)r * cols + c] = (float)v;
            }
    }
}

}  // namespace

extern "C" {

size_t odo_cnn_param_count(void) { return param_layout().total; }

int odo_cnn_create(int max_batch, odo_cnn_t **out) {
    if (!out || max_batch < 1 || max_batch > 4096) return ODO_ERR_ARG;
    *out = nullptr;
    odo_cnn_t *n = new (std::nothrow) odo_cnn();
    if (!n) return ODO_ERR_OOM;
    Net &N = n->net;
    N.max_batch = max_batch;
    N.L = param_layout();
    auto bail = [&](cudaError_t e, const char *what) {
        int rc = cfail(n, e, what);
        odo_cnn_destroy(n);
        return rc;
    };
    cudaError_t e;
    if ((e = cudaGetDevice(&n->device)) != cudaSuccess) return bail(e, "cudaGetDevice");
    if ((e = cudaStreamCreateWithFlags(&n->own_stream, cudaStreamNonBlocking)) != cudaSuccess)
        return bail(e, "cudaStreamCreate");
    n->stream = n->own_stream;
    // one arena: parameters, optimiser state, activations, gradients, scratch
    const size_t B = (size_t)max_batch;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        size_t r = o;
        o = up256(o + bytes);
        return r;
    };
    const size_t P = N.L.total;
    const size_t o_wh = take((size_t)w_rows(0) * w_cols(0) * 2);
    const size_t o_master = take(P * 4), o_wbf = take(P * 2), o_wt = take(N.L.wt_total * 2), o_grad = take(P * 4),
                 o_m = take(P * 4), o_v = take(P * 4);
    size_t o_act[kConv + 1] = {}, o_dpre[kConv + 1] = {};
    size_t dcol = 0;
    for (int l = 1; l <= kConv; ++l) {
        const size_t elems = B * kH[l] * kW[l] * kCout[l - 1];
        o_act[l] = take(elems * 2);
        o_dpre[l] = take(elems * 2);
    }
    for (int l = 1; l < kConv; ++l) {
        const size_t d = B * kH[l + 1] * kW[l + 1] * 9 * kCin[l];
        if (d > dcol) dcol = d;
    }
    const size_t o_hid = take(B * kHidden * 2), o_dhid = take(B * kHidden * 2), o_out = take(B * kOut * 4),
                 o_dout = take(B * kOut * 4), o_dcol = take(dcol * 4), o_loss = take(4), o_metric = take(kOut * kOut * 4),
                 o_err = take(4);
    if ((e = cudaMalloc(&n->arena, o)) != cudaSuccess) return bail(e, "cudaMalloc(cnn arena)");
    if ((e = cudaMemset(n->arena, 0, o)) != cudaSuccess) return bail(e, "cudaMemset(cnn arena)");
    char *a = (char *)n->arena;
    N.master = (float *)(a + o_master);
    N.wbf = (uint16_t *)(a + o_wbf);
    N.wt = (uint16_t *)(a + o_wt);
    N.wh = (uint16_t *)(a + o_wh);
    N.grad = (float *)(a + o_grad);
    N.adam_m = (float *)(a + o_m);
    N.adam_v = (float *)(a + o_v);
    for (int l = 1; l <= kConv; ++l) {
        N.act[l] = (uint16_t *)(a + o_act[l]);
        N.dpre[l] = (uint16_t *)(a + o_dpre[l]);
    }
    N.hid = (uint16_t *)(a + o_hid);
    N.dpre_hid = (uint16_t *)(a + o_dhid);
    N.out = (float *)(a + o_out);
    N.dout = (float *)(a + o_dout);
    N.dcol = (float *)(a + o_dcol);
    N.loss = (float *)(a + o_loss);
    N.metric = (float *)(a + o_metric);
    N.err = (int *)(a + o_err);
    if ((e = cudaMallocHost(&n->pack_host, sizeof(PackArgs) * B)) != cudaSuccess) return bail(e, "cudaMallocHost");
    if ((e = cudaMalloc(&n->pack_dev, sizeof(PackArgs) * B)) != cudaSuccess) return bail(e, "cudaMalloc(pack)");
    if ((e = cudaEventCreateWithFlags(&n->pack_done, cudaEventDisableTiming)) != cudaSuccess)
        return bail(e, "cudaEventCreate");
    if ((e = cudaEventCreateWithFlags(&n->done, cudaEventDisableTiming)) != cudaSuccess)
        return bail(e, "cudaEventCreate");
    if ((e = cudaMallocHost(&n->flag_host, sizeof(int))) != cudaSuccess) return bail(e, "cudaMallocHost(flag)");
    *n->flag_host = 0;
    float M[kOut * kOut] = {};
    const float sc[kOut] = {10.f, 10.f, 10.f, 6.f, 6.f, 6.f};
    for (int i = 0; i < kOut; ++i) M[i * kOut + i] = sc[i] * sc[i];
    if ((e = cudaMemcpy(N.metric, M, sizeof(M), cudaMemcpyHostToDevice)) != cudaSuccess)
        return bail(e, "cudaMemcpy(metric)");
    *out = n;
    int rc = odo_cnn_init_params(n, 1);
    if (rc != ODO_OK) {
        *out = nullptr;
        odo_cnn_destroy(n);
    }
    return rc;
}

int odo_cnn_destroy(odo_cnn_t *n) {
    if (!n) return ODO_OK;
    if (n->own_stream) cudaStreamSynchronize(n->own_stream);
    if (n->arena) cudaFree(n->arena);
    if (n->pack_host) cudaFreeHost(n->pack_host);
    if (n->pack_dev) cudaFree(n->pack_dev);
    if (n->pack_done) cudaEventDestroy(n->pack_done);
    if (n->done) cudaEventDestroy(n->done);
    if (n->flag_host) cudaFreeHost(n->flag_host);
    if (n->in_buf) cudaFree(n->in_buf);
    if (n->own_stream) cudaStreamDestroy(n->own_stream);
    delete n;
    return ODO_OK;
}

int odo_cnn_set_stream(odo_cnn_t *n, void *stream) {
    if (!n) return ODO_ERR_ARG;
    // NULL: the legacy default stream itself (no graphs are captured here)
    n->stream = stream ? (cudaStream_t)stream : cudaStreamLegacy;
    return ODO_OK;
}

int odo_cnn_set_params(odo_cnn_t *n, const float *host) {
    if (!n || !host) return ODO_ERR_ARG;
    Net &N = n->net;
    CCK(cudaMemcpyAsync(N.master, host, N.L.total * 4, cudaMemcpyHostToDevice, n->stream));
    CCK(cudaMemsetAsync(N.adam_m, 0, N.L.total * 4, n->stream));
    CCK(cudaMemsetAsync(N.adam_v, 0, N.L.total * 4, n->stream));
    N.step = 0;
    CCK(cnn_refresh_weights(N, n->stream));
    CCK(cudaStreamSynchronize(n->stream));
    return ODO_OK;
}

int odo_cnn_get_params(odo_cnn_t *n, float *host) {
    if (!n || !host) return ODO_ERR_ARG;
    CCK(cudaMemcpyAsync(host, n->net.master, n->net.L.total * 4, cudaMemcpyDeviceToHost, n->stream));
    CCK(cudaStreamSynchronize(n->stream));
    return ODO_OK;
}

int odo_cnn_init_params(odo_cnn_t *n, uint64_t seed) {
    if (!n) return ODO_ERR_ARG;
    std::vector<float> p;
    he_init(n->net.L, seed, p);
    return odo_cnn_set_params(n, p.data());
}

int odo_cnn_set_loss_metric(odo_cnn_t *n, const float metric[36]) {
    if (!n || !metric) return ODO_ERR_ARG;
    for (int i = 0; i < kOut; ++i)
        for (int j = 0; j < kOut; ++j)
            if (!(metric[i * kOut + j] == metric[j * kOut + i])) return ODO_ERR_ARG;  // symmetric, no NaN
    CCK(cudaMemcpyAsync(n->net.metric, metric, kOut * kOut * 4, cudaMemcpyHostToDevice, n->stream));
    CCK(cudaStreamSynchronize(n->stream));
    return ODO_OK;
}

int odo_cnn_forward(odo_cnn_t *n, const uint16_t *input, int batch, float *out) {
    if (!n || !input || batch < 1 || batch > n->net.max_batch) return ODO_ERR_ARG;
    CCK(cnn_forward(n->net, input, batch, n->stream));
    if (out) CCK(cudaMemcpyAsync(out, n->net.out, (size_t)batch * kOut * 4, cudaMemcpyDeviceToDevice, n->stream));
    return check_timeout(n);
}

static int pack_input_on(odo_cnn_t *n, const odo_pair *pairs, int npairs, uint16_t *input_dev, cudaStream_t s);

int odo_cnn_pack_input(odo_cnn_t *n, const odo_pair *pairs, int npairs, uint16_t *input_dev) {
    if (!n) return ODO_ERR_ARG;
    return pack_input_on(n, pairs, npairs, input_dev, n->stream);
}

static int pack_input_on(odo_cnn_t *n, const odo_pair *pairs, int npairs, uint16_t *input_dev, cudaStream_t s) {
    if (!n || !pairs || !input_dev || npairs < 1 || npairs > n->net.max_batch) return ODO_ERR_ARG;
    CCK(cudaEventSynchronize(n->pack_done));
    for (int i = 0; i < npairs; ++i) {
        const odo_pair &q = pairs[i];
        const int sc = q.width / kInW;
        if (sc < 1 || q.width != sc * kInW || q.height != sc * kInH || !q.model_verts || !q.model_rgba || !q.depth ||
            !q.rgba || q.model_pitch < (size_t)q.width * 16 || q.model_rgba_pitch < (size_t)q.width * 4 ||
            q.depth_pitch < (size_t)q.width * 2 || q.rgba_pitch < (size_t)q.width * 4)
            return ODO_ERR_ARG;
        n->pack_host[i] = PackArgs{q.model_verts, q.model_pitch, q.model_rgba, q.model_rgba_pitch,
                                   q.depth,       q.depth_pitch, q.rgba,       q.rgba_pitch,
                                   sc};
    }
    CCK(launch_host_copy(n->pack_dev, n->pack_host, sizeof(PackArgs) * npairs, s));
    CCK(cudaEventRecord(n->pack_done, s));
    CCK(cnn_pack(n->pack_dev, npairs, input_dev, s));
    return ODO_OK;
}

int cnn_propose_on(odo_cnn_t *n, const odo_pair *pairs, int npairs, float *out_dev, cudaStream_t st) {
    if (!n || !pairs || !out_dev || npairs < 1) return ODO_ERR_ARG;
    Net &N = n->net;
    if (!n->in_buf) CCK(cudaMalloc(&n->in_buf, (size_t)N.max_batch * kInH * kInW * kInC * 2));
    for (int s = 0; s < npairs; s += N.max_batch) {
        const int m = npairs - s < N.max_batch ? npairs - s : N.max_batch;
        int rc = pack_input_on(n, pairs + s, m, n->in_buf, st);
        if (rc != ODO_OK) return rc;
        CCK(cnn_forward(N, n->in_buf, m, st));
        CCK(cudaMemcpyAsync(out_dev + (size_t)6 * s, N.out, (size_t)m * kOut * 4, cudaMemcpyDeviceToDevice, st));
    }
    CCK(launch_host_copy(n->flag_host, N.err, sizeof(int), st));
    CCK(cudaEventRecord(n->done, st));
    return ODO_OK;
}

int odo_cnn_propose(odo_cnn_t *n, const odo_pair *pairs, int npairs, float *out_dev) {
    if (!n) return ODO_ERR_ARG;
    return cnn_propose_on(n, pairs, npairs, out_dev, n->stream);
}

void *odo_cnn_event(odo_cnn_t *n) { return n ? (void *)n->done : nullptr; }

int odo_cnn_wait(odo_cnn_t *n) {
    if (!n) return ODO_ERR_ARG;
    CCK(cudaEventSynchronize(n->done));
    if (*n->flag_host) {
        *n->flag_host = 0;
        n->err = "tensor-core pipeline wait timed out";
        CCK(cudaMemsetAsync(n->net.err, 0, sizeof(int), n->stream));
        return ODO_ERR_TIMEOUT;
    }
    return ODO_OK;
}

int odo_cnn_gradients(odo_cnn_t *n, const uint16_t *input, const float *labels, int batch, float *grad_host,
                      float *loss_host) {
    if (!n || !input || !labels || batch < 1 || batch > n->net.max_batch) return ODO_ERR_ARG;
    Net &N = n->net;
    CCK(cnn_forward(N, input, batch, n->stream));
    CCK(cnn_loss(N, labels, batch, n->stream));
    CCK(cnn_backward(N, input, batch, n->stream));
    if (grad_host) CCK(cudaMemcpyAsync(grad_host, N.grad, N.L.total * 4, cudaMemcpyDeviceToHost, n->stream));
    if (loss_host) CCK(cudaMemcpyAsync(loss_host, N.loss, 4, cudaMemcpyDeviceToHost, n->stream));
    return check_timeout(n);
}

int odo_cnn_train_step(odo_cnn_t *n, const uint16_t *input, const float *labels, int batch, float lr,
                       float *loss_host) {
    if (!n || !input || !labels || batch < 1 || batch > n->net.max_batch || !(lr > 0.f)) return ODO_ERR_ARG;
    Net &N = n->net;
    CCK(cnn_forward(N, input, batch, n->stream));
    CCK(cnn_loss(N, labels, batch, n->stream));
    CCK(cnn_backward(N, input, batch, n->stream));
    CCK(cnn_adam(N, lr, 0.9f, 0.999f, 1e-8f, n->stream));
    if (loss_host) {
        CCK(cudaMemcpyAsync(loss_host, N.loss, 4, cudaMemcpyDeviceToHost, n->stream));
        return check_timeout(n);
    }
    return ODO_OK;
}

int odo_cnn_debug_gemm(const uint16_t *A, const uint16_t *B, float *C, int M, int N, int K, int bn, int layout,
                       void *stream) {
    if (!A || !B || !C || M < 1 || N < 1 || K < 1 || (layout & 3) > 2 || layout < 0 || (layout > 6 && layout != 8 && layout != 9))
        return ODO_ERR_ARG;
    if (bn != 32 && bn != 64 && bn != 128 && bn != 256) return ODO_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    int *err = nullptr;
    if (cudaMalloc(&err, sizeof(int)) != cudaSuccess) return ODO_ERR_OOM;
    int flag = 0;
    cudaError_t e = cudaMemsetAsync(err, 0, sizeof(int), s);
    if (e == cudaSuccess) e = cnn_debug_gemm(A, B, C, M, N, K, bn, layout, err, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, err, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(err);
    if (e != cudaSuccess) return ODO_ERR_CUDA;
    return flag ? ODO_ERR_TIMEOUT : ODO_OK;
}

const char *odo_cnn_last_error(odo_cnn_t *n) { return n ? n->err.c_str() : "null handle"; }

}  // extern "C"
