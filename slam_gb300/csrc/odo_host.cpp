// Host driver and C ABI of the tracker (include/slam_gb300.h).
//
// Mirrors RGBDOdometryef (src/odom/RGBDOdometryef.cpp): the same buffers per
// pyramid level, the same call sequence and statistics, but
//  - frame inputs are device pointers instead of GL textures;
//  - every call is asynchronous on the handle's stream except
//    odo_get_incremental_transformation, which blocks once at the end;
//  - the Gauss-Newton loop runs on the device (see odo_track.cu), and in
//    ODO_MODE_GRAPH a whole tracking call is one CUDA graph launch;
//  - errors are returned, never fatal.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/slam_gb300.h"
#include "odo_internal.h"
#include "se3_math.h"

using namespace slamgb;

namespace {

inline size_t round_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

struct Arena {
    std::vector<void *> blocks;
    void *alloc(size_t bytes, cudaError_t &err) {
        void *p = nullptr;
        err = cudaMalloc(&p, bytes ? bytes : 1);
        if (err != cudaSuccess) return nullptr;
        blocks.push_back(p);
        return p;
    }
    void release() {
        for (void *p : blocks) cudaFree(p);
        blocks.clear();
    }
};

template <typename T>
struct DImg {
    T *data = nullptr;
    size_t pitch = 0;
    int cols = 0, rows = 0;
    Img<T> img() const { return Img<T>{data, pitch, cols, rows}; }
    Img<const T> cimg() const { return Img<const T>{data, pitch, cols, rows}; }
};

struct DMap {
    float *data = nullptr;
    size_t pitch = 0;
    int cols = 0, rows = 0;
    Map3 map() const { return Map3{data, pitch, cols, rows}; }
};

using GraphKey = std::tuple<int, int, int, int, int, int, int, int>;

}  // namespace

struct odo_handle {
    int width = 0, height = 0;
    float cx = 0, cy = 0, fx = 0, fy = 0, distThres = 0, angleThres = 0;
    int device = 0, sm_count = 0;
    cudaStream_t own_stream = nullptr, stream = nullptr;
    // set_stream(NULL): work runs on own_stream, ordered after the work
    // already queued on the legacy default stream (where the caller's inputs
    // were produced); graphs cannot be captured on the legacy stream itself
    bool follow_legacy = true;
    cudaEvent_t order_ev = nullptr;
    Arena arena;
    int dims_w[kLevels], dims_h[kLevels];
    DImg<uint16_t> depth_tmp[kLevels];
    DMap vmap_curr[kLevels], nmap_curr[kLevels], vmap_prev[kLevels], nmap_prev[kLevels];
    DImg<float> lastDepth[kLevels], nextDepth[kLevels];
    DImg<uint8_t> lastImage[kLevels], imgA[kLevels], imgB[kLevels];
    DImg<int16_t> dIdx[kLevels], dIdy[kLevels];
    DImg<Corr> corr[kLevels];
    DImg<uint8_t> cand[kLevels];
    DImg<float> vz;
    ReduceWs ws{};
    TrackState *st_dev = nullptr;
    TrackState *st_host = nullptr;  // pinned
    double *dbg_dev = nullptr;
    float *dbg_params = nullptr;
    int parity = 0;  // nextImage = parity ? imgB : imgA, lastNextImage = the other
    int mode = ODO_MODE_GRAPH;
    int precision = ODO_PREC_FP32;
    // bounded waits of the persistent kernel (odo_debug_set_wait_limit)
    long long spin_limit = kPersistentSpinLimit;
    int absent_block = -1;
    TrackLaunch cfg[kLevels];
    std::map<GraphKey, cudaGraphExec_t> graphs;
    std::string last_error;

    DImg<uint8_t> *nextImage() { return parity ? imgB : imgA; }
    DImg<uint8_t> *lastNextImage() { return parity ? imgA : imgB; }
    Intr intr(int l) const {
        // CameraModel::operator()(level), src/sensors/Camera.h:14-18
        int div = 1 << l;
        return Intr{fx / div, fy / div, cx / div, cy / div};
    }
};

namespace {

int fail(odo_t *h, cudaError_t e, const char *what) {
    if (h) {
        char buf[256];
        std::snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
        h->last_error = buf;
    }
    return e == cudaErrorMemoryAllocation ? ODO_ERR_OOM : ODO_ERR_CUDA;
}

#define CK(call)                                              \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return fail(h, e_, #call);     \
    } while (0)

template <typename T>
cudaError_t alloc_img(odo_t *h, DImg<T> &im, int cols, int rows) {
    cudaError_t e;
    im.cols = cols;
    im.rows = rows;
    im.pitch = round_up((size_t)cols * sizeof(T), 256);
    im.data = (T *)h->arena.alloc(im.pitch * rows, e);
    if (e == cudaSuccess) e = cudaMemset(im.data, 0, im.pitch * rows);
    return e;
}

cudaError_t alloc_map(odo_t *h, DMap &m, int cols, int rows) {
    cudaError_t e;
    m.cols = cols;
    m.rows = rows;
    m.pitch = round_up((size_t)cols * sizeof(float), 256);
    m.data = (float *)h->arena.alloc(m.pitch * rows * 3, e);
    if (e == cudaSuccess) e = cudaMemset(m.data, 0, m.pitch * rows * 3);
    return e;
}

// pow(minimumGradientMagnitudes[l], 2) / pow(sobelScale, 2) with the
// magnitudes 5/3/1 and sobelScale 1/8 (src/odom/RGBDOdometryef.cpp:34-35,
// 108-110, 439).
float min_scale(int l) {
    const float minGrad[kLevels] = {5, 3, 1};
    const float sobelScale = (float)(1.0 / pow(2.0, 3));
    return (float)(pow(minGrad[l], 2.0) / pow((double)sobelScale, 2.0));
}

cudaError_t enqueue_derivatives(odo_t *h, cudaStream_t s) {
    Img<const uint8_t> src[kLevels];
    Img<int16_t> dx[kLevels], dy[kLevels];
    Img<const float> nd[kLevels];
    Img<uint8_t> cand[kLevels];
    float ms[kLevels];
    for (int l = 0; l < kLevels; ++l) {
        src[l] = h->nextImage()[l].cimg();
        dx[l] = h->dIdx[l].img();
        dy[l] = h->dIdy[l].img();
        nd[l] = h->nextDepth[l].cimg();
        cand[l] = h->cand[l].img();
        ms[l] = min_scale(l);
    }
    return launch_derivatives(src, dx, dy, nd, cand, ms, kLevels, s);
}

LevelArgs level_args(odo_t *h, int l) {
    LevelArgs L{};
    L.level = l;
    L.cols = h->dims_w[l];
    L.rows = h->dims_h[l];
    L.K = h->intr(l);
    L.vmap_curr = h->vmap_curr[l].map();
    L.nmap_curr = h->nmap_curr[l].map();
    L.vmap_prev = h->vmap_prev[l].map();
    L.nmap_prev = h->nmap_prev[l].map();
    L.distThres = h->distThres;
    L.angleThres = h->angleThres;
    L.dIdx = h->dIdx[l].cimg();
    L.dIdy = h->dIdy[l].cimg();
    L.lastDepth = h->lastDepth[l].cimg();
    L.nextDepth = h->nextDepth[l].cimg();
    L.lastImage = h->lastImage[l].cimg();
    L.nextImage = h->nextImage()[l].cimg();
    L.corr = h->corr[l].img();
    L.cand = h->cand[l].cimg();
    const float sobelScale = (float)(1.0 / pow(2.0, 3));
    L.minScale = min_scale(l);
    L.maxDepthDelta = 0.07f;  // maxDepthDeltaRGB, src/odom/RGBDOdometryef.cpp:36
    L.sobelScale = sobelScale;
    return L;
}

void default_launch(odo_t *h) {
    for (int l = 0; l < kLevels; ++l) {
        const int n = h->dims_w[l] * h->dims_h[l];
        TrackLaunch c;
        c.threads = 256;
        int b = (n + c.threads * 2 - 1) / (c.threads * 2);
        if (b > 2 * h->sm_count) b = 2 * h->sm_count;
        if (b < 1) b = 1;
        c.blocks_icp = b;
        c.blocks_rgb = b;
        c.precision = h->precision;
        h->cfg[l] = c;
    }
}

// Orders the handle's stream after the work queued on the legacy default
// stream (see odo_handle::follow_legacy).
cudaError_t follow_caller(odo_t *h) {
    if (!h->follow_legacy) return cudaSuccess;
    cudaError_t e = cudaEventRecord(h->order_ev, 0);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(h->stream, h->order_ev, 0);
    return e;
}

void drop_graphs(odo_t *h) {
    for (auto &kv : h->graphs) cudaGraphExecDestroy(kv.second);
    h->graphs.clear();
}

// Enqueues one whole tracking call on the stream.
cudaError_t enqueue_track(odo_t *h, const int iterations[kLevels], int icp, int rgb, int so3) {
    cudaStream_t s = h->stream;
    // the state travels by a copy kernel (not queued behind the caller's
    // bulk copies on the copy engines)
    cudaError_t e = launch_host_copy(h->st_dev, h->st_host, sizeof(TrackState), s);
    if (e != cudaSuccess) return e;
    if (rgb && (e = enqueue_derivatives(h, s)) != cudaSuccess) return e;
    if (so3) {
        const int L2 = 2;
        if ((e = launch_so3(h->st_dev, h->lastNextImage()[L2].cimg(), h->nextImage()[L2].cimg(), h->intr(L2), s)) !=
            cudaSuccess)
            return e;
    }
    if ((e = launch_track_begin(h->st_dev, s)) != cudaSuccess) return e;
    for (int l = kLevels - 1; l >= 0; --l) {
        if (iterations[l] == 0) continue;
        LevelArgs L = level_args(h, l);
        TrackLaunch c = h->cfg[l];
        c.precision = h->precision;
        if (!rgb) c.blocks_rgb = 1;
        if (h->mode == ODO_MODE_PERSISTENT) {
            if ((e = cudaMemsetAsync(h->ws.counters, 0, 4 * sizeof(unsigned), s)) != cudaSuccess) return e;
            if ((e = launch_level_persistent(L, h->st_dev, h->ws, c, iterations[l], h->sm_count, s, h->spin_limit,
                                             h->absent_block)) != cudaSuccess)
                return e;
        } else {
            for (int j = 0; j < iterations[l]; ++j)
                if ((e = launch_level_iteration(L, h->st_dev, h->ws, c, j, s)) != cudaSuccess) return e;
        }
    }
    if ((e = launch_track_end(h->st_dev, s)) != cudaSuccess) return e;
    return launch_host_copy(h->st_host, h->st_dev, sizeof(TrackState), s);
}

int check_handle(odo_t *h) { return h ? ODO_OK : ODO_ERR_ARG; }

int copy_level(odo_t *h, int which, int level, void *host, size_t bytes, bool upload) {
    if (!h || level < 0 || level >= kLevels || !host) return ODO_ERR_ARG;
    void *dptr = nullptr;
    size_t pitch = 0, elem = 0;
    int cols = h->dims_w[level], rows = h->dims_h[level];
    switch (which) {
        case 0: dptr = h->depth_tmp[level].data; pitch = h->depth_tmp[level].pitch; elem = 2; break;
        case 1: dptr = h->vmap_curr[level].data; pitch = h->vmap_curr[level].pitch; elem = 4; rows *= 3; break;
        case 2: dptr = h->nmap_curr[level].data; pitch = h->nmap_curr[level].pitch; elem = 4; rows *= 3; break;
        case 3: dptr = h->vmap_prev[level].data; pitch = h->vmap_prev[level].pitch; elem = 4; rows *= 3; break;
        case 4: dptr = h->nmap_prev[level].data; pitch = h->nmap_prev[level].pitch; elem = 4; rows *= 3; break;
        case 5: dptr = h->lastDepth[level].data; pitch = h->lastDepth[level].pitch; elem = 4; break;
        case 6: dptr = h->nextDepth[level].data; pitch = h->nextDepth[level].pitch; elem = 4; break;
        case 7: dptr = h->lastImage[level].data; pitch = h->lastImage[level].pitch; elem = 1; break;
        case 8: dptr = h->nextImage()[level].data; pitch = h->nextImage()[level].pitch; elem = 1; break;
        case 9: dptr = h->lastNextImage()[level].data; pitch = h->lastNextImage()[level].pitch; elem = 1; break;
        case 10: dptr = h->dIdx[level].data; pitch = h->dIdx[level].pitch; elem = 2; break;
        case 11: dptr = h->dIdy[level].data; pitch = h->dIdy[level].pitch; elem = 2; break;
        case 12: dptr = h->corr[level].data; pitch = h->corr[level].pitch; elem = 16; break;
        default: return ODO_ERR_ARG;
    }
    const size_t need = (size_t)cols * elem * rows;
    if (bytes < need) return ODO_ERR_ARG;
    if (upload)
        CK(cudaMemcpy2DAsync(dptr, pitch, host, cols * elem, cols * elem, rows, cudaMemcpyHostToDevice, h->stream));
    else
        CK(cudaMemcpy2DAsync(host, cols * elem, dptr, pitch, cols * elem, rows, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return ODO_OK;
}

}  // namespace

extern "C" {

int odo_create(int width, int height, float cx, float cy, float fx, float fy, float distThresh, float angleThresh,
               odo_t **out) {
    if (!out || width < 16 || height < 16 || width > 8192 || height > 8192 || !(fx != 0) || !(fy != 0))
        return ODO_ERR_ARG;
    *out = nullptr;
    odo_t *h = new (std::nothrow) odo_t();
    if (!h) return ODO_ERR_OOM;
    h->width = width;
    h->height = height;
    h->cx = cx;
    h->cy = cy;
    h->fx = fx;
    h->fy = fy;
    h->distThres = distThresh;
    h->angleThres = angleThresh;
    auto bail = [&](cudaError_t e, const char *what) {
        int rc = fail(h, e, what);
        odo_destroy(h);
        return rc;
    };
    cudaError_t e;
    if ((e = cudaGetDevice(&h->device)) != cudaSuccess) return bail(e, "cudaGetDevice");
    if ((e = cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, h->device)) != cudaSuccess)
        return bail(e, "cudaDeviceGetAttribute");
    if ((e = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking)) != cudaSuccess)
        return bail(e, "cudaStreamCreate");
    if ((e = cudaEventCreateWithFlags(&h->order_ev, cudaEventDisableTiming)) != cudaSuccess)
        return bail(e, "cudaEventCreate");
    h->stream = h->own_stream;
    for (int l = 0; l < kLevels; ++l) {
        int w = width >> l, hh = height >> l;
        h->dims_w[l] = w;
        h->dims_h[l] = hh;
        if ((e = alloc_img(h, h->depth_tmp[l], w, hh)) != cudaSuccess ||
            (e = alloc_map(h, h->vmap_curr[l], w, hh)) != cudaSuccess ||
            (e = alloc_map(h, h->nmap_curr[l], w, hh)) != cudaSuccess ||
            (e = alloc_map(h, h->vmap_prev[l], w, hh)) != cudaSuccess ||
            (e = alloc_map(h, h->nmap_prev[l], w, hh)) != cudaSuccess ||
            (e = alloc_img(h, h->lastDepth[l], w, hh)) != cudaSuccess ||
            (e = alloc_img(h, h->nextDepth[l], w, hh)) != cudaSuccess ||
            (e = alloc_img(h, h->lastImage[l], w, hh)) != cudaSuccess ||
            (e = alloc_img(h, h->imgA[l], w, hh)) != cudaSuccess ||
            (e = alloc_img(h, h->imgB[l], w, hh)) != cudaSuccess ||
            (e = alloc_img(h, h->dIdx[l], w, hh)) != cudaSuccess ||
            (e = alloc_img(h, h->dIdy[l], w, hh)) != cudaSuccess ||
            (e = alloc_img(h, h->corr[l], w, hh)) != cudaSuccess ||
            (e = alloc_img(h, h->cand[l], w, hh)) != cudaSuccess)
            return bail(e, "device allocation");
    }
    if ((e = alloc_img(h, h->vz, width, height)) != cudaSuccess) return bail(e, "device allocation");
    h->ws.max_blocks = 4096;
    h->ws.icp_part = (float *)h->arena.alloc(sizeof(float) * 32 * h->ws.max_blocks, e);
    if (e == cudaSuccess) h->ws.rgb_part = (float *)h->arena.alloc(sizeof(float) * 32 * h->ws.max_blocks, e);
    if (e == cudaSuccess) h->ws.res_part = (int *)h->arena.alloc(sizeof(int) * 2 * h->ws.max_blocks, e);
    if (e == cudaSuccess) h->ws.counters = (unsigned *)h->arena.alloc(sizeof(unsigned) * 4, e);
    if (e == cudaSuccess) e = cudaMemset(h->ws.counters, 0, sizeof(unsigned) * 4);
    if (e == cudaSuccess) h->st_dev = (TrackState *)h->arena.alloc(sizeof(TrackState), e);
    if (e == cudaSuccess) h->dbg_dev = (double *)h->arena.alloc(sizeof(double) * 64, e);
    if (e == cudaSuccess) h->dbg_params = (float *)h->arena.alloc(sizeof(float) * 32, e);
    if (e == cudaSuccess) e = cudaMallocHost(&h->st_host, sizeof(TrackState));
    if (e != cudaSuccess) return bail(e, "device allocation");
    std::memset(h->st_host, 0, sizeof(TrackState));
    // initial statistics, src/odom/RGBDOdometryef.cpp:26-33
    h->st_host->lastICPCount = h->st_host->lastRGBCount = h->st_host->lastSO3Count = (float)(width * height);
    for (int k = 0; k < 9; ++k) h->st_host->resultR[k] = (k % 4 == 0) ? 1.0 : 0.0;
    if ((e = cudaMemcpy(h->st_dev, h->st_host, sizeof(TrackState), cudaMemcpyHostToDevice)) != cudaSuccess)
        return bail(e, "cudaMemcpy");
    if ((e = cudaDeviceSynchronize()) != cudaSuccess) return bail(e, "cudaDeviceSynchronize");
    default_launch(h);
    *out = h;
    return ODO_OK;
}

int odo_destroy(odo_t *h) {
    if (!h) return ODO_ERR_ARG;
    if (h->stream) cudaStreamSynchronize(h->stream);
    drop_graphs(h);
    h->arena.release();
    if (h->st_host) cudaFreeHost(h->st_host);
    if (h->order_ev) cudaEventDestroy(h->order_ev);
    if (h->own_stream) cudaStreamDestroy(h->own_stream);
    delete h;
    return ODO_OK;
}

int odo_set_stream(odo_t *h, void *stream) {
    if (!h) return ODO_ERR_ARG;
    cudaStream_t s = stream ? (cudaStream_t)stream : h->own_stream;
    if (s != h->stream) {
        CK(cudaStreamSynchronize(h->stream));
        drop_graphs(h);
        h->stream = s;
    }
    h->follow_legacy = stream == nullptr;
    return ODO_OK;
}

int odo_set_mode(odo_t *h, int mode) {
    if (!h || mode < ODO_MODE_GRAPH || mode > ODO_MODE_PERSISTENT) return ODO_ERR_ARG;
    if (mode != h->mode) drop_graphs(h);
    h->mode = mode;
    return ODO_OK;
}

int odo_set_precision(odo_t *h, int precision) {
    if (!h || (precision != ODO_PREC_FP32 && precision != ODO_PREC_COMPENSATED)) return ODO_ERR_ARG;
    if (precision != h->precision) drop_graphs(h);
    h->precision = precision;
    return ODO_OK;
}

// Level-0 depth in depth_tmp[0] (copied or filtered there): the pyramid and
// the vertex / normal maps of every level (src/odom/RGBDOdometryef.cpp:131-139).
static int icp_depth_from_level0(odo_t *h, float depthCutoff) {
    cudaStream_t s = h->stream;
    for (int l = 1; l < kLevels; ++l)
        CK(launch_pyr_down_depth(h->depth_tmp[l - 1].cimg(), h->depth_tmp[l].img(), s));
    Img<const uint16_t> d[kLevels];
    Map3 v[kLevels], n[kLevels];
    Intr K[kLevels];
    for (int l = 0; l < kLevels; ++l) {
        d[l] = h->depth_tmp[l].cimg();
        v[l] = h->vmap_curr[l].map();
        n[l] = h->nmap_curr[l].map();
        K[l] = h->intr(l);
    }
    CK(launch_vmap_nmap(d, v, n, K, depthCutoff, kLevels, s));
    return ODO_OK;
}

int odo_init_icp_depth(odo_t *h, const uint16_t *depth, size_t pitch_bytes, float depthCutoff) {
    if (!h || !depth || pitch_bytes < (size_t)h->width * 2) return ODO_ERR_ARG;
    CK(follow_caller(h));
    CK(cudaMemcpy2DAsync(h->depth_tmp[0].data, h->depth_tmp[0].pitch, depth, pitch_bytes, (size_t)h->width * 2,
                         h->height, cudaMemcpyDeviceToDevice, h->stream));
    return icp_depth_from_level0(h, depthCutoff);
}

int odo_init_icp_raw_depth(odo_t *h, const uint16_t *raw_depth, size_t pitch_bytes, float maxD, float depthCutoff) {
    if (!h || !raw_depth || pitch_bytes < (size_t)h->width * 2 || (pitch_bytes % 2) || ((uintptr_t)raw_depth % 2) ||
        !(maxD == maxD))
        return ODO_ERR_ARG;
    CK(follow_caller(h));
    CK(launch_depth_bilateral(raw_depth, pitch_bytes, h->depth_tmp[0].data, h->depth_tmp[0].pitch, h->width,
                              h->height, maxD, h->stream));
    return icp_depth_from_level0(h, depthCutoff);
}

static int init_maps(odo_t *h, const float *verts, const float *norms, size_t pitch_bytes, const float *pose,
                     bool model) {
    if (!h || !verts || !norms || pitch_bytes < (size_t)h->width * 16 || (pitch_bytes % 16) != 0 ||
        ((uintptr_t)verts % 16) != 0 || ((uintptr_t)norms % 16) != 0)
        return ODO_ERR_ARG;
    CK(follow_caller(h));
    Map3 v[kLevels], n[kLevels];
    for (int l = 0; l < kLevels; ++l) {
        v[l] = model ? h->vmap_prev[l].map() : h->vmap_curr[l].map();
        n[l] = model ? h->nmap_prev[l].map() : h->nmap_curr[l].map();
    }
    float R[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1}, t[3] = {0, 0, 0};
    if (pose) {
        const float Rp[9] = {pose[0], pose[1], pose[2], pose[4], pose[5], pose[6], pose[8], pose[9], pose[10]};
        std::memcpy(R, Rp, sizeof(R));
        t[0] = pose[3];
        t[1] = pose[7];
        t[2] = pose[11];
    }
    CK(launch_model_maps(verts, norms, pitch_bytes, h->width, h->height, v, n, kLevels, model ? 1 : 0, R, t,
                         h->vz.data, h->vz.pitch, h->stream));
    return ODO_OK;
}

int odo_init_icp_maps(odo_t *h, const float *verts, const float *norms, size_t pitch_bytes, float depthCutoff) {
    (void)depthCutoff;  // unused by the reference too (src/odom/RGBDOdometryef.cpp:144-167)
    return init_maps(h, verts, norms, pitch_bytes, nullptr, false);
}

int odo_init_icp_model(odo_t *h, const float *verts, const float *norms, size_t pitch_bytes, float depthCutoff,
                       const float pose[16]) {
    (void)depthCutoff;
    if (!pose) return ODO_ERR_ARG;
    return init_maps(h, verts, norms, pitch_bytes, pose, true);
}

// populateRGBDData, src/odom/RGBDOdometryef.cpp:208-235
static int populate(odo_t *h, const uint8_t *rgba, size_t pitch_bytes, DImg<float> *depths, DImg<uint8_t> *images) {
    if (!h || !rgba || pitch_bytes < (size_t)h->width * 4 || (pitch_bytes % 4) != 0 || ((uintptr_t)rgba % 4) != 0)
        return ODO_ERR_ARG;
    cudaStream_t s = h->stream;
    const int do_depth = depths != nullptr;
    CK(launch_rgbd_level0(h->vz.data, h->vz.pitch, rgba, pitch_bytes, h->width, h->height,
                          do_depth ? depths[0].img() : Img<float>{nullptr, 0, 0, 0}, images[0].img(), do_depth, s));
    for (int l = 0; l + 1 < kLevels; ++l)
        CK(launch_gauss_down(do_depth ? depths[l].cimg() : Img<const float>{nullptr, 0, 0, 0},
                             do_depth ? depths[l + 1].img() : Img<float>{nullptr, 0, 0, 0}, images[l].cimg(),
                             images[l + 1].img(), do_depth, s));
    return ODO_OK;
}

int odo_init_rgb(odo_t *h, const uint8_t *rgba, size_t pitch_bytes) {
    if (!h) return ODO_ERR_ARG;
    CK(follow_caller(h));
    return populate(h, rgba, pitch_bytes, h->nextDepth, h->nextImage());
}

int odo_init_rgb_model(odo_t *h, const uint8_t *rgba, size_t pitch_bytes) {
    if (!h) return ODO_ERR_ARG;
    CK(follow_caller(h));
    return populate(h, rgba, pitch_bytes, h->lastDepth, h->lastImage);
}

int odo_init_first_rgb(odo_t *h, const uint8_t *rgba, size_t pitch_bytes) {
    if (!h) return ODO_ERR_ARG;
    CK(follow_caller(h));
    return populate(h, rgba, pitch_bytes, nullptr, h->lastNextImage());
}

int odo_get_incremental_transformation(odo_t *h, float trans[3], float rot[9], int rgbOnly, float icpWeight,
                                       int pyramid, int fastOdom, int so3) {
    if (!h || !trans || !rot) return ODO_ERR_ARG;
    CK(follow_caller(h));
    const int icp = !rgbOnly && icpWeight > 0;
    const int rgb = rgbOnly || icpWeight < 100;
    // src/odom/RGBDOdometryef.cpp:382-384
    const int iterations[kLevels] = {fastOdom ? 3 : 10, pyramid ? 5 : 0, pyramid ? 4 : 0};
    TrackState *st = h->st_host;
    std::memcpy(st->Rprev, rot, sizeof(float) * 9);
    std::memcpy(st->tprev, trans, sizeof(float) * 3);
    st->icpWeight = icpWeight;
    st->rgbOnly = rgbOnly ? 1 : 0;
    st->icp = icp;
    st->rgb = rgb;
    st->so3 = so3 ? 1 : 0;
    st->status = 0;
    for (int l = 0; l < kLevels; ++l) {
        const Intr K = level_args(h, l).K;
        st->Kl[l][0] = K.fx;
        st->Kl[l][1] = K.fy;
        st->Kl[l][2] = K.cx;
        st->Kl[l][3] = K.cy;
        st->sched[l] = iterations[l];
    }
    if (h->mode == ODO_MODE_GRAPH) {
        GraphKey key{icp, rgb, so3 ? 1 : 0, iterations[0], iterations[1], iterations[2], h->parity, h->precision};
        auto it = h->graphs.find(key);
        if (it == h->graphs.end()) {
            cudaGraph_t g = nullptr;
            CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
            cudaError_t e = enqueue_track(h, iterations, icp, rgb, so3 ? 1 : 0);
            cudaError_t e2 = cudaStreamEndCapture(h->stream, &g);
            if (e != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                return fail(h, e, "enqueue_track (capture)");
            }
            if (e2 != cudaSuccess) return fail(h, e2, "cudaStreamEndCapture");
            cudaGraphExec_t ex = nullptr;
            e = cudaGraphInstantiate(&ex, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) return fail(h, e, "cudaGraphInstantiate");
            it = h->graphs.emplace(key, ex).first;
        }
        CK(cudaGraphLaunch(it->second, h->stream));
    } else {
        cudaError_t e = enqueue_track(h, iterations, icp, rgb, so3 ? 1 : 0);
        if (e != cudaSuccess) return fail(h, e, "enqueue_track");
    }
    CK(cudaStreamSynchronize(h->stream));
    if (st->status != 0) {
        h->last_error = "a bounded device-side wait gave up";
        return st->status;
    }
    std::memcpy(trans, st->out_t, sizeof(float) * 3);
    std::memcpy(rot, st->out_R, sizeof(float) * 9);
    if (so3) h->parity ^= 1;  // std::swap(lastNextImage, nextImage), src/odom/RGBDOdometryef.cpp:585-591
    return ODO_OK;
}

int odo_get_covariance(odo_t *h, double out[36]) {
    if (!h || !out) return ODO_ERR_ARG;
    se3::inverse6(h->st_host->lastA, out);
    return ODO_OK;
}

int odo_get_stats(odo_t *h, odo_stats *out) {
    if (!h || !out) return ODO_ERR_ARG;
    const TrackState *st = h->st_host;
    out->lastICPError = st->lastICPError;
    out->lastICPCount = st->lastICPCount;
    out->lastRGBError = st->lastRGBError;
    out->lastRGBCount = st->lastRGBCount;
    out->lastSO3Error = st->lastSO3Error;
    out->lastSO3Count = st->lastSO3Count;
    std::memcpy(out->lastA, st->lastA, sizeof(out->lastA));
    std::memcpy(out->lastb, st->lastb, sizeof(out->lastb));
    return ODO_OK;
}

int odo_get_iterations(odo_t *h, int out[4]) {
    if (!h || !out) return ODO_ERR_ARG;
    out[0] = h->st_host->so3_iters;
    for (int l = 0; l < kLevels; ++l) out[1 + l] = h->st_host->iters_run[l];
    return ODO_OK;
}

size_t odo_state_bytes(void) { return sizeof(TrackState); }

const char *odo_last_error(odo_t *h) { return h ? h->last_error.c_str() : ""; }

const char *odo_status_string(int status) {
    switch (status) {
        case ODO_OK: return "ok";
        case ODO_ERR_ARG: return "invalid argument";
        case ODO_ERR_CUDA: return "CUDA error";
        case ODO_ERR_STATE: return "call-order violation";
        case ODO_ERR_OOM: return "out of device memory";
        case ODO_ERR_TIMEOUT: return "device-side wait timed out";
        case ODO_ERR_SIZE: return "image exceeds ODO_NOALLOC_MAX_PIXELS of the allocation-free entry point";
    }
    return "unknown status";
}

int odo_debug_download(odo_t *h, int which, int level, void *host_dst, size_t bytes) {
    return copy_level(h, which, level, host_dst, bytes, false);
}

int odo_debug_upload(odo_t *h, int which, int level, const void *host_src, size_t bytes) {
    return copy_level(h, which, level, const_cast<void *>(host_src), bytes, true);
}

int odo_debug_icp_step(odo_t *h, int level, const float Rcurr[9], const float tcurr[3], const float Rprev_inv[9],
                       const float tprev[3], int32_t *assoc, double out29[29]) {
    if (!h || level < 0 || level >= kLevels || !Rcurr || !tcurr || !Rprev_inv || !tprev || !out29) return ODO_ERR_ARG;
    LevelArgs L = level_args(h, level);
    int32_t *assoc_dev = nullptr;
    const size_t n = (size_t)L.cols * L.rows;
    if (assoc) CK(cudaMalloc(&assoc_dev, n * sizeof(int32_t)));
    cudaError_t e = launch_debug_icp(L, Rcurr, tcurr, Rprev_inv, tprev, assoc_dev, h->dbg_dev, h->ws, h->cfg[level],
                                     h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out29, h->dbg_dev, 29 * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess && assoc)
        e = cudaMemcpyAsync(assoc, assoc_dev, n * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (assoc_dev) cudaFree(assoc_dev);
    if (e != cudaSuccess) return fail(h, e, "odo_debug_icp_step");
    return ODO_OK;
}

int odo_debug_icp_sums(odo_t *h, int level, const float Rcurr[9], const float tcurr[3], const float Rprev_inv[9],
                       const float tprev[3], double out29[29]) {
    if (!h || level < 0 || level >= kLevels || !Rcurr || !tcurr || !Rprev_inv || !tprev || !out29) return ODO_ERR_ARG;
    LevelArgs L = level_args(h, level);
    TrackLaunch c = h->cfg[level];
    c.precision = h->precision;
    CK(launch_debug_icp_sums(L, Rcurr, tcurr, Rprev_inv, tprev, h->dbg_dev, h->ws, c, h->stream));
    CK(cudaMemcpyAsync(out29, h->dbg_dev, 29 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return ODO_OK;
}

int odo_debug_rgb_sums(odo_t *h, int level, float sigma, double out29[29]) {
    if (!h || level < 0 || level >= kLevels || !out29) return ODO_ERR_ARG;
    LevelArgs L = level_args(h, level);
    TrackLaunch c = h->cfg[level];
    c.precision = h->precision;
    CK(launch_debug_rgb_sums(L, sigma, h->dbg_dev, h->ws, c, h->stream));
    CK(cudaMemcpyAsync(out29, h->dbg_dev, 29 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return ODO_OK;
}

int odo_debug_rgb_residual(odo_t *h, int level, const float krkinv[9], const float kt[3], int32_t out2[2]) {
    if (!h || level < 0 || level >= kLevels || !krkinv || !kt || !out2) return ODO_ERR_ARG;
    LevelArgs L = level_args(h, level);
    CK(launch_debug_rgb_residual(L, krkinv, kt, (int *)h->dbg_dev, h->ws, h->cfg[level], h->stream));
    double o[2];
    CK(cudaMemcpyAsync(o, h->dbg_dev, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    out2[0] = (int32_t)o[0];
    out2[1] = (int32_t)o[1];
    return ODO_OK;
}

int odo_debug_rgb_step(odo_t *h, int level, float sigma, double out29[29]) {
    if (!h || level < 0 || level >= kLevels || !out29) return ODO_ERR_ARG;
    LevelArgs L = level_args(h, level);
    CK(launch_debug_rgb_step(L, sigma, h->dbg_dev, h->ws, h->cfg[level], h->stream));
    CK(cudaMemcpyAsync(out29, h->dbg_dev, 29 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return ODO_OK;
}

int odo_debug_so3_step(odo_t *h, const float homography[9], const float kinv[9], const float krlr[9],
                       double out11[11]) {
    if (!h || !homography || !kinv || !krlr || !out11) return ODO_ERR_ARG;
    float p[27];
    std::memcpy(p, homography, 36);
    std::memcpy(p + 9, kinv, 36);
    std::memcpy(p + 18, krlr, 36);
    CK(cudaMemcpyAsync(h->dbg_params, p, sizeof(p), cudaMemcpyHostToDevice, h->stream));
    CK(launch_debug_so3(h->lastNextImage()[2].cimg(), h->nextImage()[2].cimg(), h->dbg_params, h->dbg_dev, h->stream));
    CK(cudaMemcpyAsync(out11, h->dbg_dev, 11 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return ODO_OK;
}

int odo_debug_derivatives(odo_t *h) {
    if (!h) return ODO_ERR_ARG;
    CK(enqueue_derivatives(h, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return ODO_OK;
}

int odo_debug_history(odo_t *h, double *out, int max_rows) {
    if (!h || !out || max_rows < 0) return ODO_ERR_ARG;
    int n = h->st_host->nhist < max_rows ? h->st_host->nhist : max_rows;
    for (int r = 0; r < n; ++r)
        for (int k = 0; k < 9; ++k) out[r * 9 + k] = h->st_host->hist[r][k];
    return n;
}

int odo_debug_set_wait_limit(odo_t *h, long long polls, int absent_block) {
    if (!h || polls < 1 || absent_block < -1) return ODO_ERR_ARG;
    h->spin_limit = polls;
    h->absent_block = absent_block;
    return ODO_OK;
}

int odo_debug_profile(odo_t *h, double out[8], int reset) {
    if (!h || !out) return ODO_ERR_ARG;
    for (int k = 0; k < 8; ++k) out[k] = h->st_host->prof[k];
    if (reset)
        for (int k = 0; k < 8; ++k) h->st_host->prof[k] = 0;
    return ODO_OK;
}

int odo_debug_time_iteration(odo_t *h, int level, int reps, float out_ms[3]) {
    if (!h || level < 0 || level >= kLevels || reps < 1 || !out_ms) return ODO_ERR_ARG;
    LevelArgs L = level_args(h, level);
    TrackLaunch c = h->cfg[level];
    c.precision = h->precision;
    cudaStream_t s = h->stream;
    TrackState saved = *h->st_host;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    cudaError_t e = cudaSuccess;
    float ms[3] = {0, 0, 0};
    for (int part = 0; part < 3 && e == cudaSuccess; ++part) {
        // restore the state of the last tracking call so every rep does the same work
        e = cudaMemcpyAsync(h->st_dev, h->st_host, sizeof(TrackState), cudaMemcpyHostToDevice, s);
        // one untimed warm-up
        if (e == cudaSuccess) e = launch_level_iteration(L, h->st_dev, h->ws, c, 1, s);
        if (e == cudaSuccess) e = cudaEventRecord(e0, s);
        for (int r = 0; r < reps && e == cudaSuccess; ++r) {
            if (part == 2) e = launch_level_iteration(L, h->st_dev, h->ws, c, 1, s);
            else e = launch_iteration_part(L, h->st_dev, h->ws, c, 1, part, s);
        }
        if (e == cudaSuccess) e = cudaEventRecord(e1, s);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms[part], e0, e1);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(h->st_dev, h->st_host, sizeof(TrackState), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *h->st_host = saved;
    if (e != cudaSuccess) return fail(h, e, "odo_debug_time_iteration");
    for (int k = 0; k < 3; ++k) out_ms[k] = ms[k] / reps;
    return ODO_OK;
}

}  // extern "C"
