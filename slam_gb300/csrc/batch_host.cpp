// Batched tracking: many independent frame pairs (e.g. loop-closure
// candidate verification, src/lc/Ferns.cpp:237-279, or model-to-model checks,
// src/apps/elastic_fusion_file.cpp:450-498) of uneven resolutions tracked in
// one CUDA graph.  Every stage of a single-pair call runs as one batched launch
// over all pairs (the pair is a grid coordinate), so the per-pixel arithmetic,
// the reductions and the per-iteration solve are exactly the single-pair
// path's; with the default launch shape each pair's result is bit-identical to
// odo_get_incremental_transformation on the same inputs.  An autotuner picks
// the block size and pixels per thread of the two iteration kernels.
#include <cuda_runtime.h>

#include <chrono>
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

// The warm-start network's proposals enqueued on stream `st` instead of the
// network's own (cnn_host.cpp); the batch runs them beside its preprocessing.
extern "C" int cnn_propose_on(odo_cnn_t *n, const odo_pair *pairs, int npairs, float *out_dev, cudaStream_t st);

using namespace slamgb;

namespace {

inline size_t round_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

struct PairBufs {
    int w = 0, h = 0;
    int dims_w[kLevels], dims_h[kLevels];
    size_t off = 0;  // offset of this pair's storage in the pixel arena
    // device pointers (carved from the arena)
    Img<uint16_t> depth[kLevels];
    Map3 vc[kLevels], nc[kLevels], vp[kLevels], np[kLevels];
    Img<float> dep[kLevels];  // photometric depth (last, and next for depth input: both from the model vertices)
    Img<float> depn[kLevels]; // next photometric depth for live maps input (from the live vertices)
    Img<uint8_t> last[kLevels], next[kLevels], lastnext[kLevels];
    Img<int16_t> dx[kLevels], dy[kLevels];
    Img<Corr> corr[kLevels];
    Img<uint8_t> cand[kLevels];
    ReduceWs ws;
};

using Layout = std::vector<std::tuple<int, int>>;
using GKey = std::tuple<int, int, int, int, int, int, int, int, int, int, int>;

}  // namespace

struct odo_batch {
    int max_pairs = 0;
    int device = 0, sm_count = 0;
    cudaStream_t own_stream = nullptr, stream = nullptr;
    // pixel arena (per-pair buffers) and argument arena
    void *arena = nullptr;
    size_t arena_bytes = 0;
    Layout layout;
    std::vector<PairBufs> bufs;
    std::vector<int> slot;  // pair i of the current call uses bufs[slot[i]]
    unsigned char *args_dev = nullptr, *args_host = nullptr;  // host pinned
    size_t args_bytes = 0;
    TrackState *st_dev = nullptr, *st_host = nullptr;           // host pinned
    // offsets of the argument blocks in the argument arena
    size_t o_model, o_live, o_rgbd[3], o_gauss[3][2], o_pyr[2], o_vn, o_deriv, o_so3, o_pass[kLevels];
    int threads = 256, ppt = 2;
    // 1: the last iteration stage is the photometric pass plus a
    // one-block-per-pair solve kernel (the pass then carries no FP64 solve
    // code and its registers); 0: the single-pair layout (the solve in the
    // last block of the photometric pass).  Both give the same poses.
    int split_solve = 1;
    int max_nb[kLevels];
    int max_w = 0, max_h = 0;
    float *init_dev = nullptr;  // [max_pairs][6] warm-start motions (odo_batch_track_init)
    float *prop_host = nullptr; // pinned copy of the network's proposals (fall-back decisions)
    int last_n = 0, last_rgb = 0;  // pair count and photometric flag of the last tracking call
    bool follow_legacy = true;     // stream NULL: order after the legacy default stream's work
    cudaEvent_t order_ev = nullptr;
    // warm start: the network's proposals run on side_stream beside the
    // preprocessing; warm_ev marks their end and the tracking graph waits on
    // it right before seeding the pairs (an external-event wait node)
    cudaStream_t side_stream = nullptr;
    cudaEvent_t fork_ev = nullptr, warm_ev = nullptr;
    std::map<GKey, cudaGraphExec_t> graphs;
    std::string last_error;
};

namespace {

int bfail(odo_batch_t *b, cudaError_t e, const char *what) {
    if (b) {
        char buf[256];
        std::snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
        b->last_error = buf;
    }
    return e == cudaErrorMemoryAllocation ? ODO_ERR_OOM : ODO_ERR_CUDA;
}

#define BCK(call)                                          \
    do {                                                   \
        cudaError_t e_ = (call);                           \
        if (e_ != cudaSuccess) return bfail(b, e_, #call); \
    } while (0)

void drop_graphs(odo_batch_t *b) {
    for (auto &kv : b->graphs) cudaGraphExecDestroy(kv.second);
    b->graphs.clear();
}

template <typename T>
Img<T> carve_img(unsigned char *base, size_t &off, int cols, int rows) {
    Img<T> im;
    im.cols = cols;
    im.rows = rows;
    im.pitch = round_up((size_t)cols * sizeof(T), 256);
    im.data = (T *)(base + off);
    off += im.pitch * rows;
    return im;
}
Map3 carve_map(unsigned char *base, size_t &off, int cols, int rows) {
    Map3 m;
    m.cols = cols;
    m.rows = rows;
    m.pitch = round_up((size_t)cols * sizeof(float), 256);
    m.data = (float *)(base + off);
    off += m.pitch * rows * 3;
    return m;
}

int blocks_for(const odo_batch_t *b, int n) {
    int per = b->threads * b->ppt;
    int nb = (n + per - 1) / per;
    if (nb > 2 * b->sm_count) nb = 2 * b->sm_count;
    return nb < 1 ? 1 : nb;
}

// (Re)builds the per-pair buffers for a new list of image sizes.
int ensure_layout(odo_batch_t *b, const odo_pair *pairs, int n) {
    Layout lay;
    for (int i = 0; i < n; ++i) lay.emplace_back(pairs[i].width, pairs[i].height);
    b->slot.resize(n);
    if (lay == b->layout && b->arena) {
        for (int i = 0; i < n; ++i) b->slot[i] = i;
        return ODO_OK;
    }
    // a call with fewer pairs reuses free slots of the same size (no new arena)
    if (b->arena && n < (int)b->layout.size()) {
        std::vector<char> used(b->layout.size(), 0);
        bool ok = true;
        for (int i = 0; i < n && ok; ++i) {
            int s = -1;
            for (size_t j = 0; j < b->layout.size(); ++j)
                if (!used[j] && b->layout[j] == lay[i]) {
                    s = (int)j;
                    break;
                }
            if (s < 0) ok = false;
            else {
                used[s] = 1;
                b->slot[i] = s;
            }
        }
        if (ok) return ODO_OK;
    }
    for (int i = 0; i < n; ++i) b->slot[i] = i;
    BCK(cudaStreamSynchronize(b->stream));
    drop_graphs(b);
    if (b->arena) cudaFree(b->arena);
    b->arena = nullptr;
    b->bufs.assign(n, PairBufs());
    // pass 1: sizes
    size_t total = 0;
    const int maxb = 2 * b->sm_count;
    b->max_w = b->max_h = 0;
    for (int i = 0; i < n; ++i) {
        PairBufs &p = b->bufs[i];
        p.w = pairs[i].width;
        p.h = pairs[i].height;
        if (p.w > b->max_w) b->max_w = p.w;
        if (p.h > b->max_h) b->max_h = p.h;
        p.off = total;
        size_t off = 0;
        unsigned char *nul = nullptr;
        for (int l = 0; l < kLevels; ++l) {
            int w = p.w >> l, h = p.h >> l;
            p.dims_w[l] = w;
            p.dims_h[l] = h;
            carve_img<uint16_t>(nul, off, w, h);
            for (int k = 0; k < 4; ++k) carve_map(nul, off, w, h);
            carve_img<float>(nul, off, w, h);
            for (int k = 0; k < 3; ++k) carve_img<uint8_t>(nul, off, w, h);
            carve_img<int16_t>(nul, off, w, h);
            carve_img<int16_t>(nul, off, w, h);
            carve_img<Corr>(nul, off, w, h);
            carve_img<uint8_t>(nul, off, w, h);
            carve_img<float>(nul, off, w, h);
        }
        carve_img<float>(nul, off, p.w, p.h);
        carve_img<float>(nul, off, p.w, p.h);
        off = round_up(off, 256) + round_up(sizeof(float) * 32 * maxb, 256) * 2 +
              round_up(sizeof(int) * 2 * maxb, 256) + 256;
        total += round_up(off, 256);
    }
    cudaError_t e = cudaMalloc(&b->arena, total ? total : 256);
    if (e != cudaSuccess) return bfail(b, e, "cudaMalloc(batch arena)");
    b->arena_bytes = total;
    BCK(cudaMemset(b->arena, 0, total ? total : 256));
    // pass 2: carve
    for (int i = 0; i < n; ++i) {
        PairBufs &p = b->bufs[i];
        unsigned char *base = (unsigned char *)b->arena + p.off;
        size_t off = 0;
        for (int l = 0; l < kLevels; ++l) {
            int w = p.dims_w[l], h = p.dims_h[l];
            p.depth[l] = carve_img<uint16_t>(base, off, w, h);
            p.vc[l] = carve_map(base, off, w, h);
            p.nc[l] = carve_map(base, off, w, h);
            p.vp[l] = carve_map(base, off, w, h);
            p.np[l] = carve_map(base, off, w, h);
            p.dep[l] = carve_img<float>(base, off, w, h);
            p.last[l] = carve_img<uint8_t>(base, off, w, h);
            p.next[l] = carve_img<uint8_t>(base, off, w, h);
            p.lastnext[l] = carve_img<uint8_t>(base, off, w, h);
            p.dx[l] = carve_img<int16_t>(base, off, w, h);
            p.dy[l] = carve_img<int16_t>(base, off, w, h);
            p.corr[l] = carve_img<Corr>(base, off, w, h);
            p.cand[l] = carve_img<uint8_t>(base, off, w, h);
            p.depn[l] = carve_img<float>(base, off, w, h);
        }
        off = round_up(off, 256);
        p.ws.icp_part = (float *)(base + off);
        off += round_up(sizeof(float) * 32 * maxb, 256);
        p.ws.rgb_part = (float *)(base + off);
        off += round_up(sizeof(float) * 32 * maxb, 256);
        p.ws.res_part = (int *)(base + off);
        off += round_up(sizeof(int) * 2 * maxb, 256);
        p.ws.counters = (unsigned *)(base + off);
        p.ws.max_blocks = maxb;
    }
    b->layout = lay;
    return ODO_OK;
}

// Writes every per-pair argument block into the pinned argument arena.
void build_args(odo_batch_t *b, const odo_pair *pairs, int n, int rgbOnly, float icpWeight, int fastOdom, int so3,
                int live_maps) {
    unsigned char *H = b->args_host;
    auto at = [&](size_t o) { return H + o; };
    const int icp = !rgbOnly && icpWeight > 0;
    const int rgb = rgbOnly || icpWeight < 100;
    for (int i = 0; i < kLevels; ++i) b->max_nb[i] = 1;
    for (int i = 0; i < n; ++i) {
        const odo_pair &q = pairs[i];
        PairBufs &p = b->bufs[b->slot[i]];
        const Intr K0{q.fx, q.fy, q.cx, q.cy};
        auto intr = [&](int l) {
            int div = 1 << l;
            return Intr{K0.fx / div, K0.fy / div, K0.cx / div, K0.cy / div};
        };
        // model maps (initICPModel): planar pyramid + transform by the model pose
        ModelArgs m{};
        m.v4 = q.model_verts;
        m.n4 = q.model_norms;
        m.pitch4 = q.model_pitch;
        m.cols0 = p.w;
        m.rows0 = p.h;
        for (int l = 0; l < kLevels; ++l) {
            m.vmap[l] = p.vp[l];
            m.nmap[l] = p.np[l];
        }
        m.do_transform = 1;
        const float Rp[9] = {q.pose[0], q.pose[1], q.pose[2], q.pose[4], q.pose[5], q.pose[6], q.pose[8], q.pose[9],
                             q.pose[10]};
        for (int k = 0; k < 9; ++k) m.R[k] = Rp[k];
        m.t[0] = q.pose[3];
        m.t[1] = q.pose[7];
        m.t[2] = q.pose[11];
        m.vz = p.dep[0].data;  // the model's level-0 photometric depth, written by the import
        m.vz_pitch = p.dep[0].pitch;
        std::memcpy(at(b->o_model) + i * sizeof(ModelArgs), &m, sizeof(m));
        // live maps (initICP(verts, norms)): planar pyramid, no transform,
        // raw vertex z for the live photometric depth
        if (live_maps) {
            ModelArgs lm{};
            lm.v4 = q.live_verts;
            lm.n4 = q.live_norms;
            lm.pitch4 = q.live_pitch;
            lm.cols0 = p.w;
            lm.rows0 = p.h;
            for (int l = 0; l < kLevels; ++l) {
                lm.vmap[l] = p.vc[l];
                lm.nmap[l] = p.nc[l];
            }
            lm.do_transform = 0;
            lm.vz = p.depn[0].data;
            lm.vz_pitch = p.depn[0].pitch;
            std::memcpy(at(b->o_live) + i * sizeof(ModelArgs), &lm, sizeof(lm));
        }
        // photometric depth of the live frame: the model's (depth input, the
        // reference's quirk) or the live maps' own
        Img<float> *depn = live_maps ? p.depn : p.dep;
        // photometric level 0: model image + depth from the model vertices,
        // live image, previous live image (SO3)
        const uint8_t *src[3] = {q.model_rgba, q.rgba, q.prev_rgba ? q.prev_rgba : q.rgba};
        const size_t sp[3] = {q.model_rgba_pitch, q.rgba_pitch, q.prev_rgba ? q.prev_rgba_pitch : q.rgba_pitch};
        Img<uint8_t> *imgs[3] = {p.last, p.next, p.lastnext};
        for (int r = 0; r < 3; ++r) {
            // depth rows: the model's (role 0) and, for live maps, the live one
            // (role 1); their level 0 is written by the map import
            const int with_depth = r == 0 || (r == 1 && live_maps);
            Img<float> *dp = r == 1 ? depn : p.dep;
            RgbdArgs a{nullptr, 0, src[r], sp[r], dp[0], imgs[r][0], 0};
            std::memcpy(at(b->o_rgbd[r]) + i * sizeof(RgbdArgs), &a, sizeof(a));
            for (int l = 0; l < 2; ++l) {
                Img<const float> ds{dp[l].data, dp[l].pitch, dp[l].cols, dp[l].rows};
                Img<const uint8_t> is{imgs[r][l].data, imgs[r][l].pitch, imgs[r][l].cols, imgs[r][l].rows};
                GaussArgs g{ds, dp[l + 1], is, imgs[r][l + 1], with_depth};
                std::memcpy(at(b->o_gauss[r][l]) + i * sizeof(GaussArgs), &g, sizeof(g));
            }
        }
        // depth pyramid (the level-0 input is read in place)
        for (int l = 0; l < 2; ++l) {
            Img<const uint16_t> s0 = l == 0 ? Img<const uint16_t>{q.depth, q.depth_pitch, p.w, p.h}
                                            : Img<const uint16_t>{p.depth[l].data, p.depth[l].pitch, p.depth[l].cols,
                                                                  p.depth[l].rows};
            PyrArgs a{s0, p.depth[l + 1]};
            std::memcpy(at(b->o_pyr[l]) + i * sizeof(PyrArgs), &a, sizeof(a));
        }
        VNArgs v{};
        for (int l = 0; l < kLevels; ++l) {
            v.depth[l] = l == 0 ? Img<const uint16_t>{q.depth, q.depth_pitch, p.w, p.h}
                                : Img<const uint16_t>{p.depth[l].data, p.depth[l].pitch, p.depth[l].cols,
                                                      p.depth[l].rows};
            v.vmap[l] = p.vc[l];
            v.nmap[l] = p.nc[l];
            const Intr K = intr(l);
            v.fx_inv[l] = 1.f / K.fx;
            v.fy_inv[l] = 1.f / K.fy;
            v.cx[l] = K.cx;
            v.cy[l] = K.cy;
        }
        v.cutoff = q.depthCutoff > 0 ? q.depthCutoff : 20.0f;  // maxDepthProcessed (src/configs/ef_file.cfg:16)
        std::memcpy(at(b->o_vn) + i * sizeof(VNArgs), &v, sizeof(v));
        DerivArgs d{};
        const float minGrad[kLevels] = {5, 3, 1};
        const float sobelScale = (float)(1.0 / pow(2.0, 3));
        for (int l = 0; l < kLevels; ++l) {
            d.src[l] = Img<const uint8_t>{p.next[l].data, p.next[l].pitch, p.next[l].cols, p.next[l].rows};
            d.dx[l] = p.dx[l];
            d.dy[l] = p.dy[l];
            d.depth[l] = Img<const float>{depn[l].data, depn[l].pitch, depn[l].cols, depn[l].rows};
            d.cand[l] = p.cand[l];
            d.minScale[l] = (float)(pow(minGrad[l], 2.0) / pow((double)sobelScale, 2.0));
        }
        std::memcpy(at(b->o_deriv) + i * sizeof(DerivArgs), &d, sizeof(d));
        So3Args so{b->st_dev + i,
                   Img<const uint8_t>{p.lastnext[2].data, p.lastnext[2].pitch, p.lastnext[2].cols, p.lastnext[2].rows},
                   Img<const uint8_t>{p.next[2].data, p.next[2].pitch, p.next[2].cols, p.next[2].rows}, intr(2)};
        std::memcpy(at(b->o_so3) + i * sizeof(So3Args), &so, sizeof(so));
        // iteration schedule (src/odom/RGBDOdometryef.cpp:382-384), restricted to `levels`
        const int base[kLevels] = {fastOdom ? 3 : 10, 5, 4};
        int sched[kLevels];
        for (int l = 0; l < kLevels; ++l) {
            PassArgs a{};
            LevelArgs &L = a.L;
            L.level = l;
            L.cols = p.dims_w[l];
            L.rows = p.dims_h[l];
            L.K = intr(l);
            L.vmap_curr = p.vc[l];
            L.nmap_curr = p.nc[l];
            L.vmap_prev = p.vp[l];
            L.nmap_prev = p.np[l];
            L.angleThres = q.angleThresh > 0 ? q.angleThresh : ODO_DEFAULT_ANGLE_THRESH;
            L.distThres = q.distThresh > 0 ? q.distThresh : ODO_DEFAULT_DIST_THRESH;
            L.dIdx = Img<const int16_t>{p.dx[l].data, p.dx[l].pitch, p.dx[l].cols, p.dx[l].rows};
            L.dIdy = Img<const int16_t>{p.dy[l].data, p.dy[l].pitch, p.dy[l].cols, p.dy[l].rows};
            L.lastDepth = Img<const float>{p.dep[l].data, p.dep[l].pitch, p.dep[l].cols, p.dep[l].rows};
            L.nextDepth = Img<const float>{depn[l].data, depn[l].pitch, depn[l].cols, depn[l].rows};
            L.lastImage = Img<const uint8_t>{p.last[l].data, p.last[l].pitch, p.last[l].cols, p.last[l].rows};
            L.nextImage = Img<const uint8_t>{p.next[l].data, p.next[l].pitch, p.next[l].cols, p.next[l].rows};
            L.corr = p.corr[l];
            L.cand = Img<const uint8_t>{p.cand[l].data, p.cand[l].pitch, p.cand[l].cols, p.cand[l].rows};
            L.minScale = d.minScale[l];
            L.maxDepthDelta = 0.07f;
            L.sobelScale = sobelScale;
            a.st = b->st_dev + i;
            a.ws = p.ws;
            a.iters = (l < q.levels) ? (q.iterations[l] > 0 ? q.iterations[l] : base[l]) : 0;
            sched[l] = a.iters;
            const int npx = L.cols * L.rows;
            a.nb_icp = a.iters ? blocks_for(b, npx) : 0;
            a.nb_rgb = a.iters ? (rgb ? a.nb_icp : 1) : 0;
            a.invFx = 1.0f / L.K.fx;
            a.invFy = 1.0f / L.K.fy;
            a.km = make_kmats(L.K);
            if (a.nb_icp > b->max_nb[l]) b->max_nb[l] = a.nb_icp;
            std::memcpy(at(b->o_pass[l]) + i * sizeof(PassArgs), &a, sizeof(a));
        }
        // initial state of the call (src/odom/RGBDOdometryef.cpp:278-282)
        TrackState &st = b->st_host[i];
        std::memset(&st, 0, sizeof(st));
        for (int k = 0; k < 9; ++k) st.Rprev[k] = Rp[k];
        st.tprev[0] = q.pose[3];
        st.tprev[1] = q.pose[7];
        st.tprev[2] = q.pose[11];
        st.icpWeight = icpWeight;
        st.rgbOnly = rgbOnly ? 1 : 0;
        st.icp = icp;
        st.rgb = rgb;
        st.so3 = so3 ? 1 : 0;
        for (int k = 0; k < 9; ++k) st.resultR[k] = (k % 4 == 0) ? 1.0 : 0.0;
        st.lastICPCount = st.lastRGBCount = st.lastSO3Count = (float)(p.w * p.h);
        for (int l = 0; l < kLevels; ++l) {
            const Intr K = intr(l);
            st.Kl[l][0] = K.fx;
            st.Kl[l][1] = K.fy;
            st.Kl[l][2] = K.cx;
            st.Kl[l][3] = K.cy;
            st.sched[l] = sched[l];
        }
    }
}

// prep = false skips the per-frame preprocessing whose results are already in
// the pairs' buffers (a fall-back call right after the warm-started call on
// the same slots) except the extra intensity pyramid the SO3 stage reads.
cudaError_t enqueue_batch(odo_batch_t *b, int n, int rgb, int so3, int warm, const int max_iters[kLevels],
                          bool prep = true, int live_maps = 0) {
    cudaStream_t s = b->stream;
    // argument blocks and states travel by a copy kernel over the pinned
    // host buffers, not queued behind the caller's bulk copies on the copy
    // engines
    cudaError_t e = launch_host_copy(b->args_dev, b->args_host, b->args_bytes, s);
    if (e == cudaSuccess) e = launch_host_copy(b->st_dev, b->st_host, sizeof(TrackState) * n, s);
    auto A = [&](size_t o) { return (const void *)(b->args_dev + o); };
    const int W = b->max_w, Hh = b->max_h;
    if (e == cudaSuccess) e = launch_stamp_batch(b->st_dev, n, s);
    if (e == cudaSuccess && prep) e = launch_model_maps_batch((const ModelArgs *)A(b->o_model), n, W, Hh, s);
    if (e == cudaSuccess && prep && live_maps)
        e = launch_model_maps_batch((const ModelArgs *)A(b->o_live), n, W, Hh, s);
    const int roles = so3 ? 3 : 2, r0 = prep ? 0 : 2;
    for (int r = r0; r < roles && e == cudaSuccess; ++r)
        e = launch_rgbd_level0_batch((const RgbdArgs *)A(b->o_rgbd[r]), n, W, Hh, s);
    for (int l = 0; l < 2 && e == cudaSuccess; ++l)
        for (int r = r0; r < roles && e == cudaSuccess; ++r)
            e = launch_gauss_down_batch((const GaussArgs *)A(b->o_gauss[r][l]), n, W >> (l + 1), Hh >> (l + 1), s);
    for (int l = 0; l < 2 && e == cudaSuccess && prep && !live_maps; ++l)
        e = launch_pyr_down_depth_batch((const PyrArgs *)A(b->o_pyr[l]), n, W >> (l + 1), Hh >> (l + 1), s);
    if (e == cudaSuccess && prep && !live_maps) e = launch_vmap_nmap_batch((const VNArgs *)A(b->o_vn), n, W, Hh, s);
    if (e == cudaSuccess && rgb && prep)
        e = launch_derivatives_batch((const DerivArgs *)A(b->o_deriv), n, W, Hh, s);
    if (e == cudaSuccess && so3) e = launch_so3_batch((const So3Args *)A(b->o_so3), n, s);
    if (e == cudaSuccess) e = launch_track_begin_batch(b->st_dev, n, s);
    if (e == cudaSuccess && warm) e = cudaStreamWaitEvent(s, b->warm_ev, cudaEventWaitExternal);
    if (e == cudaSuccess && warm) e = launch_warm_seed_batch(b->st_dev, b->init_dev, n, s);
    for (int l = kLevels - 1; l >= 0 && e == cudaSuccess; --l)
        for (int j = 0; j < max_iters[l] && e == cudaSuccess; ++j)
            e = launch_level_iteration_batch((const PassArgs *)A(b->o_pass[l]), n, b->max_nb[l],
                                             rgb ? b->max_nb[l] : 1, b->threads, 0, j, s, 3, b->split_solve);
    if (e == cudaSuccess) e = launch_track_end_batch(b->st_dev, n, s);
    if (e == cudaSuccess) e = launch_host_copy(b->st_host, b->st_dev, sizeof(TrackState) * n, s);
    return e;
}

}  // namespace

extern "C" {

int odo_batch_create(int max_pairs, odo_batch_t **out) {
    if (!out || max_pairs < 1 || max_pairs > 65535) return ODO_ERR_ARG;
    *out = nullptr;
    odo_batch_t *b = new (std::nothrow) odo_batch_t();
    if (!b) return ODO_ERR_OOM;
    b->max_pairs = max_pairs;
    auto bail = [&](cudaError_t e, const char *what) {
        int rc = bfail(b, e, what);
        odo_batch_destroy(b);
        return rc;
    };
    cudaError_t e;
    if ((e = cudaGetDevice(&b->device)) != cudaSuccess) return bail(e, "cudaGetDevice");
    if ((e = cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, b->device)) != cudaSuccess)
        return bail(e, "cudaDeviceGetAttribute");
    if ((e = cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking)) != cudaSuccess)
        return bail(e, "cudaStreamCreate");
    b->stream = b->own_stream;
    // argument arena layout
    size_t o = 0;
    auto take = [&](size_t bytes) {
        size_t r = o;
        o = round_up(o + bytes, 256);
        return r;
    };
    const size_t np = (size_t)max_pairs;
    b->o_model = take(np * sizeof(ModelArgs));
    b->o_live = take(np * sizeof(ModelArgs));
    for (int r = 0; r < 3; ++r) b->o_rgbd[r] = take(np * sizeof(RgbdArgs));
    for (int r = 0; r < 3; ++r)
        for (int l = 0; l < 2; ++l) b->o_gauss[r][l] = take(np * sizeof(GaussArgs));
    for (int l = 0; l < 2; ++l) b->o_pyr[l] = take(np * sizeof(PyrArgs));
    b->o_vn = take(np * sizeof(VNArgs));
    b->o_deriv = take(np * sizeof(DerivArgs));
    b->o_so3 = take(np * sizeof(So3Args));
    for (int l = 0; l < kLevels; ++l) b->o_pass[l] = take(np * sizeof(PassArgs));
    b->args_bytes = o;
    if ((e = cudaMalloc(&b->args_dev, o)) != cudaSuccess) return bail(e, "cudaMalloc(args)");
    if ((e = cudaMallocHost(&b->args_host, o)) != cudaSuccess) return bail(e, "cudaMallocHost(args)");
    std::memset(b->args_host, 0, o);
    if ((e = cudaMalloc(&b->st_dev, sizeof(TrackState) * np)) != cudaSuccess) return bail(e, "cudaMalloc(states)");
    if ((e = cudaMalloc(&b->init_dev, sizeof(float) * 6 * np)) != cudaSuccess) return bail(e, "cudaMalloc(init)");
    if ((e = cudaMallocHost(&b->prop_host, sizeof(float) * 6 * np)) != cudaSuccess)
        return bail(e, "cudaMallocHost(proposals)");
    if ((e = cudaEventCreateWithFlags(&b->order_ev, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&b->fork_ev, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&b->warm_ev, cudaEventDisableTiming)) != cudaSuccess)
        return bail(e, "cudaEventCreate");
    if ((e = cudaStreamCreateWithFlags(&b->side_stream, cudaStreamNonBlocking)) != cudaSuccess)
        return bail(e, "cudaStreamCreate(side)");
    if ((e = cudaMallocHost(&b->st_host, sizeof(TrackState) * np)) != cudaSuccess)
        return bail(e, "cudaMallocHost(states)");
    *out = b;
    return ODO_OK;
}

int odo_batch_destroy(odo_batch_t *b) {
    if (!b) return ODO_ERR_ARG;
    if (b->stream) cudaStreamSynchronize(b->stream);
    drop_graphs(b);
    if (b->arena) cudaFree(b->arena);
    if (b->args_dev) cudaFree(b->args_dev);
    if (b->args_host) cudaFreeHost(b->args_host);
    if (b->st_dev) cudaFree(b->st_dev);
    if (b->st_host) cudaFreeHost(b->st_host);
    if (b->init_dev) cudaFree(b->init_dev);
    if (b->prop_host) cudaFreeHost(b->prop_host);
    if (b->order_ev) cudaEventDestroy(b->order_ev);
    if (b->side_stream) {
        cudaStreamSynchronize(b->side_stream);
        cudaStreamDestroy(b->side_stream);
    }
    if (b->fork_ev) cudaEventDestroy(b->fork_ev);
    if (b->warm_ev) cudaEventDestroy(b->warm_ev);
    if (b->own_stream) cudaStreamDestroy(b->own_stream);
    delete b;
    return ODO_OK;
}

int odo_batch_set_stream(odo_batch_t *b, void *stream) {
    if (!b) return ODO_ERR_ARG;
    cudaStream_t s = stream ? (cudaStream_t)stream : b->own_stream;
    if (s != b->stream) {
        BCK(cudaStreamSynchronize(b->stream));
        drop_graphs(b);
        b->stream = s;
    }
    b->follow_legacy = stream == nullptr;
    return ODO_OK;
}

int odo_batch_debug_set_split(odo_batch_t *b, int on) {
    if (!b) return ODO_ERR_ARG;
    if (b->split_solve != (on ? 1 : 0)) drop_graphs(b);
    b->split_solve = on ? 1 : 0;
    return ODO_OK;
}

int odo_batch_set_launch(odo_batch_t *b, int threads, int pixels_per_thread) {
    if (!b || (threads != 128 && threads != 256) || pixels_per_thread < 1 || pixels_per_thread > 64)
        return ODO_ERR_ARG;
    if (threads != b->threads || pixels_per_thread != b->ppt) drop_graphs(b);
    b->threads = threads;
    b->ppt = pixels_per_thread;
    return ODO_OK;
}

}  // extern "C"

namespace {

// graph = false enqueues the kernels directly (for one-off batch sizes, e.g.
// the fall-back subset of a warm-started batch, where instantiating a graph
// would cost more than it saves).  reuse_slots (graph-less calls only): the
// arena slot of every pair, whose buffers already hold this frame pair's
// preprocessing from the previous call; that preprocessing is skipped.
int track_impl(odo_batch_t *b, const odo_pair *pairs, int npairs, const float *init, int rgbOnly, float icpWeight,
               int fastOdom, int so3, odo_pair_result *results, bool graph = true,
               const int *reuse_slots = nullptr) {
    if (!b || !pairs || !results || npairs < 1 || npairs > b->max_pairs) return ODO_ERR_ARG;
    const int live_maps = pairs[0].live_verts != nullptr;
    for (int i = 0; i < npairs; ++i) {
        const odo_pair &q = pairs[i];
        if (q.width < 16 || q.height < 16 || q.width > 8192 || q.height > 8192 || q.levels < 1 || q.levels > 3 ||
            !q.model_verts || !q.model_norms || !q.model_rgba || !q.rgba ||
            q.model_pitch < (size_t)q.width * 16 || q.rgba_pitch < (size_t)q.width * 4 ||
            q.model_rgba_pitch < (size_t)q.width * 4 || !(q.fx != 0) || !(q.fy != 0) ||
            (q.model_pitch % 16) != 0 || ((uintptr_t)q.model_verts % 16) != 0 || ((uintptr_t)q.model_norms % 16) != 0)
            return ODO_ERR_ARG;
        if ((q.live_verts != nullptr) != (live_maps != 0)) return ODO_ERR_ARG;  // one kind of live input per call
        if (live_maps) {
            if (!q.live_norms || q.live_pitch < (size_t)q.width * 16 || (q.live_pitch % 16) != 0 ||
                ((uintptr_t)q.live_verts % 16) != 0 || ((uintptr_t)q.live_norms % 16) != 0)
                return ODO_ERR_ARG;
        } else if (!q.depth || q.depth_pitch < (size_t)q.width * 2) {
            return ODO_ERR_ARG;
        }
        for (int l = 0; l < kLevels; ++l)
            if (q.iterations[l] < 0 || q.iterations[l] > 20) return ODO_ERR_ARG;
    }
    const int warm = init != nullptr;
    if (warm) so3 = 0;
    if (b->follow_legacy) {  // the inputs were produced on the legacy default stream
        BCK(cudaEventRecord(b->order_ev, 0));
        BCK(cudaStreamWaitEvent(b->stream, b->order_ev, 0));
    }
    bool reuse = reuse_slots != nullptr && !graph && b->arena != nullptr;
    for (int i = 0; i < npairs && reuse; ++i) {
        const int s = reuse_slots[i];
        reuse = s >= 0 && s < (int)b->layout.size() && b->layout[s] == std::make_tuple(pairs[i].width, pairs[i].height);
    }
    int rc = ODO_OK;
    if (reuse) b->slot.assign(reuse_slots, reuse_slots + npairs);
    else rc = ensure_layout(b, pairs, npairs);
    if (rc != ODO_OK) return rc;
    const int rgb = rgbOnly || icpWeight < 100;
    build_args(b, pairs, npairs, rgbOnly, icpWeight, fastOdom, so3, live_maps);
    int max_iters[kLevels] = {0, 0, 0};
    const int base[kLevels] = {fastOdom ? 3 : 10, 5, 4};
    for (int i = 0; i < npairs; ++i)
        for (int l = 0; l < pairs[i].levels; ++l) {
            const int it = pairs[i].iterations[l] > 0 ? pairs[i].iterations[l] : base[l];
            if (it > max_iters[l]) max_iters[l] = it;
        }
    if (warm && init != b->init_dev)
        BCK(cudaMemcpyAsync(b->init_dev, init, sizeof(float) * 6 * npairs, cudaMemcpyDeviceToDevice, b->stream));
    if (!graph) {
        BCK(enqueue_batch(b, npairs, rgb, so3 ? 1 : 0, warm, max_iters, !reuse, live_maps));
    } else {
        GKey key{npairs, rgb, so3 ? 1 : 0, warm, max_iters[0], max_iters[1], max_iters[2], b->threads, b->ppt,
                 b->split_solve, live_maps};
        auto it = b->graphs.find(key);
        if (it == b->graphs.end()) {
            cudaGraph_t g = nullptr;
            BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
            cudaError_t e = enqueue_batch(b, npairs, rgb, so3 ? 1 : 0, warm, max_iters, true, live_maps);
            cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
            if (e != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                return bfail(b, e, "enqueue_batch (capture)");
            }
            if (e2 != cudaSuccess) return bfail(b, e2, "cudaStreamEndCapture");
            cudaGraphExec_t ex = nullptr;
            e = cudaGraphInstantiate(&ex, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) return bfail(b, e, "cudaGraphInstantiate");
            it = b->graphs.emplace(key, ex).first;
        }
        BCK(cudaGraphLaunch(it->second, b->stream));
    }
    BCK(cudaStreamSynchronize(b->stream));
    b->last_n = npairs;
    b->last_rgb = rgb;
    for (int i = 0; i < npairs; ++i) {
        const TrackState &st = b->st_host[i];
        if (st.status != 0) return st.status;
        odo_pair_result &r = results[i];
        for (int a = 0; a < 3; ++a) {
            for (int c = 0; c < 3; ++c) r.pose[a * 4 + c] = st.out_R[a * 3 + c];
            r.pose[a * 4 + 3] = st.out_t[a];
        }
        r.pose[12] = r.pose[13] = r.pose[14] = 0.f;
        r.pose[15] = 1.f;
        r.lastICPError = st.lastICPError;
        r.lastICPCount = st.lastICPCount;
        r.lastRGBError = st.lastRGBError;
        r.lastRGBCount = st.lastRGBCount;
        r.lastSO3Error = st.lastSO3Error;
        r.lastSO3Count = st.lastSO3Count;
        r.iterations[0] = st.so3_iters;
        for (int l = 0; l < kLevels; ++l) r.iterations[1 + l] = st.iters_run[l];
        r.done_us = (double)((st.t_solve ? st.t_solve : st.t_end) - st.t_start) * 1e-3;
        std::memcpy(r.lastA, st.lastA, sizeof(r.lastA));
        std::memcpy(r.lastb, st.lastb, sizeof(r.lastb));
    }
    return ODO_OK;
}

}  // namespace

extern "C" {

int odo_batch_track(odo_batch_t *b, const odo_pair *pairs, int npairs, int rgbOnly, float icpWeight, int fastOdom,
                    int so3, odo_pair_result *results) {
    return track_impl(b, pairs, npairs, nullptr, rgbOnly, icpWeight, fastOdom, so3, results);
}

int odo_batch_verify(odo_batch_t *b, const odo_pair *pairs, int npairs, const odo_verify_params *vp,
                     odo_pair_result *results, double *covariance, int *accept) {
    if (!vp || !accept) return ODO_ERR_ARG;
    const int rc = track_impl(b, pairs, npairs, nullptr, vp->rgbOnly, vp->icpWeight, vp->fastOdom, vp->so3, results);
    if (rc != ODO_OK) return rc;
    for (int i = 0; i < npairs; ++i) {
        const odo_pair_result &r = results[i];
        // getCovariance: lastA.cast<double>().lu().inverse() (src/odom/RGBDOdometryef.cpp:597-600)
        double cov[36];
        se3::inverse6(r.lastA, cov);
        if (covariance) std::memcpy(covariance + 36 * (size_t)i, cov, sizeof(cov));
        bool ok = true;
        // src/apps/elastic_fusion_file.cpp:479-488: covar(i, i) > covThresh rejects
        if (vp->max_covariance > 0)
            for (int k = 0; k < 6; ++k) ok = ok && !(cov[k * 7] > vp->max_covariance);
        // src/lc/Ferns.cpp:279, src/apps/elastic_fusion_file.cpp:498
        if (vp->min_icp_count > 0) ok = ok && r.lastICPCount > vp->min_icp_count;
        if (vp->max_icp_error > 0) ok = ok && r.lastICPError < vp->max_icp_error;
        accept[i] = ok ? 1 : 0;
    }
    return ODO_OK;
}

int odo_batch_track_init(odo_batch_t *b, const odo_pair *pairs, int npairs, const float *init_dev, int rgbOnly,
                         float icpWeight, int fastOdom, odo_pair_result *results) {
    if (!init_dev) return ODO_ERR_ARG;
    return track_impl(b, pairs, npairs, init_dev, rgbOnly, icpWeight, fastOdom, 0, results);
}

int odo_batch_track_warm(odo_batch_t *b, odo_cnn_t *net, const odo_pair *pairs, int npairs,
                         const odo_warm_params *wp, odo_pair_result *results, int *fallback) {
    if (!b || !net || !pairs || !wp || !results || npairs < 1 || npairs > b->max_pairs) return ODO_ERR_ARG;
    if (wp->levels < 1 || wp->levels > 3) return ODO_ERR_ARG;
    // 1. proposals straight into the warm-start buffer, on the side stream
    //    (after the work already on the batch stream); the tracking graph's
    //    preprocessing runs beside them and its seeding waits for warm_ev
    if (b->follow_legacy) {
        BCK(cudaEventRecord(b->order_ev, 0));
        BCK(cudaStreamWaitEvent(b->stream, b->order_ev, 0));
    }
    BCK(cudaEventRecord(b->fork_ev, b->stream));
    BCK(cudaStreamWaitEvent(b->side_stream, b->fork_ev, 0));
    int rc = cnn_propose_on(net, pairs, npairs, b->init_dev, b->side_stream);
    if (rc != ODO_OK) return rc;
    BCK(cudaEventRecord(b->warm_ev, b->side_stream));
    // 2. tracking from the proposals with the short schedule
    std::vector<odo_pair> warm(pairs, pairs + npairs);
    for (auto &q : warm) {
        q.levels = wp->levels;
        for (int l = 0; l < kLevels; ++l) q.iterations[l] = wp->iterations[l];
    }
    rc = track_impl(b, warm.data(), npairs, b->init_dev, wp->rgbOnly, wp->icpWeight, wp->fastOdom, 0, results);
    const std::vector<int> warm_slot = b->slot;  // where each pair's preprocessed buffers are
    const int rc2 = odo_cnn_wait(net);
    if (rc != ODO_OK) return rc;
    if (rc2 != ODO_OK) return rc2;
    // 3. fall-back decisions on the host: residual, and the angle between the
    //    refined rotation and the proposed one, R_prop = R_pose exp(w)
    BCK(launch_host_copy(b->prop_host, b->init_dev, sizeof(float) * 6 * npairs, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    const float *prop = b->prop_host;
    std::vector<int> idx;
    for (int i = 0; i < npairs; ++i) {
        bool fb = wp->residual_limit > 0 && !(results[i].lastICPError <= wp->residual_limit);
        if (!fb && wp->max_disagree > 0) {
            double w[3] = {prop[6 * i + 3], prop[6 * i + 4], prop[6 * i + 5]}, Rr[9], Rp[9], Rq[9];
            se3::rodrigues(w, Rr);
            for (int k = 0; k < 9; ++k) Rp[k] = pairs[i].pose[(k / 3) * 4 + k % 3];
            se3::mm33(Rp, Rr, Rq);
            // cos(angle) = (trace(R_res^T R_prop) - 1) / 2
            double tr = 0;
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) tr += (double)results[i].pose[r * 4 + c] * Rq[r * 3 + c];
            const double cs = 0.5 * (tr - 1.0);
            fb = cs < std::cos((double)wp->max_disagree);
        }
        if (fallback) fallback[i] = fb ? 1 : 0;
        if (fb) idx.push_back(i);
    }
    if (idx.empty()) return ODO_OK;
    // 4. the pairs that fell back: plain schedule with the SO3 stage, on the
    //    preprocessing of step 2 (same inputs, same slots) when it covered
    //    every pyramid level these pairs use
    std::vector<odo_pair> sub;
    std::vector<int> sub_slot;
    bool reuse = true;
    for (int i : idx) {
        sub.push_back(pairs[i]);
        sub_slot.push_back(warm_slot[i]);
        reuse = reuse && pairs[i].levels <= wp->levels;
    }
    std::vector<odo_pair_result> sres(idx.size());
    // The launch shape is tuned for whole batches; for a small subset it
    // leaves the level-0 launch below one wave of long-running blocks.  The
    // subset runs with fewer pixels per thread, halved until its level-0
    // launch has at least 8 waves of blocks (3 resident per SM); the shape
    // is restored after the call, so the cached graphs stay valid.
    const int saved_ppt = b->ppt;
    long long px = 0;
    for (const odo_pair &q : sub) px += (long long)q.width * q.height;
    const long long want_blocks = 8ll * 3 * (b->sm_count > 0 ? b->sm_count : 1);
    while (b->ppt > 2 && px / ((long long)b->threads * b->ppt) < want_blocks) b->ppt >>= 1;
    rc = track_impl(b, sub.data(), (int)sub.size(), nullptr, wp->rgbOnly, wp->icpWeight, wp->fastOdom, 1, sres.data(),
                    false, reuse ? sub_slot.data() : nullptr);
    b->ppt = saved_ppt;
    if (rc != ODO_OK) return rc;
    for (size_t k = 0; k < idx.size(); ++k) results[idx[k]] = sres[k];
    return ODO_OK;
}

int odo_batch_debug_time_iteration(odo_batch_t *b, int level, int reps, float out_ms[3]) {
    if (!b || level < 0 || level >= kLevels || reps < 1 || !out_ms || b->last_n < 1) return ODO_ERR_ARG;
    const int n = b->last_n;
    const PassArgs *args = (const PassArgs *)(b->args_dev + b->o_pass[level]);
    cudaStream_t s = b->stream;
    cudaEvent_t e0, e1;
    BCK(cudaEventCreate(&e0));
    BCK(cudaEventCreate(&e1));
    cudaError_t e = cudaSuccess;
    float ms[3] = {0, 0, 0};
    for (int part = 0; part < 3 && e == cudaSuccess; ++part) {
        const int mask = part == 2 ? 3 : part + 1;
        // restore the states of the last call so every repetition does the same work
        e = cudaMemcpyAsync(b->st_dev, b->st_host, sizeof(TrackState) * n, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess)
            e = launch_level_iteration_batch(args, n, b->max_nb[level], b->last_rgb ? b->max_nb[level] : 1, b->threads,
                                             0, 1, s, 3, b->split_solve);
        if (e == cudaSuccess) e = cudaEventRecord(e0, s);
        for (int r = 0; r < reps && e == cudaSuccess; ++r)
            e = launch_level_iteration_batch(args, n, b->max_nb[level], b->last_rgb ? b->max_nb[level] : 1, b->threads,
                                             0, 1, s, mask, b->split_solve);
        if (e == cudaSuccess) e = cudaEventRecord(e1, s);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms[part], e0, e1);
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->st_dev, b->st_host, sizeof(TrackState) * n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return bfail(b, e, "odo_batch_debug_time_iteration");
    for (int k = 0; k < 3; ++k) out_ms[k] = ms[k] / reps;
    return ODO_OK;
}

int odo_batch_autotune(odo_batch_t *b, const odo_pair *pairs, int npairs, int rgbOnly, float icpWeight, int fastOdom,
                       int so3, odo_pair_result *scratch_results, int *threads, int *pixels_per_thread,
                       float *best_ms) {
    if (!b || !threads || !pixels_per_thread) return ODO_ERR_ARG;
    const int cand_t[2] = {128, 256};
    const int cand_p[6] = {2, 4, 8, 16, 32, 64};
    float best = 1e30f;
    int bt = b->threads, bp = b->ppt;
    cudaEvent_t e0, e1;
    BCK(cudaEventCreate(&e0));
    BCK(cudaEventCreate(&e1));
    for (int ti = 0; ti < 2; ++ti)
        for (int pi = 0; pi < 6; ++pi) {
            int rc = odo_batch_set_launch(b, cand_t[ti], cand_p[pi]);
            if (rc == ODO_OK) rc = odo_batch_track(b, pairs, npairs, rgbOnly, icpWeight, fastOdom, so3, scratch_results);
            if (rc != ODO_OK) {
                cudaEventDestroy(e0);
                cudaEventDestroy(e1);
                return rc;
            }
            float ms = 0;
            BCK(cudaEventRecord(e0, b->stream));
            for (int r = 0; r < 2 && rc == ODO_OK; ++r)
                rc = odo_batch_track(b, pairs, npairs, rgbOnly, icpWeight, fastOdom, so3, scratch_results);
            BCK(cudaEventRecord(e1, b->stream));
            BCK(cudaEventSynchronize(e1));
            BCK(cudaEventElapsedTime(&ms, e0, e1));
            ms /= 2;
            if (rc == ODO_OK && ms < best) {
                best = ms;
                bt = cand_t[ti];
                bp = cand_p[pi];
            }
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    int rc = odo_batch_set_launch(b, bt, bp);
    *threads = bt;
    *pixels_per_thread = bp;
    if (best_ms) *best_ms = best;
    return rc;
}

const char *odo_batch_last_error(odo_batch_t *b) { return b ? b->last_error.c_str() : ""; }

}  // extern "C"
