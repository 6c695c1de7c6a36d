// Internal types shared by the host driver (odo_host.cpp) and the kernels
// (odo_maps.cu, odo_track.cu).  Plain C++ (no CUDA headers beyond the
// runtime's vector types), so g++ can compile the host side.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace slamgb {

constexpr int kLevels = 3;

// Pitched 2-D image view (pitch in bytes), like the reference's
// PtrStepSz<T> (src/cuda/containers/kernel_containers.hpp:72-92).
// 16-byte aligned so that a kernel holding the descriptor in shared memory
// reads {data, pitch} with one 16-byte load.
template <typename T>
struct __align__(16) Img {
    T *data;
    size_t pitch;
    int cols, rows;
};

// Planar 3-channel map [3][rows][cols] with a row pitch in bytes (the
// reference's DeviceArray2D<float>(rows*3, cols), src/odom/RGBDOdometryef.cpp:97-101).
struct __align__(16) Map3 {
    float *data;
    size_t pitch;
    int cols, rows;
};

// Photometric correspondence, 16 bytes, written by the residual pass and
// read by the photometric reduction as one vector: model pixel (u0, v0),
// intensity difference, valid flag, the model depth at (u0, v0) and the
// live image derivatives at this pixel, so that the reduction gathers
// nothing.  Replaces the 16-byte DataTerm (src/cuda/types.cuh:75-81); the
// live pixel is implied by the position.
struct __align__(16) Corr {
    int16_t u0, v0, diff, valid;
    float z;
    int16_t dx, dy;
};
static_assert(sizeof(Corr) == 16, "Corr layout");

struct Intr {
    float fx, fy, cx, cy;
};

// Device-resident state of one getIncrementalTransformation call.
struct TrackState {
    // inputs
    float Rprev[9], tprev[3], Rprev_inv[9];
    float icpWeight;
    int rgbOnly, icp, rgb, so3;
    // evolving pose
    double resultRt[16];
    double resultR[9];   // SO3 pre-alignment result
    float Rcurr[9], tcurr[3];
    float krkinv[9], kt[3];  // photometric warp of the next iteration (same level)
    // photometric warp of the first iteration of each level (computed from
    // resultRt when the previous level ends), the levels' intrinsics
    // (fx, fy, cx, cy) and the iterations scheduled per level
    float krk0[kLevels][9], kt0[kLevels][3];
    float Kl[kLevels][4];
    int sched[kLevels];
    float sigmaVal;
    int level_break;     // rgbOnly early exit for the current level
    // statistics (RGBDOdometryef public members)
    float lastICPError, lastICPCount, lastRGBError, lastRGBCount, lastSO3Error, lastSO3Count;
    double lastA[36], lastb[6];
    int so3_iters, iters_run[kLevels];
    int status;          // 0 ok, else ODO_ERR_* (timeouts of bounded waits)
    // device-side phase timers (ns, accumulated; globaltimer): [0] last-block
    // partial reduction, [1] FP64 solve + pose update, [2] residual finish,
    // [3] number of solves, [4] LDLT, [5] exp + compose, [6] FP32 pose +
    // polar factor, [7] next warp
    double prof[8];
    // per Gauss-Newton iteration (debugging): icp count, rgb count, sigma,
    // increment x[0..5]
    int nhist;
    double hist[32][9];
    unsigned long long t_begin, t_end;  // device globaltimer at the start / end of the call
    unsigned long long t_start;         // batch: globaltimer when the batch's first kernel ran
    unsigned long long t_solve;         // globaltimer at the end of the pair's last Gauss-Newton solve
    // output
    float out_R[9], out_t[3];
};

struct LevelArgs {
    int level;
    int cols, rows;
    Intr K;
    // ICP
    Map3 vmap_curr, nmap_curr, vmap_prev, nmap_prev;
    float distThres, angleThres;
    // photometric
    Img<const int16_t> dIdx, dIdy;
    Img<const float> lastDepth, nextDepth;
    Img<const uint8_t> lastImage, nextImage;
    Img<Corr> corr;
    Img<const uint8_t> cand;  // pose-independent photometric preconditions, per pixel
    float minScale;
    float maxDepthDelta;
    float sobelScale;
};

// Reduction workspace (owned by the handle).
struct ReduceWs {
    float *icp_part;       // [max_blocks][32]
    float *rgb_part;       // [max_blocks][32]
    int *res_part;         // [max_blocks][2]
    unsigned *counters;    // [4]
    int max_blocks;
};

// ---- per-image argument blocks of the preprocessing kernels (one per
// frame pair; the batched launchers take device arrays of them) ----
struct PyrArgs {
    Img<const uint16_t> src;
    Img<uint16_t> dst;
};
struct VNArgs {
    Img<const uint16_t> depth[kLevels];
    Map3 vmap[kLevels], nmap[kLevels];
    float fx_inv[kLevels], fy_inv[kLevels], cx[kLevels], cy[kLevels];
    float cutoff;
};
struct ModelArgs {
    const float *v4, *n4;
    size_t pitch4;
    int cols0, rows0;
    Map3 vmap[kLevels], nmap[kLevels];
    int do_transform;
    float R[9], t[3];
    // level-0 photometric depth of these maps: the vertex z cut at 6 m
    // (verticesToDepth), written beside the import
    float *vz;
    size_t vz_pitch;
};
struct RgbdArgs {
    const float *vz;
    size_t vz_pitch;
    const uint8_t *rgba;
    size_t rgba_pitch;
    Img<float> depth0;
    Img<uint8_t> img0;
    int do_depth;
};
struct GaussArgs {
    Img<const float> dsrc;
    Img<float> ddst;
    Img<const uint8_t> isrc;
    Img<uint8_t> idst;
    int do_depth;
};
struct DerivArgs {
    Img<const uint8_t> src[kLevels];
    Img<int16_t> dx[kLevels], dy[kLevels];
    Img<const float> depth[kLevels];
    Img<uint8_t> cand[kLevels];
    float minScale[kLevels];
};

// Batched launches: `args` is a device array of npairs blocks; the grid
// covers the largest image (max_cols x max_rows at level 0), blocks outside a
// smaller pair's image return at once.
cudaError_t launch_pyr_down_depth_batch(const PyrArgs *args, int npairs, int max_cols, int max_rows, cudaStream_t s);
cudaError_t launch_vmap_nmap_batch(const VNArgs *args, int npairs, int max_cols, int max_rows, cudaStream_t s);
cudaError_t launch_model_maps_batch(const ModelArgs *args, int npairs, int max_cols, int max_rows, cudaStream_t s);
cudaError_t launch_rgbd_level0_batch(const RgbdArgs *args, int npairs, int max_cols, int max_rows, cudaStream_t s);
cudaError_t launch_gauss_down_batch(const GaussArgs *args, int npairs, int max_cols, int max_rows, cudaStream_t s);
cudaError_t launch_derivatives_batch(const DerivArgs *args, int npairs, int max_cols, int max_rows, cudaStream_t s);

// ---- launchers: preprocessing (odo_maps.cu) ----
cudaError_t launch_pyr_down_depth(Img<const uint16_t> src, Img<uint16_t> dst, cudaStream_t s);
cudaError_t launch_vmap_nmap(const Img<const uint16_t> *depth, const Map3 *vmap, const Map3 *nmap, const Intr *K,
                             float cutoff, int nlevels, cudaStream_t s);
cudaError_t launch_model_maps(const float *v4, const float *n4, size_t pitch4, int cols, int rows, const Map3 *vmap,
                              const Map3 *nmap, int nlevels, int do_transform, const float R[9], const float t[3],
                              float *vz, size_t vz_pitch, cudaStream_t s);
cudaError_t launch_rgbd_level0(const float *vz, size_t vz_pitch, const uint8_t *rgba, size_t rgba_pitch, int cols,
                               int rows, Img<float> depth0, Img<uint8_t> img0, int do_depth, cudaStream_t s);
cudaError_t launch_gauss_down(Img<const float> dsrc, Img<float> ddst, Img<const uint8_t> isrc, Img<uint8_t> idst,
                              int do_depth, cudaStream_t s);
cudaError_t launch_derivatives(const Img<const uint8_t> *src, const Img<int16_t> *dx, const Img<int16_t> *dy,
                               const Img<const float> *nextDepth, const Img<uint8_t> *cand, const float *minScale,
                               int nlevels, cudaStream_t s);

// ---- launchers: tracking (odo_track.cu) ----
// FP64 intrinsics and inverse of one pyramid level (computed on the host).
struct KMats {
    double K[9], Kinv[9];
};

// One pair's arguments of the two per-iteration kernels at one level.
struct PassArgs {
    LevelArgs L;
    TrackState *st;
    ReduceWs ws;
    int nb_icp, nb_rgb;  // blocks of this pair in the two kernels (0: level unused)
    int iters;           // iterations of this pair at this level
    float invFx, invFy;
    KMats km;
};

// One pair's SO3 inputs (level 2 images and intrinsics).
struct So3Args {
    TrackState *st;
    Img<const uint8_t> last, next;
    Intr K2;
};

struct TrackLaunch {
    int blocks_icp;    // grid of the association/reduction kernel
    int blocks_rgb;    // grid of the photometric reduction kernel
    int threads;       // block size of both
    int precision;     // 0 FP32, 1 compensated
};
cudaError_t launch_track_begin(TrackState *st, cudaStream_t s);
cudaError_t launch_so3(TrackState *st, Img<const uint8_t> last, Img<const uint8_t> next, Intr K2, cudaStream_t s);
cudaError_t launch_level_iteration(const LevelArgs &L, TrackState *st, ReduceWs ws, const TrackLaunch &cfg, int iter,
                                   cudaStream_t s);
// depth pre-filter (depth_filter.cu)
cudaError_t launch_depth_bilateral(const uint16_t *src, size_t sp, uint16_t *dst, size_t dp, int cols, int rows,
                                   float maxD, cudaStream_t s);

// grid barriers of the persistent kernel give up after this many polls
constexpr long long kPersistentSpinLimit = 1ll << 26;
cudaError_t launch_level_persistent(const LevelArgs &L, TrackState *st, ReduceWs ws, const TrackLaunch &cfg,
                                    int iterations, int sm_count, cudaStream_t s,
                                    long long spin_limit = kPersistentSpinLimit, int absent = -1);
cudaError_t launch_track_end(TrackState *st, cudaStream_t s);
cudaError_t launch_iteration_part(const LevelArgs &L, TrackState *st, ReduceWs ws, const TrackLaunch &cfg, int iter,
                                  int which, cudaStream_t s);
int persistent_max_blocks(int threads);
KMats make_kmats(const Intr &K);

// batched tracking launches (pair = blockIdx.y of the pass kernels, one
// thread-block cluster per pair for SO3); `states` is a device array
cudaError_t launch_track_begin_batch(TrackState *states, int npairs, cudaStream_t s);
cudaError_t launch_stamp_batch(TrackState *states, int npairs, cudaStream_t s);
cudaError_t launch_warm_seed_batch(TrackState *states, const float *init, int npairs, cudaStream_t s);
cudaError_t launch_track_end_batch(TrackState *states, int npairs, cudaStream_t s);
cudaError_t launch_so3_batch(const So3Args *args, int npairs, cudaStream_t s);
// parts: bit 0 the association/residual kernel, bit 1 the photometric/solve kernel
cudaError_t launch_level_iteration_batch(const PassArgs *args, int npairs, int max_nb_icp, int max_nb_rgb,
                                         int threads, int precision, int iter, cudaStream_t s, int parts = 3,
                                         int split_solve = 1);

// debug single passes
cudaError_t launch_debug_icp(const LevelArgs &L, const float Rcurr[9], const float tcurr[3], const float Rprev_inv[9],
                             const float tprev[3], int32_t *assoc, double *out29_dev, ReduceWs ws,
                             const TrackLaunch &cfg, cudaStream_t s);
cudaError_t launch_debug_icp_sums(const LevelArgs &L, const float Rcurr[9], const float tcurr[3],
                                  const float Rprev_inv[9], const float tprev[3], double *out29_dev, ReduceWs ws,
                                  const TrackLaunch &cfg, cudaStream_t s);
cudaError_t launch_debug_rgb_sums(const LevelArgs &L, float sigma, double *out29_dev, ReduceWs ws,
                                  const TrackLaunch &cfg, cudaStream_t s);
cudaError_t launch_debug_rgb_residual(const LevelArgs &L, const float krkinv[9], const float kt[3], int *out2_dev,
                                      ReduceWs ws, const TrackLaunch &cfg, cudaStream_t s);
cudaError_t launch_debug_rgb_step(const LevelArgs &L, float sigma, double *out29_dev, ReduceWs ws,
                                  const TrackLaunch &cfg, cudaStream_t s);
cudaError_t launch_debug_so3(Img<const uint8_t> last, Img<const uint8_t> next, const float *params_dev,
                             double *out11_dev, cudaStream_t s);

// Copy between pinned host memory (addressed by the device directly) and
// device memory by a kernel on stream s, not by the copy engines
// (transfer.cu).
cudaError_t launch_host_copy(void *dst, const void *src, size_t bytes, cudaStream_t s);

}  // namespace slamgb
