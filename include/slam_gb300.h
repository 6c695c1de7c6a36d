/*
 * slam_gb300 -- GB300-native dense RGB-D tracking (frame-to-model
 * ICP + photometric odometry), C ABI.
 *
 * Drop-in for the reference class RGBDOdometryef
 * (src/odom/RGBDOdometryef.h:28-131).  The reference takes GL textures
 * (GPUTexture*, src/gl/types.h:9-37) and maps them through CUDA-GL interop;
 * here every frame input is a plain DEVICE pointer with a row pitch in bytes,
 * read on the handle's CUDA stream:
 *   filtered depth   GL_LUMINANCE16UI  ->  const uint16_t*  (millimetres)
 *   RGB              GL_RGBA8          ->  const uint8_t*   (RGBA, 4 B/px)
 *   vertices/normals GL_RGBA32F        ->  const float*     (4 floats/px,
 *                                           camera frame; z == 0 marks a hole)
 * Poses are row-major: rot[9] = R (3x3), trans[3] = t, pose[16] = 4x4
 * camera-to-world.
 *
 * Every function returns ODO_OK (0) or an error code and never exits the
 * process (the reference's cudaSafeCall calls exit(0),
 * src/cuda/convenience.cuh:64-71).  A handle owns its device buffers and one
 * CUDA stream; it is not thread-safe, but separate handles are independent
 * (no mutable globals, unlike the reference's __constant__/texture globals,
 * src/odom/utils.cu:548, 579-580; the one exception is the fixed device
 * array of the allocation-free entry point below, which needs no handle).
 *
 * Call order per frame, as in the reference (src/apps/elastic_fusion_file.cpp:367-374):
 *   odo_init_icp_model -> odo_init_rgb_model -> odo_init_icp_depth (or
 *   odo_init_icp_maps) -> odo_init_rgb -> odo_get_incremental_transformation.
 * NOTE (kept from the reference, src/odom/RGBDOdometryef.cpp:239,245): the
 * depth pyramids used by the photometric term come from the vertex map last
 * passed to odo_init_icp_model / odo_init_icp_maps, not from the depth image.
 */
#ifndef SLAM_GB300_H
#define SLAM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ODO_OK 0
#define ODO_ERR_ARG 1      /* bad argument (NULL, size, pitch, level) */
#define ODO_ERR_CUDA 2     /* a CUDA runtime call failed; see odo_last_error */
#define ODO_ERR_STATE 3    /* call-order violation */
#define ODO_ERR_OOM 4      /* device allocation failed */
#define ODO_ERR_TIMEOUT 5  /* a bounded device-side wait gave up */
#define ODO_ERR_SIZE 6     /* image larger than the allocation-free entry point's fixed scratch allows */

typedef struct odo_handle odo_t;

/* The reference's default thresholds (src/odom/RGBDOdometryef.h:35-36):
 * distThresh = 0.10f, angleThresh = sin(20.f * 3.14159254f / 180.f), the
 * latter evaluated as the reference evaluates it (float argument, result
 * rounded to float). */
#define ODO_DEFAULT_DIST_THRESH 0.10f
#define ODO_DEFAULT_ANGLE_THRESH 0.342020094f

/* The public metric members of RGBDOdometryef (src/odom/RGBDOdometryef.h:62-70). */
typedef struct {
    float lastICPError;
    float lastICPCount;
    float lastRGBError;
    float lastRGBCount;
    float lastSO3Error;
    float lastSO3Count;
    double lastA[36]; /* row-major 6x6 */
    double lastb[6];
} odo_stats;

/* RGBDOdometryef::RGBDOdometryef, src/odom/RGBDOdometryef.cpp:21-111.
 * Pass ODO_DEFAULT_DIST_THRESH and ODO_DEFAULT_ANGLE_THRESH for the
 * reference defaults (src/odom/RGBDOdometryef.h:35-36).  width/height must be >= 8 and
 * <= 8192. */
int odo_create(int width, int height, float cx, float cy, float fx, float fy, float distThresh, float angleThresh,
               odo_t **out);
int odo_destroy(odo_t *h);

/* Use `stream` (a cudaStream_t) for all work of this handle.  NULL (the
 * default) means the legacy default stream: the handle then works on its own
 * stream (its CUDA graphs cannot be captured on the legacy stream) and orders
 * every call after the work already queued on the legacy default stream,
 * where the caller produced its inputs. */
int odo_set_stream(odo_t *h, void *stream);

/* initICP(GPUTexture* filteredDepth, depthCutoff), src/odom/RGBDOdometryef.cpp:118-142 */
int odo_init_icp_depth(odo_t *h, const uint16_t *depth, size_t pitch_bytes, float depthCutoff);

/* The reference's depth pre-filter followed by initICP(depth): the FILTER
 * compute pack (src/gl/shaders/depth_bilateral.frag:30-76, a 13x13 bilateral
 * filter of the raw depth that zeroes values outside [300 mm, maxD]) feeding
 * initICP(DEPTH_FILTERED) (src/apps/elastic_fusion_file.cpp:349-370).  The
 * filtered image goes straight into the handle's level-0 depth. */
int odo_init_icp_raw_depth(odo_t *h, const uint16_t *raw_depth, size_t pitch_bytes, float maxD, float depthCutoff);

/* The depth pre-filter alone, device to device on `stream` (NULL: legacy
 * default stream); no handle:
 *  odo_filter_depth  depth_bilateral.frag (src/gl/shaders/depth_bilateral.frag:30-76),
 *                    u16 mm -> u16 mm;
 *  odo_depth_metric  depth_metric.frag (src/gl/shaders/depth_metric.frag:28-40),
 *                    u16 mm -> float m, 0 outside [300 mm, maxD].
 * maxD in metres (the reference's maxDepthProcessed / depthCutoff); out must
 * not overlap raw. */
int odo_filter_depth(const uint16_t *raw, size_t raw_pitch, uint16_t *out, size_t out_pitch, int width, int height,
                     float maxD, void *stream);
int odo_depth_metric(const uint16_t *raw, size_t raw_pitch, float *out, size_t out_pitch, int width, int height,
                     float maxD, void *stream);

/* ---- model prediction and fill-in (the producers of initICPModel's maps) ----
 * IndexMap::combinedPredict (src/model/IndexMap.cpp:243-345, shaders
 * src/model/shaders/splat.vert + combo_splat.frag) as CUDA splatting of the
 * surfel map: surfels [n][12] float (device, 16-byte aligned): position xyz +
 * confidence, colour (packed rgb as float) + unused + init time + last
 * update time, normal xyz + radius -- the reference's Vertex layout
 * (3 x vec4).  t_inv = the inverse of the camera pose (row-major 4x4; only
 * its first three rows are read).  Outputs (device, any may be NULL): RGBA
 * image (4 B/px), vertex and normal maps (RGBA32F, camera frame; all zero
 * where nothing was drawn) and the u16 time map.  scratch: device memory of
 * odo_model_predict_scratch_bytes(width, height) bytes, 8-byte aligned (the
 * depth-test buffer).  Asynchronous on `stream`. */
typedef struct {
    int width, height;
    float cx, cy, fx, fy;
    float maxDepth;       /* depthCutoff */
    float confThreshold;
    int time, maxTime, timeDelta;
} odo_predict_params;
size_t odo_model_predict_scratch_bytes(int width, int height);
int odo_model_predict(const float *surfels, int nsurfels, const float t_inv[16], const odo_predict_params *p,
                      void *scratch, uint8_t *image, size_t image_pitch, float *vertex, float *normal,
                      size_t map_pitch, uint16_t *time, size_t time_pitch, void *stream);
/* FillIn::vertex / normal / image (src/gl/FillIn.cpp, shaders
 * src/gl/shaders/fill_vertex.frag, fill_normal.frag, fill_rgb.frag): the
 * predicted maps with their holes (vertex or normal z == 0, rgb sum 0) -- or
 * everything when passthrough != 0 -- filled from the raw frame: vertices
 * from the filtered u16 depth (mm), normals from forward differences of
 * those vertices, colour from raw_rgba.  Outputs may be NULL (that fill is
 * skipped); asynchronous on `stream`. */
int odo_fill_in(const float *pred_vertex, const float *pred_normal, size_t pred_map_pitch, const uint8_t *pred_image,
                size_t pred_image_pitch, const uint16_t *raw_depth, size_t raw_depth_pitch, const uint8_t *raw_rgba,
                size_t raw_rgba_pitch, int width, int height, float cx, float cy, float fx, float fy,
                int passthrough, float *out_vertex, float *out_normal, size_t out_map_pitch, uint8_t *out_image,
                size_t out_image_pitch, void *stream);

/* initICP(GPUTexture* verts, GPUTexture* norms, depthCutoff), src/odom/RGBDOdometryef.cpp:144-167 */
int odo_init_icp_maps(odo_t *h, const float *verts, const float *norms, size_t pitch_bytes, float depthCutoff);

/* initICPModel(verts, norms, depthCutoff, modelPose), src/odom/RGBDOdometryef.cpp:169-206 */
int odo_init_icp_model(odo_t *h, const float *verts, const float *norms, size_t pitch_bytes, float depthCutoff,
                       const float pose[16]);

/* initRGB / initRGBModel / initFirstRGB, src/odom/RGBDOdometryef.cpp:237-265 */
int odo_init_rgb(odo_t *h, const uint8_t *rgba, size_t pitch_bytes);
int odo_init_rgb_model(odo_t *h, const uint8_t *rgba, size_t pitch_bytes);
int odo_init_first_rgb(odo_t *h, const uint8_t *rgba, size_t pitch_bytes);

/* getIncrementalTransformation, src/odom/RGBDOdometryef.cpp:267-595.
 * trans/rot: in = previous pose, out = tracked pose.  Blocks until the
 * result is on the host. */
int odo_get_incremental_transformation(odo_t *h, float trans[3], float rot[9], int rgbOnly, float icpWeight,
                                       int pyramid, int fastOdom, int so3);

/* getCovariance, src/odom/RGBDOdometryef.cpp:597-600: inverse of lastA (row-major 6x6). */
int odo_get_covariance(odo_t *h, double out[36]);

/* lastICPError ... lastb of the last odo_get_incremental_transformation. */
int odo_get_stats(odo_t *h, odo_stats *out);

/* Iterations actually run by the last tracking call: out[0] = SO3
 * iterations, out[1..3] = Gauss-Newton iterations at levels 0, 1, 2. */
int odo_get_iterations(odo_t *h, int out[4]);

/* Execution mode of odo_get_incremental_transformation:
 *  ODO_MODE_GRAPH      (default) the whole tracking call is one captured CUDA
 *                      graph: per iteration one association/reduction
 *                      kernel and one photometric/solve kernel, the 6x6
 *                      solve and pose update on the device;
 *  ODO_MODE_STREAM     the same kernels launched one by one (no graph);
 *  ODO_MODE_PERSISTENT one cooperative kernel per pyramid level that runs all
 *                      iterations with grid-wide barriers. */
#define ODO_MODE_GRAPH 0
#define ODO_MODE_STREAM 1
#define ODO_MODE_PERSISTENT 2
int odo_set_mode(odo_t *h, int mode);

/* Reduction precision:
 *  ODO_PREC_FP32         FP32 accumulation as in the reference;
 *  ODO_PREC_COMPENSATED  FP32 with Kahan-compensated per-thread sums and
 *                        compensated tree reductions. */
#define ODO_PREC_FP32 0
#define ODO_PREC_COMPENSATED 1
int odo_set_precision(odo_t *h, int precision);

/* Bytes copied device -> host by one odo_get_incremental_transformation
 * (the pose and statistics block). */
size_t odo_state_bytes(void);

/* Message of the last failing CUDA call on this handle ("" if none). */
const char *odo_last_error(odo_t *h);
const char *odo_status_string(int status);

/* ---- batched tracking ----
 * Many independent frame pairs of any sizes tracked together, e.g. the
 * loop-closure candidate checks of the reference (Ferns::findFrame,
 * src/lc/Ferns.cpp:237-279; model-to-model verification,
 * src/apps/elastic_fusion_file.cpp:450-498).  For each pair the call does what
 * initFirstRGB(prev_rgba) + initICPModel(model_verts, model_norms, cutoff,
 * pose) + initRGBModel(model_rgba) + initICP(depth, cutoff) + initRGB(rgba) +
 * getIncrementalTransformation(pose) do on one handle
 * (src/odom/RGBDOdometryef.cpp:118-595), with the iteration schedule
 * 10/5/4 restricted to the pair's first `levels` pyramid levels.  All pairs
 * run in one CUDA graph; with the default launch shape every pair's result is
 * bit-identical to the single-pair call. */
typedef struct odo_batch odo_batch_t;

typedef struct {
    int width, height;           /* level-0 size, 16..8192 */
    float fx, fy, cx, cy;
    float distThresh, angleThresh; /* <= 0: ODO_DEFAULT_DIST_THRESH, ODO_DEFAULT_ANGLE_THRESH */
    float depthCutoff;           /* <= 0: 20 m (maxDepthProcessed, src/configs/ef_file.cfg:16) */
    int levels;                  /* pyramid levels iterated, 1..3 */
    int iterations[3];           /* per-level Gauss-Newton iterations (0: the reference's 10 (3 fastOdom) / 5 / 4), <= 20 */
    const float *model_verts, *model_norms; /* RGBA32F, row pitch model_pitch */
    size_t model_pitch;
    const uint8_t *model_rgba;
    size_t model_rgba_pitch;
    const uint16_t *depth;       /* live depth, mm */
    size_t depth_pitch;
    const uint8_t *rgba;         /* live RGBA */
    size_t rgba_pitch;
    const uint8_t *prev_rgba;    /* previous live RGBA for the SO3 stage (may be NULL when so3 = 0) */
    size_t prev_rgba_pitch;
    float pose[16];              /* model pose = starting pose, row-major camera-to-world */
    /* Live side as camera-frame RGBA32F vertex / normal maps instead of a
     * depth image: initICP(verts, norms) (src/odom/RGBDOdometryef.cpp:144-167)
     * in place of initICP(depth).  When set, `depth` is not read and the live
     * photometric depth comes from these vertices (as the reference's
     * initRGB after initICP(verts, norms) does); NULL: depth input.  All
     * pairs of one call use the same kind of live input. */
    const float *live_verts, *live_norms;
    size_t live_pitch;
} odo_pair;

typedef struct {
    float pose[16];              /* tracked pose */
    float lastICPError, lastICPCount, lastRGBError, lastRGBCount, lastSO3Error, lastSO3Count;
    int iterations[4];           /* SO3, level 0, level 1, level 2 */
    double done_us;              /* time from the batch's first kernel to the end of this pair's last solve */
    double lastA[36], lastb[6];
} odo_pair_result;

int odo_batch_create(int max_pairs, odo_batch_t **out);
int odo_batch_destroy(odo_batch_t *b);
/* stream: as odo_set_stream (NULL: follow the legacy default stream). */
int odo_batch_set_stream(odo_batch_t *b, void *stream);
/* Launch shape of the two iteration kernels: threads per block (128 or 256)
 * and pixels per thread (each pair gets ceil(pixels / (threads * ppt))
 * blocks, at most 2 per SM).  Default 256 x 2 (the single-pair shape). */
int odo_batch_set_launch(odo_batch_t *b, int threads, int pixels_per_thread);
int odo_batch_track(odo_batch_t *b, const odo_pair *pairs, int npairs, int rgbOnly, float icpWeight, int fastOdom,
                    int so3, odo_pair_result *results);
/* As odo_batch_track, but every pair starts from its own motion estimate
 * instead of the SO3 pre-alignment: init_dev[i] (device, 6 floats:
 * translation m, rotation vector rad) is the live camera's motion in the
 * model camera's frame, so tracking starts at pose * exp(init) (no
 * counterpart in the reference; used by the learned warm start). */
int odo_batch_track_init(odo_batch_t *b, const odo_pair *pairs, int npairs, const float *init_dev, int rgbOnly,
                         float icpWeight, int fastOdom, odo_pair_result *results);
/* Loop-closure verification of candidate pairs, as the reference's callers
 * decide it after one tracking call each:
 *  - Ferns::findFrame (src/lc/Ferns.cpp:253-279): ICP only (icpWeight 100),
 *    no pyramid (levels = 1), no SO3, live side as maps; accept when
 *    lastICPError < max_icp_error (3e-4) and lastICPCount > min_icp_count
 *    (2400, or 1400 when tracking is lost);
 *  - model-to-model (src/apps/elastic_fusion_file.cpp:462-498): ICP + RGB
 *    (icpWeight 10), pyramid, no SO3; accept when every diagonal entry of
 *    getCovariance() is <= max_covariance (covThresh 1e-5),
 *    lastICPCount > min_icp_count (icpCountThresh 40000) and
 *    lastICPError < max_icp_error (icpErrThresh 5e-5).
 * A test whose threshold is <= 0 is skipped.  All candidates run in one
 * batched call (odo_batch_track); covariance (host, may be NULL) gets each
 * pair's row-major 6x6 inverse of lastA, accept (host) 1 or 0 per pair. */
typedef struct {
    int rgbOnly;
    float icpWeight;
    int fastOdom;
    int so3;
    float max_icp_error;
    float min_icp_count;
    double max_covariance;
} odo_verify_params;
int odo_batch_verify(odo_batch_t *b, const odo_pair *pairs, int npairs, const odo_verify_params *vp,
                     odo_pair_result *results, double *covariance, int *accept);
/* Times every launch shape ({128, 256} threads x {2, 4, 8, 16, 32, 64} pixels
 * per thread) on these pairs, keeps the fastest and returns it. */
int odo_batch_autotune(odo_batch_t *b, const odo_pair *pairs, int npairs, int rgbOnly, float icpWeight, int fastOdom,
                       int so3, odo_pair_result *scratch_results, int *threads, int *pixels_per_thread,
                       float *best_ms);
const char *odo_batch_last_error(odo_batch_t *b);
/* Times `reps` Gauss-Newton iterations at `level` over all pairs of the last
 * odo_batch_track call (CUDA events on the batch stream): out_ms[0] / [1] the
 * association and photometric/solve kernels alone, out_ms[2] both; restores
 * the tracking states afterwards. */
int odo_batch_debug_time_iteration(odo_batch_t *b, int level, int reps, float out_ms[3]);

/* ---- parity / debugging access (used by the tests) ----
 * Buffer ids: 0 depth pyramid (u16), 1 vmap_curr, 2 nmap_curr, 3 vmap_prev,
 * 4 nmap_prev (planar float [3][rows][cols]), 5 lastDepth, 6 nextDepth
 * (float), 7 lastImage, 8 nextImage, 9 lastNextImage (u8), 10 dIdx, 11 dIdy
 * (int16), 12 correspondences (16 bytes per pixel: int16 u0, v0, diff,
 * valid; float model depth at (u0, v0); int16 dIdx, dIdy at the pixel).
 * Copies are dense (pitch = cols * element size) and synchronous. */
int odo_debug_download(odo_t *h, int which, int level, void *host_dst, size_t bytes);
int odo_debug_upload(odo_t *h, int which, int level, const void *host_src, size_t bytes);

/* One ICP association/reduction pass at `level` with explicit poses
 * (icpStep, src/odom/reduce.cu:418-490).  assoc (host, rows*cols int32,
 * may be NULL) gets the gathered model pixel index or -1; out29 the 27
 * products, residual^2 and inlier count (summed in FP64 from block
 * partials). */
int odo_debug_icp_step(odo_t *h, int level, const float Rcurr[9], const float tcurr[3], const float Rprev_inv[9],
                       const float tprev[3], int32_t *assoc, double out29[29]);

/* The ICP sums exactly as a tracking iteration hands them to the 6x6 solve:
 * the same pass in the handle's precision (odo_set_precision), reduced
 * across blocks in FP32 (or compensated FP32) in the tracker's order, then
 * widened to FP64.  Used to measure summation error against an FP64 oracle. */
int odo_debug_icp_sums(odo_t *h, int level, const float Rcurr[9], const float tcurr[3], const float Rprev_inv[9],
                       const float tprev[3], double out29[29]);

/* The photometric sums of buffer 12 as a tracking iteration hands them to
 * the solve (handle's precision, tracker's reduction order). */
int odo_debug_rgb_sums(odo_t *h, int level, float sigma, double out29[29]);

/* One photometric residual pass (computeRgbResidual, src/odom/reduce.cu:869-935)
 * writing buffer 12; out2 = {count, sum of squared differences (int32)}. */
int odo_debug_rgb_residual(odo_t *h, int level, const float krkinv[9], const float kt[3], int32_t out2[2]);

/* One photometric reduction (rgbStep, src/odom/reduce.cu:626-678) over
 * buffer 12 at `level` with weight parameter sigma. */
int odo_debug_rgb_step(odo_t *h, int level, float sigma, double out29[29]);

/* One SO3 reduction at level 2 (so3Step, src/odom/reduce.cu:1082-1140) on
 * lastNextImage vs nextImage. */
int odo_debug_so3_step(odo_t *h, const float homography[9], const float kinv[9], const float krlr[9],
                       double out11[11]);

/* Derivative images of nextImage at all levels (computeDerivativeImages,
 * src/odom/utils.cu:608-638). */
int odo_debug_derivatives(odo_t *h);

/* Times `reps` Gauss-Newton iterations at `level` (the two iteration kernels,
 * launched back to back on the handle's stream with the pose state of the
 * last tracking call) with CUDA events on that stream.  out_ms[0] / out_ms[1]
 * = mean duration of the association/reduction kernel and of the
 * photometric/solve kernel, each timed alone; out_ms[2] = mean time of one
 * whole iteration.  Leaves the tracking state as it found it. */
int odo_debug_time_iteration(odo_t *h, int level, int reps, float out_ms[3]);

/* The batched tracker's last iteration stage on this batch handle: 1
 * (default) the photometric pass and a one-block-per-pair solve kernel, 0 the
 * single-pair layout (the solve in the last block of the photometric pass).
 * Both give the same poses; takes effect for the next batch call. */
int odo_batch_debug_set_split(odo_batch_t *b, int on);

/* Failure detection of the persistent mode's grid-wide barriers: each wait
 * gives up after `polls` polls (default 2^26) and the tracking call returns
 * ODO_ERR_TIMEOUT.  absent_block >= 0 makes that block of every persistent
 * level kernel return at once without arriving at any barrier (a block that
 * died), so that the others' waits run out; -1 (default) for normal work.
 * The handle stays usable afterwards. */
int odo_debug_set_wait_limit(odo_t *h, long long polls, int absent_block);

/* Device-side phase timers accumulated over tracking calls (ns):
 * out[0] last-block reduction of the block partials, out[1] FP64 solve and
 * pose update, out[2] photometric residual finish, out[3] number of solves,
 * out[4..7] parts of out[1]: LDLT, SE(3) exp + compose, FP32 pose + polar
 * factor, next photometric warp.  reset != 0 clears them. */
int odo_debug_profile(odo_t *h, double out[8], int reset);

/* Per Gauss-Newton iteration of the last tracking call, 9 doubles per row:
 * ICP inliers, photometric count, sigma, increment (v, omega).  Returns the
 * number of rows written (<= max_rows); ODO_ERR_ARG on bad arguments. */
int odo_debug_history(odo_t *h, double *out, int max_rows);

/* ---- allocation-free ICP reduction ----
 * No counterpart in the reference: an extra entry point for callers that
 * cannot allocate device memory after start-up -- a tracker running inside
 * a fixed device-memory budget, or a real-time loop where cudaMalloc/cudaFree
 * would synchronise the device and stall other streams.  It computes one
 * ICP association + reduction pass: the caller passes the four planar maps
 * ([3][rows][cols] float, row pitch in bytes) and the poses; it returns the
 * 6x6 matrix A (row-major), b and {sum of squared residuals, inliers} on the
 * host.  It needs no handle and allocates nothing: its
 * block partials live in one fixed device array of this library
 * (ODO_NOALLOC_SCRATCH_BYTES, held by every device that loads the library
 * until the process exits).
 *  - Images up to ODO_NOALLOC_MAX_PIXELS pixels (cols * rows), and maps
 *    whose 3 * rows * pitch_bytes stays below 4 GiB (the kernels address
 *    them with 32-bit offsets); others return ODO_ERR_SIZE without touching
 *    the GPU.
 *  - The first call on a device looks up the array's device address (once
 *    per device, with that device current); make that first call before any
 *    stream capture.
 *  - Every call shares the array: calls that overlap on the GPU (other
 *    streams, other host threads) race on it and must be serialised by the
 *    caller.  Nothing in it needs to start at zero (each call overwrites
 *    every value it reads).
 *  - stream: a cudaStream_t (NULL = the legacy default stream); the call
 *    returns after its results are on the host.
 * intr = {fx, fy, cx, cy} of the maps' pyramid level. */
#define ODO_NOALLOC_MAX_PIXELS 1048576
#define ODO_NOALLOC_SCRATCH_BYTES 139520
int odo_icp_step_noalloc(const float *vmap_curr, const float *nmap_curr, const float *vmap_prev,
                         const float *nmap_prev, size_t pitch_bytes, int cols, int rows, const float intr[4],
                         float distThresh, float angleThresh, const float Rcurr[9], const float tcurr[3],
                         const float Rprev_inv[9], const float tprev[3], void *stream, float matrixA[36],
                         float vectorB[6], float residual[2]);

/* ---- Learned warm start (no counterpart in the reference) ----
 * A BF16 CNN that proposes the coarse SE(3) motion of a frame pair from both
 * frames' 160x120 depth and gray images; forward and backward products run
 * on the tcgen05 tensor cores (FP32 accumulation).
 * Input [B][120][160][8] FP16 NHWC: model depth (m), model gray (0..1), live
 * depth (m), live gray, and four channels derived from them: live - model
 * gray, live - model depth, valid-depth fractions of the model and live
 * blocks.  Output [B][6]: translation (m)
 * and rotation vector (rad) of the live camera in the model camera's frame.
 * Six 3x3/stride-2 convolutions (8->32->64->128->128->128->128, ReLU; the
 * first one with FP16 operands, the others BF16), fc
 * 768->768 (ReLU), fc 768->6; odo_cnn_param_count() FP32 parameters.
 * Loss: mean over the batch of e^T M e, e = out - label, M a symmetric 6x6
 * metric (default diag(100, 100, 100, 36, 36, 36)); Adam. */
typedef struct odo_cnn odo_cnn_t;
size_t odo_cnn_param_count(void);
int odo_cnn_create(int max_batch, odo_cnn_t **out);
int odo_cnn_destroy(odo_cnn_t *n);
/* stream: all work of the network; NULL = the legacy default stream itself. */
int odo_cnn_set_stream(odo_cnn_t *n, void *stream);
int odo_cnn_init_params(odo_cnn_t *n, uint64_t seed);          /* He-normal weights, zero biases */
int odo_cnn_set_params(odo_cnn_t *n, const float *host_params); /* also resets the optimiser */
int odo_cnn_get_params(odo_cnn_t *n, float *host_params);
int odo_cnn_set_loss_metric(odo_cnn_t *n, const float metric[36]); /* row-major, symmetric */
/* out_dev (may be NULL): [batch][6] FP32 on the device */
int odo_cnn_forward(odo_cnn_t *n, const uint16_t *input_dev, int batch, float *out_dev);
/* Network inputs [npairs][120][160][8] of frame pairs whose level-0 size is
 * (160 s) x (120 s): s x s block means of the model depth (vertex z) and
 * intensity and of the live depth and intensity, and the derived channels
 * (asynchronous, on the network's stream). */
int odo_cnn_pack_input(odo_cnn_t *n, const odo_pair *pairs, int npairs, uint16_t *input_dev);
/* Motion proposals [npairs][6] (device) of frame pairs whose level-0 size is
 * (160 s) x (120 s): packing and forward pass in chunks of the network's
 * batch size, asynchronous on the network's stream; odo_cnn_event() is
 * recorded at its end (a cudaEvent_t) and odo_cnn_wait() waits for it and
 * reports a tensor-core time-out (ODO_ERR_TIMEOUT). */
int odo_cnn_propose(odo_cnn_t *n, const odo_pair *pairs, int npairs, float *out_dev);
void *odo_cnn_event(odo_cnn_t *n);
int odo_cnn_wait(odo_cnn_t *n);
/* forward + loss + backward + Adam (beta 0.9/0.999, eps 1e-8); loss_host may be NULL (no sync) */
int odo_cnn_train_step(odo_cnn_t *n, const uint16_t *input_dev, const float *labels_dev, int batch, float lr,
                       float *loss_host);
/* forward + loss + backward without an update; gradients in the parameter layout */
int odo_cnn_gradients(odo_cnn_t *n, const uint16_t *input_dev, const float *labels_dev, int batch,
                      float *grad_host, float *loss_host);
const char *odo_cnn_last_error(odo_cnn_t *n);
/* Learned warm start of batched tracking: proposals of the network for every
 * pair, tracking from pose * exp(proposal) with the short schedule of `wp`
 * (no SO3 stage), and a fall-back to the pair's own plain schedule (SO3 on)
 * for the pairs whose final ICP residual exceeds wp->residual_limit or whose
 * refined rotation differs from the proposal by more than wp->max_disagree
 * (rad).  fallback (host, may be NULL) gets 1 for those pairs. */
typedef struct {
    int levels;            /* pyramid levels iterated after the warm start, 1..3 */
    int iterations[3];     /* per-level iterations (0: the reference's 10 / 5 / 4) */
    float residual_limit;  /* <= 0: no residual test */
    float max_disagree;    /* rad; <= 0: no disagreement test */
    int rgbOnly;
    float icpWeight;
    int fastOdom;
} odo_warm_params;
int odo_batch_track_warm(odo_batch_t *b, odo_cnn_t *net, const odo_pair *pairs, int npairs,
                         const odo_warm_params *wp, odo_pair_result *results, int *fallback);

/* Copies `bytes` between pinned host memory (cudaMallocHost / cudaHostAlloc
 * / pinned tensors: the device addresses it directly) and device memory, in
 * either direction, by a kernel on `stream` instead of the copy engines --
 * the way the tracker moves its own argument blocks and states, so that it
 * never waits behind a caller's bulk copies; callers may use it for their
 * frames too.  Asynchronous; ODO_ERR_ARG on NULL pointers. */
int odo_host_copy(void *dst, const void *src, size_t bytes, void *stream);

/* PNG scanline filter reconstruction (filter types 0-4 of the PNG format)
 * for the TUM-format frame reader, whose reference reads its PNG images
 * through OpenCV (src/inputs/FileReader.cpp:43-55): `filtered` holds
 * `height` rows of 1 filter-type byte + row_bytes bytes (the inflated IDAT
 * stream), `out` receives height x row_bytes bytes; bpp = bytes per pixel
 * (1..8).  Host memory; ODO_ERR_ARG on an unknown filter type. */
int odo_png_unfilter(const uint8_t *filtered, int height, size_t row_bytes, int bpp, uint8_t *out);

/* GPU ray caster of the synthetic test scenes (scene struct of the synthetic
 * data generator, synth_scene): view i of scene view_scene[i] at
 * camera-to-world pose poses[16 i .. 16 i + 15] (row-major), depth noise
 * seed noise_seeds[i]; outputs (device, any may be NULL) stacked per view:
 * depth mm [n][h][w], RGBA [n][h][w][4], camera-frame vertices and normals
 * RGBA32F [n][h][w][4].  Synchronous on `stream`. */
int odo_synth_render(const void *scenes_host, int nscenes, const int *view_scene, const float *poses,
                     const uint64_t *noise_seeds, int n, int w, int h, float fx, float fy, float cx, float cy,
                     float noise_k, float dropout, int min_mm, int max_mm, uint16_t *depth_dev, uint8_t *rgba_dev,
                     float *vert_dev, float *norm_dev, void *stream);
/* C[M][N] (FP32) = A[M][K] B[N][K]^T with BF16 A, B (rows padded to a
 * multiple of 8 elements) on the tensor-core GEMM; bn = tile width 32..256,
 * layout = 0 (the library's operand layout), 1 (offsets exchanged; a
 * self-check of the layout) or 2 (layout 0 with FP16 operands), plus 4 for
 * the failure-detection test of the bounded tensor-core waits (one wait
 * runs out on a barrier that nothing arrives at; returns ODO_ERR_TIMEOUT
 * after draining the issued MMAs; needs K > 128); layout = 8: the
 * asynchronously fed kernel (operands copied into shared memory by
 * cp.async, a few K chunks in flight), BF16; layout = 9: the same with B
 * loaded by TMA, as the network's forward pass runs it (K a multiple of 8). */
int odo_cnn_debug_gemm(const uint16_t *A_dev, const uint16_t *B_dev, float *C_dev, int M, int N, int K, int bn,
                       int layout, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* SLAM_GB300_H */
