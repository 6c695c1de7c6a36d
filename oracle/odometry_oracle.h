/*
 * CPU oracle for the dense RGB-D tracking path (test infrastructure only).
 *
 * This is a plain-C restatement of the reference's odometry kernels and host
 * loop, used by the tests, by smoke() and by bench.py's CPU-baseline leg as the
 * checker.  Nothing in the product library links or calls it.
 *
 * The same source is compiled twice:
 *   orc32_*  -- FP32 arithmetic as in the reference (host solve in FP64)
 *   orc64_*  -- every floating-point value in FP64 (the precision oracle)
 * Kernels whose outputs are integers (depth pyramid, intensity, u8 pyramid,
 * derivative images) are shared and always computed in FP32 as the reference
 * does (orc_*).
 *
 * Images are dense row-major (pitch == width).  Vertex/normal maps are planar
 * [3][rows][cols] as in the reference's DeviceArray2D<float> layout
 * (src/odom/RGBDOdometryef.cpp:97-101).
 */
#ifndef SLAM_GB300_ODOMETRY_ORACLE_H
#define SLAM_GB300_ODOMETRY_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Correspondence record, same fields as the reference DataTerm
 * (src/cuda/types.cuh:75-81). */
typedef struct {
    int16_t zero_x, zero_y; /* pixel in the last (model) image */
    int16_t one_x, one_y;   /* pixel in the next (live) image */
    float diff;             /* next - last intensity */
    int32_t valid;
} orc_dataterm;

typedef struct {
    float lastICPError, lastICPCount;
    float lastRGBError, lastRGBCount;
    float lastSO3Error, lastSO3Count;
    double lastA[36];
    double lastb[6];
} orc_stats;

/* ---- integer-output image kernels (shared by both precisions) ---- */
void orc_pyr_down_depth(const uint16_t *src, int sw, int sh, uint16_t *dst);
void orc_bgr_to_intensity(const uint8_t *rgba, int w, int h, uint8_t *dst, uint8_t *tie);
void orc_pyr_down_uchar_gauss(const uint8_t *src, int sw, int sh, uint8_t *dst, uint8_t *tie);
void orc_derivatives(const uint8_t *src, int w, int h, int16_t *dx, int16_t *dy, uint8_t *tie);
/* depth pre-filter shaders of the reference (src/gl/shaders/depth_bilateral.frag,
 * depth_metric.frag) */
void orc_depth_bilateral(const uint16_t *raw, int w, int h, float maxD, uint16_t *out, uint8_t *tie);
void orc_depth_metric(const uint16_t *raw, int w, int h, float maxD, float *out);
/* model prediction and fill-in (src/model/shaders/splat.vert + combo_splat.frag,
 * src/gl/shaders/fill_*.frag) */
void orc_model_predict(const float *surfels, int n, const float *t_inv, int cols, int rows, float cx, float cy,
                       float fx, float fy, float maxDepth, float confThreshold, int time, int maxTime, int timeDelta,
                       uint8_t *image, float *vertex, float *normal, uint16_t *tmap);
void orc_fill_in(const float *pv, const float *pn, const uint8_t *pi, const uint16_t *raw_d, const uint8_t *raw_rgba,
                 int cols, int rows, float cx, float cy, float fx, float fy, int passthrough, float *ov, float *on,
                 uint8_t *oi);

#ifdef __cplusplus
}
#endif
#endif
