/*
 * CPU oracle for the dense RGB-D tracking path -- TEST INFRASTRUCTURE ONLY.
 *
 * Plain-C restatement of the reference (siw-engineering/slam, an ElasticFusion
 * fork).  Every function cites the reference file:line it follows.  Only the
 * tests, smoke() and bench.py's CPU-baseline leg load this code; the product
 * library never does.
 *
 * Compiled twice from this one file:
 *   -DORC_REAL_F32 : orc32_*  (FP32 arithmetic, host solve in FP64, as in the
 *                    reference)
 *   -DORC_REAL_F64 : orc64_*  (every float in FP64: the precision oracle)
 * Integer-output image kernels are shared and built once (ORC_SHARED).
 *
 * Floating-point conventions (the oracle is built with -ffp-contract=off):
 *  - accumulations of the form  acc += a * b  use an explicit fma(), because
 *    nvcc (fmad=true, as in the reference build) always fuses that pattern;
 *  - every other expression is evaluated with separately rounded IEEE ops;
 *  - divisions are IEEE.  The reference was built with --prec-div=false
 *    --prec-sqrt=false (src/CMakeLists.txt:116), whose GPU results may differ
 *    by a few ulp.  Where such a difference can flip an integer or a
 *    threshold decision the oracle raises a per-pixel "tie" flag, and the
 *    tests accept a GPU/oracle mismatch only on flagged pixels.
 *
 * Third-party arithmetic: the reference solves with Eigen (not vendored; the
 * Dockerfile installs Ubuntu 18.04 libeigen3-dev, Eigen 3.3.4).  The oracle
 * restates the published algorithms it uses:
 *  - LDLT with symmetric pivoting on the largest remaining |diagonal| and a
 *    pseudo-inverse of D (entries with |d| <= DBL_MIN / FLT_MIN give 0);
 *  - 3x3 inverse by cofactors; 4x4 rigid inverse; LU with partial pivoting;
 *  - Transform::rotation() of Eigen 3.3 = polar factor of the linear part
 *    (computed here with Newton iterations X <- (X + X^-T)/2 in FP64).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>
#include <limits.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "odometry_oracle.h"

#define NUM_PYRS 3

/* ====================================================================== */
/* Shared integer-output kernels (built once)                              */
/* ====================================================================== */
#ifdef ORC_SHARED

static int near_int(double q, double rel) {
    double r = nearbyint(q);
    return fabs(q - r) <= rel * (fabs(q) > 1.0 ? fabs(q) : 1.0);
}

/* pyrDownGaussKernel, src/odom/utils.cu:57-94 (sigma_color 30, :103). */
void orc_pyr_down_depth(const uint16_t *src, int sw, int sh, uint16_t *dst) {
    const int dw = sw / 2, dh = sh / 2, D = 5;
    const float weights[3] = {0.375f, 0.25f, 0.0625f};
    const float sigma_color = 30.f;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < dh; ++y) {
        for (int x = 0; x < dw; ++x) {
            int center = src[(2 * y) * sw + 2 * x];
            int x_mi = (2 * x - D / 2 > 0 ? 2 * x - D / 2 : 0) - 2 * x;
            int y_mi = (2 * y - D / 2 > 0 ? 2 * y - D / 2 : 0) - 2 * y;
            int x_ma = (sw < 2 * x - D / 2 + D ? sw : 2 * x - D / 2 + D) - 2 * x;
            int y_ma = (sh < 2 * y - D / 2 + D ? sh : 2 * y - D / 2 + D) - 2 * y;
            float sum = 0.f, wall = 0.f;
            for (int yi = y_mi; yi < y_ma; ++yi)
                for (int xi = x_mi; xi < x_ma; ++xi) {
                    int val = src[(2 * y + yi) * sw + 2 * x + xi];
                    if ((float)abs(val - center) < 3 * sigma_color) {
                        float wx = weights[abs(xi)], wy = weights[abs(yi)];
                        sum = fmaf((float)val * wx, wy, sum);
                        wall = fmaf(wx, wy, wall);
                    }
                }
            /* all partial sums are exact binary fractions (<= 24 bits) */
            dst[y * dw + x] = (uint16_t)(int)(sum / wall);
        }
    }
}

/* bgr2IntensityKernel, src/odom/utils.cu:550-563.  The input is the RGBA
 * texture, so byte 0 (R) is weighted 0.114 and byte 2 (B) 0.587. */
void orc_bgr_to_intensity(const uint8_t *rgba, int w, int h, uint8_t *dst, uint8_t *tie) {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            const uint8_t *p = rgba + 4 * ((size_t)y * w + x);
            float v = (float)p[0] * 0.114f + (float)p[1] * 0.299f + (float)p[2] * 0.587f;
            dst[(size_t)y * w + x] = (uint8_t)(int)v;
            if (tie) {
                double e = (double)p[0] * 0.114f + (double)p[1] * 0.299f + (double)p[2] * 0.587f;
                tie[(size_t)y * w + x] = near_int(e, 1e-6);
            }
        }
}

static const float gauss5x5[25] = {1, 4, 6, 4, 1, 4, 16, 24, 16, 4, 6, 24, 36, 24, 6,
                                   4, 16, 24, 16, 4, 1, 4, 6, 4, 1};

/* pyrDownKernelIntensityGauss, src/odom/utils.cu:470-500: masked (> 0)
 * Gaussian, window clamped to cols-1/rows-1 (exclusive), reversed kernel
 * index, int count, float->u8 truncation (0/0 gives NaN, stored as 0). */
void orc_pyr_down_uchar_gauss(const uint8_t *src, int sw, int sh, uint8_t *dst, uint8_t *tie) {
    const int dw = sw / 2, dh = sh / 2, D = 5;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < dh; ++y)
        for (int x = 0; x < dw; ++x) {
            int tx = 2 * x - D / 2 + D < sw - 1 ? 2 * x - D / 2 + D : sw - 1;
            int ty = 2 * y - D / 2 + D < sh - 1 ? 2 * y - D / 2 + D : sh - 1;
            int cy = 2 * y - D / 2 > 0 ? 2 * y - D / 2 : 0;
            float sum = 0.f;
            int count = 0;
            for (; cy < ty; ++cy)
                for (int cx = (2 * x - D / 2 > 0 ? 2 * x - D / 2 : 0); cx < tx; ++cx) {
                    uint8_t s = src[cy * sw + cx];
                    if (s > 0) {
                        float g = gauss5x5[(ty - cy - 1) * 5 + (tx - cx - 1)];
                        sum = fmaf((float)s, g, sum);
                        count = (int)((float)count + g);
                    }
                }
            float q = sum / (float)count;
            dst[y * dw + x] = (q != q) ? 0 : (uint8_t)(int)q;
            if (tie) tie[y * dw + x] = (count > 0) && near_int((double)sum / count, 1e-6);
        }
}

/* applyKernel + computeDerivativeImages, src/odom/utils.cu:582-638:
 * 3x3 filter, kernel index runs 8..0 over the (border-truncated) window. */
void orc_derivatives(const uint8_t *src, int w, int h, int16_t *dx, int16_t *dy, uint8_t *tie) {
    const float gx[9] = {0.52201f, 0.00000f, -0.52201f, 0.79451f, -0.00000f,
                         -0.79451f, 0.52201f, 0.00000f, -0.52201f};
    const float gy[9] = {0.52201f, 0.79451f, 0.52201f, 0.00000f, 0.00000f,
                         0.00000f, -0.52201f, -0.79451f, -0.52201f};
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            float dxv = 0.f, dyv = 0.f;
            double ex = 0.0, ey = 0.0;
            int k = 8;
            int j1 = y + 1 < h - 1 ? y + 1 : h - 1, i1 = x + 1 < w - 1 ? x + 1 : w - 1;
            for (int j = (y - 1 > 0 ? y - 1 : 0); j <= j1; j++)
                for (int i = (x - 1 > 0 ? x - 1 : 0); i <= i1; i++) {
                    float s = (float)src[j * w + i];
                    dxv = fmaf(s, gx[k], dxv);
                    dyv = fmaf(s, gy[k], dyv);
                    ex += (double)s * gx[k];
                    ey += (double)s * gy[k];
                    --k;
                }
            dx[y * w + x] = (int16_t)(int)dxv;
            dy[y * w + x] = (int16_t)(int)dyv;
            if (tie) tie[y * w + x] = near_int(ex, 1e-6) || near_int(ey, 1e-6);
        }
}

/* uint(maxD * 1000.0f) of the depth shaders */
static unsigned depth_max_mm(float maxD) {
    float m = maxD * 1000.0f;
    return m <= 0.f ? 0u : (m >= 4294967040.f ? 0xffffffffu : (unsigned)m);
}

/* depth_bilateral.frag, src/gl/shaders/depth_bilateral.frag:30-76 (a GL
 * fragment shader in the reference): for a raw depth value in
 * [300, uint(maxD * 1000)], round(sum1 / sum2) over the 13x13 window clipped
 * to the image, taps row by row, w = exp(-(space2 * 0.024691358 + color2 *
 * 0.000555556)); other pixels 0.  The neighbours are read at their own texel
 * (the shader samples the texel corner cx / cols, which selects texel cx).
 * Rounding to nearest, ties to even; tie[] flags quotients within 2e-3 of a
 * half-integer, where another exp implementation may round the other way. */
void orc_depth_bilateral(const uint16_t *raw, int w, int h, float maxD, uint16_t *out, uint8_t *tie) {
    const unsigned max_mm = depth_max_mm(maxD);
    const float ks = 0.024691358f, kc = 0.000555556f;
    #pragma omp parallel for schedule(static)
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            const unsigned value = raw[(size_t)y * w + x];
            uint16_t o = 0;
            uint8_t t = 0;
            if (!(value > max_mm || value < 300u)) {
                const float v = (float)value;
                const int tx = x - 6 + 13 < w ? x - 6 + 13 : w;
                const int ty = y - 6 + 13 < h ? y - 6 + 13 : h;
                float sum1 = 0.f, sum2 = 0.f;
                for (int cy = y - 6 > 0 ? y - 6 : 0; cy < ty; ++cy)
                    for (int cx = x - 6 > 0 ? x - 6 : 0; cx < tx; ++cx) {
                        const float tmp = (float)raw[(size_t)cy * w + cx];
                        const float dx = (float)x - (float)cx, dy = (float)y - (float)cy;
                        const float space2 = dx * dx + dy * dy;
                        const float dc = v - tmp;
                        const float color2 = dc * dc;
                        const float weight = expf(-(space2 * ks + color2 * kc));
                        sum1 += tmp * weight;
                        sum2 += weight;
                    }
                const float q = sum1 / sum2;
                o = (uint16_t)nearbyintf(q);
                t = fabsf(fabsf(q - floorf(q)) - 0.5f) < 2e-3f;
            }
            out[(size_t)y * w + x] = o;
            if (tie) tie[(size_t)y * w + x] = t;
        }
}

/* depth_metric.frag, src/gl/shaders/depth_metric.frag:28-40: metres, 0
 * outside [300, uint(maxD * 1000)]. */
void orc_depth_metric(const uint16_t *raw, int w, int h, float maxD, float *out) {
    const unsigned max_mm = depth_max_mm(maxD);
    for (size_t i = 0; i < (size_t)w * h; ++i)
        out[i] = (raw[i] > max_mm || raw[i] < 300u) ? 0.f : (float)raw[i] / 1000.0f;
}

/* ---- model prediction (src/model/shaders/splat.vert, combo_splat.frag) and
 * fill-in (src/gl/shaders/fill_vertex.frag, fill_normal.frag, fill_rgb.frag),
 * single-operation rounded FP32 in the shaders' order, IEEE division and
 * square root; the depth test keeps the nearest fragment, the lower surfel
 * index on equal depth. */
typedef struct { float px, py, pz, conf, nx, ny, nz, rad, xw, yw, size; } orc_splat;

static void norm3f(float *x, float *y, float *z) {
    float l = sqrtf(*x * *x + *y * *y + *z * *z);
    *x = *x / l; *y = *y / l; *z = *z / l;
}

/* splat.vert, src/model/shaders/splat.vert:45-80 */
static int splat_vertex(const float *t, const float *S, float cx, float cy, float fx, float fy, int cols, int rows,
                        float maxDepth, float confThreshold, int time, int maxTime, int timeDelta, orc_splat *s) {
    const float *P = S, *C = S + 4, *N = S + 8;
    float hx = t[0] * P[0] + t[1] * P[1] + t[2] * P[2] + t[3];
    float hy = t[4] * P[0] + t[5] * P[1] + t[6] * P[2] + t[7];
    float hz = t[8] * P[0] + t[9] * P[1] + t[10] * P[2] + t[11];
    if (hz > maxDepth || hz < 0.f || P[3] < confThreshold || (float)time - C[3] > (float)timeDelta ||
        C[3] > (float)maxTime)
        return 0;
    s->px = hx; s->py = hy; s->pz = hz; s->conf = P[3];
    float nx = t[0] * N[0] + t[1] * N[1] + t[2] * N[2];
    float ny = t[4] * N[0] + t[5] * N[1] + t[6] * N[2];
    float nz = t[8] * N[0] + t[9] * N[1] + t[10] * N[2];
    norm3f(&nx, &ny, &nz);
    s->nx = nx; s->ny = ny; s->nz = nz; s->rad = N[3];
    float hc = (float)cols * 0.5f, hr = (float)rows * 0.5f;
    float ndx = ((fx * hx) / hz + cx - hc) / hc, ndy = ((fy * hy) / hz + cy - hr) / hr;
    s->xw = (ndx + 1.f) * hc;
    s->yw = (ndy + 1.f) * hr;
    float ax = ny - nz, ay = -nx, az = nx;
    norm3f(&ax, &ay, &az);
    ax = ax * N[3] * 1.41421356f; ay = ay * N[3] * 1.41421356f; az = az * N[3] * 1.41421356f;
    float bx = ny * az - nz * ay, by = nz * ax - nx * az, bz = nx * ay - ny * ax;
    float ox[4] = {ax, bx, -bx, -ax}, oy[4] = {ay, by, -by, -ay}, oz[4] = {az, bz, -bz, -az};
    float xmin = 3.4e38f, xmax = -3.4e38f, ymin = 3.4e38f, ymax = -3.4e38f;
    for (int q = 0; q < 4; ++q) {
        float qx = hx + ox[q], qy = hy + oy[q], qz = hz + oz[q];
        float u = (fx * qx) / qz + cx, v = (fy * qy) / qz + cy;
        xmin = fminf(xmin, u); xmax = fmaxf(xmax, u); ymin = fminf(ymin, v); ymax = fmaxf(ymax, v);
    }
    float size = fmaxf(0.f, fmaxf(fabsf(xmax - xmin), fabsf(ymax - ymin)));
    s->size = fminf(fmaxf(size, 1.f), 2047.f);
    (void)rows;
    return 1;
}

/* combo_splat.frag, src/model/shaders/combo_splat.frag:35-58 */
static int splat_fragment(const orc_splat *s, int x, int y, float cx, float cy, float fx, float fy, float *z) {
    float u = (float)x + 0.5f, v = (float)y + 0.5f;
    float lx = (u - cx) / fx, ly = (v - cy) / fy, lz = 1.f;
    norm3f(&lx, &ly, &lz);
    float f = (s->px * s->nx + s->py * s->ny + s->pz * s->nz) / (lx * s->nx + ly * s->ny + lz * s->nz);
    float qx = f * lx, qy = f * ly, qz = f * lz;
    float dx = qx - s->px, dy = qy - s->py, dz = qz - s->pz;
    if (dx * dx + dy * dy + dz * dz > s->rad * s->rad) return 0;
    *z = qz;
    return 1;
}

/* IndexMap::combinedPredict, src/model/IndexMap.cpp:243-345.  surfels [n][12];
 * outputs image [h][w][4] u8, vertex / normal [h][w][4] f32, time [h][w] u16. */
void orc_model_predict(const float *surfels, int n, const float *t_inv, int cols, int rows, float cx, float cy,
                       float fx, float fy, float maxDepth, float confThreshold, int time, int maxTime, int timeDelta,
                       uint8_t *image, float *vertex, float *normal, uint16_t *tmap) {
    const size_t np = (size_t)cols * rows;
    uint64_t *z = (uint64_t *)malloc(np * sizeof(uint64_t));
    for (size_t i = 0; i < np; ++i) z[i] = ~0ull;
    for (int i = 0; i < n; ++i) {
        orc_splat s;
        if (!splat_vertex(t_inv, surfels + 12 * (size_t)i, cx, cy, fx, fy, cols, rows, maxDepth, confThreshold, time,
                          maxTime, timeDelta, &s))
            continue;
        if (!isfinite(s.xw) || !isfinite(s.yw)) continue;
        float h = s.size * 0.5f;
        float lo_x = s.xw - h - 0.5f, hi_x = s.xw + h - 0.5f, lo_y = s.yw - h - 0.5f, hi_y = s.yw + h - 0.5f;
        int x0 = (int)ceilf(fmaxf(lo_x, 0.f)), y0 = (int)ceilf(fmaxf(lo_y, 0.f));
        int x1 = (int)ceilf(fminf(hi_x, (float)cols)) - 1, y1 = (int)ceilf(fminf(hi_y, (float)rows)) - 1;
        for (int y = y0; y <= y1; ++y)
            for (int x = x0; x <= x1; ++x) {
                float zz;
                if (!splat_fragment(&s, x, y, cx, cy, fx, fy, &zz)) continue;
                float depth = zz / (2.f * maxDepth) + 0.5f;
                depth = fminf(fmaxf(depth, 0.f), 1.f);
                if (!(depth < 1.f)) continue;
                uint32_t db;
                memcpy(&db, &depth, 4);
                uint64_t key = ((uint64_t)db << 32) | (uint32_t)i;
                if (key < z[(size_t)y * cols + x]) z[(size_t)y * cols + x] = key;
            }
    }
    const float ifx = 1.f / fx, ify = 1.f / fy;
    for (int y = 0; y < rows; ++y)
        for (int x = 0; x < cols; ++x) {
            size_t p = (size_t)y * cols + x;
            uint8_t im[4] = {0, 0, 0, 0};
            float vo[4] = {0, 0, 0, 0}, no[4] = {0, 0, 0, 0};
            uint16_t tm = 0;
            if (z[p] != ~0ull) {
                const float *S = surfels + 12 * (size_t)(uint32_t)(z[p] & 0xffffffffu);
                orc_splat s;
                float zz = 0.f;
                splat_vertex(t_inv, S, cx, cy, fx, fy, cols, rows, maxDepth, confThreshold, time, maxTime, timeDelta,
                             &s);
                splat_fragment(&s, x, y, cx, cy, fx, fy, &zz);
                int c = (int)S[4];
                im[0] = (uint8_t)((c >> 16) & 0xff); im[1] = (uint8_t)((c >> 8) & 0xff); im[2] = (uint8_t)(c & 0xff);
                im[3] = 255;
                vo[0] = ((float)x + 0.5f - cx) * zz * ifx; vo[1] = ((float)y + 0.5f - cy) * zz * ify;
                vo[2] = zz; vo[3] = s.conf;
                no[0] = s.nx; no[1] = s.ny; no[2] = s.nz; no[3] = s.rad;
                float tf = S[6];
                tm = tf <= 0.f ? 0 : (tf >= 65535.f ? 65535 : (uint16_t)tf);
            }
            if (image) memcpy(image + 4 * p, im, 4);
            if (vertex) memcpy(vertex + 4 * p, vo, 16);
            if (normal) memcpy(normal + 4 * p, no, 16);
            if (tmap) tmap[p] = tm;
        }
    free(z);
}

/* getVertex of src/gl/shaders/geometry.glsl:48-53 on u16 mm depth, edge-clamped */
static void fill_raw_vertex(const uint16_t *d, int cols, int rows, float cx, float cy, float ifx, float ify, int x,
                            int y, float *v) {
    x = x < 0 ? 0 : (x >= cols ? cols - 1 : x);
    y = y < 0 ? 0 : (y >= rows ? rows - 1 : y);
    float z = (float)d[(size_t)y * cols + x] / 1000.0f;
    v[0] = ((float)x - cx) * z * ifx; v[1] = ((float)y - cy) * z * ify; v[2] = z;
}

/* FillIn::vertex / normal / image (fill_vertex.frag:37-53, fill_normal.frag:34-50,
 * fill_rgb.frag:29-37); dense images, outputs may be NULL. */
void orc_fill_in(const float *pv, const float *pn, const uint8_t *pi, const uint16_t *raw_d, const uint8_t *raw_rgba,
                 int cols, int rows, float cx, float cy, float fx, float fy, int passthrough, float *ov, float *on,
                 uint8_t *oi) {
    const float ifx = 1.f / fx, ify = 1.f / fy;
    for (int y = 0; y < rows; ++y)
        for (int x = 0; x < cols; ++x) {
            size_t p = (size_t)y * cols + x;
            if (ov) {
                memcpy(ov + 4 * p, pv + 4 * p, 16);
                if (pv[4 * p + 2] == 0.f || passthrough) {
                    float v[3];
                    fill_raw_vertex(raw_d, cols, rows, cx, cy, ifx, ify, x, y, v);
                    ov[4 * p] = v[0]; ov[4 * p + 1] = v[1]; ov[4 * p + 2] = v[2]; ov[4 * p + 3] = 1.f;
                }
            }
            if (on) {
                memcpy(on + 4 * p, pn + 4 * p, 16);
                if (pn[4 * p + 2] == 0.f || passthrough) {
                    float v[3], vx[3], vy[3];
                    fill_raw_vertex(raw_d, cols, rows, cx, cy, ifx, ify, x, y, v);
                    fill_raw_vertex(raw_d, cols, rows, cx, cy, ifx, ify, x + 1, y, vx);
                    fill_raw_vertex(raw_d, cols, rows, cx, cy, ifx, ify, x, y + 1, vy);
                    float ax = vx[0] - v[0], ay = vx[1] - v[1], az = vx[2] - v[2];
                    float bx = vy[0] - v[0], by = vy[1] - v[1], bz = vy[2] - v[2];
                    float nx = ay * bz - az * by, ny = az * bx - ax * bz, nz = ax * by - ay * bx;
                    norm3f(&nx, &ny, &nz);
                    on[4 * p] = nx; on[4 * p + 1] = ny; on[4 * p + 2] = nz; on[4 * p + 3] = 1.f;
                }
            }
            if (oi) {
                memcpy(oi + 4 * p, pi + 4 * p, 4);
                if ((int)pi[4 * p] + pi[4 * p + 1] + pi[4 * p + 2] == 0 || passthrough) {
                    memcpy(oi + 4 * p, raw_rgba + 4 * p, 3);
                    oi[4 * p + 3] = 255;
                }
            }
        }
}

/* thread control for the timed CPU baseline */
void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
int orc_get_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

#endif /* ORC_SHARED */

/* ====================================================================== */
/* Precision-generic part                                                  */
/* ====================================================================== */
#if defined(ORC_REAL_F32) || defined(ORC_REAL_F64)

#ifdef ORC_REAL_F64
typedef double real;
#define ORC(n) orc64_##n
#define RSQRT(v) (1.0 / sqrt(v))
#define SQRT(v) sqrt(v)
#define FMA(a, b, c) fma(a, b, c)
#define ABS(v) fabs(v)
#define RNEAR(v) nearbyint(v)
#define R_EPS DBL_EPSILON
#define R_TINY DBL_MIN
#else
typedef float real;
#define ORC(n) orc32_##n
#define RSQRT(v) (1.0f / sqrtf(v))
#define SQRT(v) sqrtf(v)
#define FMA(a, b, c) fmaf(a, b, c)
#define ABS(v) fabsf(v)
#define RNEAR(v) nearbyintf(v)
#define R_EPS FLT_EPSILON
#define R_TINY FLT_MIN
#endif

void orc_pyr_down_depth(const uint16_t *src, int sw, int sh, uint16_t *dst);
void orc_bgr_to_intensity(const uint8_t *rgba, int w, int h, uint8_t *dst, uint8_t *tie);
void orc_pyr_down_uchar_gauss(const uint8_t *src, int sw, int sh, uint8_t *dst, uint8_t *tie);
void orc_derivatives(const uint8_t *src, int w, int h, int16_t *dx, int16_t *dy, uint8_t *tie);

typedef struct { real x, y, z; } v3;
typedef struct { v3 r[3]; } m33; /* rows, like the reference mat33 */

static inline v3 mk(real x, real y, real z) { v3 a = {x, y, z}; return a; }
static inline v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 add(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
/* src/cuda/operators.cuh:67-91 */
static inline v3 cross(v3 a, v3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline real dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline real norm3(v3 a) { return SQRT(dot(a, a)); }
static inline v3 normalized(v3 a) {
    real rn = RSQRT(dot(a, a));
    return mk(a.x * rn, a.y * rn, a.z * rn);
}
static inline v3 mv(const m33 *m, v3 a) { return mk(dot(m->r[0], a), dot(m->r[1], a), dot(m->r[2], a)); }
static inline int isnan_r(real v) { return v != v; }
static inline real qnan(void) { return (real)NAN; }

/* __float2int_rn: round half to even, NaN -> 0, saturating. */
static inline int f2i_rn(real v) {
    if (v != v) return 0;
    double r = nearbyint((double)v);
    if (r >= 2147483647.0) return INT_MAX;
    if (r <= -2147483648.0) return INT_MIN;
    return (int)r;
}
static inline int near_half(real q, double rel, double scale) {
    double f = (double)q - floor((double)q);
    return fabs(f - 0.5) <= rel * scale;
}
static inline int near_thr(double a, double t, double rel) {
    double s = fabs(a) > fabs(t) ? fabs(a) : fabs(t);
    return fabs(a - t) <= rel * (s > 1e-30 ? s : 1e-30);
}
#define TIE_REL 4e-6

/* Tie flipping (test infrastructure): when set, every decision flagged as a
 * tie -- a quotient rounded to an integer within TIE_REL of the half-way
 * point, a threshold comparison within TIE_REL of the threshold -- is taken
 * the other way.  The pose difference between a normal and a flipped run
 * measures how much the tracking result depends on decisions the reference's
 * approximate division may take differently from IEEE arithmetic. */
/* 0 none, 1 all ties, m >= 2: half (m - 2) % 2 of the ties by a hash of the
 * tied value with seed (m - 2) / 2 (modes 2 and 3 are complementary halves,
 * 4 and 5 another split, ...) */
static int g_flip_ties = 0;
void ORC(set_flip_ties)(int on) { g_flip_ties = on; }

static inline int flip_this(double v) {
    if (g_flip_ties == 1) return 1;
    uint64_t b;
    memcpy(&b, &v, sizeof(b));
    b ^= 0x9e3779b97f4a7c15ull * (uint64_t)((g_flip_ties - 2) / 2);
    b ^= b >> 33; b *= 0xff51afd7ed558ccdull; b ^= b >> 33;
    return (int)(b & 1) == (g_flip_ties - 2) % 2;
}

/* __float2int_rn of a quotient, flagging (and, when flipping, reversing) a
 * rounding that sits on a tie. */
static inline int round_q(real q, int *tie) {
    int r = f2i_rn(q);
    if (near_half(q, TIE_REL, fabs((double)q) + 1.0)) {
        *tie = 1;
        if (g_flip_ties && flip_this((double)q)) {
            const double fl = floor((double)q);
            r = (r == (int)fl) ? (int)fl + 1 : (int)fl;
        }
    }
    return r;
}
/* a comparison result, reversed when flipping and its operands are a tie */
static inline int decide(int result, double a, double t, int *tie) {
    if (near_thr(a, t, TIE_REL)) {
        *tie = 1;
        if (g_flip_ties && flip_this(a)) return !result;
    }
    return result;
}

/* ------------------------------------------------------------------ */
/* Map kernels (src/odom/utils.cu)                                     */
/* ------------------------------------------------------------------ */

/* computeVmapKernel, src/odom/utils.cu:109-133.  Invalid pixels get NaN in
 * the x plane only; y/z keep whatever the buffer held. */
void ORC(create_vmap)(const uint16_t *depth, int w, int h, real fx_inv, real fy_inv, real cx, real cy,
                      real cutoff, real *vmap) {
    const size_t n = (size_t)w * h;
#pragma omp parallel for schedule(static)
    for (int v = 0; v < h; ++v)
        for (int u = 0; u < w; ++u) {
            real z = (real)depth[(size_t)v * w + u] / (real)1000;
            if (z != 0 && z < cutoff) {
                vmap[(size_t)v * w + u] = z * ((real)u - cx) * fx_inv;
                vmap[n + (size_t)v * w + u] = z * ((real)v - cy) * fy_inv;
                vmap[2 * n + (size_t)v * w + u] = z;
            } else {
                vmap[(size_t)v * w + u] = qnan();
            }
        }
}

/* computeNmapKernel, src/odom/utils.cu:151-188. */
void ORC(create_nmap)(const real *vmap, int w, int h, real *nmap) {
    const size_t n = (size_t)w * h;
#pragma omp parallel for schedule(static)
    for (int v = 0; v < h; ++v)
        for (int u = 0; u < w; ++u) {
            size_t i = (size_t)v * w + u;
            if (u == w - 1 || v == h - 1) { nmap[i] = qnan(); continue; }
            v3 v00, v01, v10;
            v00.x = vmap[i]; v01.x = vmap[i + 1]; v10.x = vmap[i + w];
            if (!isnan_r(v00.x) && !isnan_r(v01.x) && !isnan_r(v10.x)) {
                v00.y = vmap[n + i]; v01.y = vmap[n + i + 1]; v10.y = vmap[n + i + w];
                v00.z = vmap[2 * n + i]; v01.z = vmap[2 * n + i + 1]; v10.z = vmap[2 * n + i + w];
                v3 r = normalized(cross(sub(v01, v00), sub(v10, v00)));
                nmap[i] = r.x; nmap[n + i] = r.y; nmap[2 * n + i] = r.z;
            } else {
                nmap[i] = qnan();
            }
        }
}

/* tranformMapsKernel, src/odom/utils.cu:206-248 (in place allowed). */
void ORC(transform_maps)(const real *vsrc, const real *nsrc, int w, int h, const real R[9], const real t[3],
                         real *vdst, real *ndst) {
    const size_t n = (size_t)w * h;
    m33 M;
    M.r[0] = mk(R[0], R[1], R[2]); M.r[1] = mk(R[3], R[4], R[5]); M.r[2] = mk(R[6], R[7], R[8]);
    v3 tv = mk(t[0], t[1], t[2]);
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < n; ++i) {
        v3 vd = mk(qnan(), qnan(), qnan());
        real vx = vsrc[i];
        if (!isnan_r(vx)) {
            vd = add(mv(&M, mk(vx, vsrc[n + i], vsrc[2 * n + i])), tv);
            vdst[n + i] = vd.y; vdst[2 * n + i] = vd.z;
        }
        vdst[i] = vd.x;
        v3 nd = mk(qnan(), qnan(), qnan());
        real nx = nsrc[i];
        if (!isnan_r(nx)) {
            nd = mv(&M, mk(nx, nsrc[n + i], nsrc[2 * n + i]));
            ndst[n + i] = nd.y; ndst[2 * n + i] = nd.z;
        }
        ndst[i] = nd.x;
    }
}

/* copyMapsKernel, src/odom/utils.cu:270-310: RGBA32F -> planar, invalid if
 * the vertex z is 0 (all three planes written). */
void ORC(copy_maps)(const float *v4, const float *n4, int w, int h, real *vmap, real *nmap) {
    const size_t n = (size_t)w * h;
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < n; ++i) {
        int ok = !(v4[4 * i + 2] == 0);
        vmap[i] = ok ? (real)v4[4 * i + 0] : qnan();
        vmap[n + i] = ok ? (real)v4[4 * i + 1] : qnan();
        vmap[2 * n + i] = ok ? (real)v4[4 * i + 2] : qnan();
        nmap[i] = ok ? (real)n4[4 * i + 0] : qnan();
        nmap[n + i] = ok ? (real)n4[4 * i + 1] : qnan();
        nmap[2 * n + i] = ok ? (real)n4[4 * i + 2] : qnan();
    }
}

/* resizeMapKernel<normalize>, src/odom/utils.cu:365-416: 2x2 mean, NaN (x
 * plane only) if any x tap is NaN. */
void ORC(resize_map)(const real *in, int sw, int sh, real *out, int normalize) {
    const int dw = sw / 2, dh = sh / 2;
    const size_t sn = (size_t)sw * sh, dn = (size_t)dw * dh;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < dh; ++y)
        for (int x = 0; x < dw; ++x) {
            size_t s = (size_t)(2 * y) * sw + 2 * x, d = (size_t)y * dw + x;
            real x00 = in[s], x01 = in[s + 1], x10 = in[s + sw], x11 = in[s + sw + 1];
            if (isnan_r(x00) || isnan_r(x01) || isnan_r(x10) || isnan_r(x11)) { out[d] = qnan(); continue; }
            v3 m;
            m.x = (x00 + x01 + x10 + x11) / 4;
            m.y = (in[sn + s] + in[sn + s + 1] + in[sn + s + sw] + in[sn + s + sw + 1]) / 4;
            m.z = (in[2 * sn + s] + in[2 * sn + s + 1] + in[2 * sn + s + sw] + in[2 * sn + s + sw + 1]) / 4;
            if (normalize) m = normalized(m);
            out[d] = m.x; out[dn + d] = m.y; out[2 * dn + d] = m.z;
        }
}

/* pyrDownKernelGaussF, src/odom/utils.cu:332-363. */
void ORC(pyr_down_gauss_f)(const real *src, int sw, int sh, real *dst) {
    static const real g[25] = {1, 4, 6, 4, 1, 4, 16, 24, 16, 4, 6, 24, 36, 24, 6,
                               4, 16, 24, 16, 4, 1, 4, 6, 4, 1};
    const int dw = sw / 2, dh = sh / 2, D = 5;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < dh; ++y)
        for (int x = 0; x < dw; ++x) {
            int tx = 2 * x - D / 2 + D < sw - 1 ? 2 * x - D / 2 + D : sw - 1;
            int ty = 2 * y - D / 2 + D < sh - 1 ? 2 * y - D / 2 + D : sh - 1;
            int cy = 2 * y - D / 2 > 0 ? 2 * y - D / 2 : 0;
            real sum = 0;
            int count = 0;
            for (; cy < ty; ++cy)
                for (int cx = (2 * x - D / 2 > 0 ? 2 * x - D / 2 : 0); cx < tx; ++cx) {
                    real s = src[cy * sw + cx];
                    if (!isnan_r(s)) {
                        real gw = g[(ty - cy - 1) * 5 + (tx - cx - 1)];
                        sum = FMA(s, gw, sum);
                        count = (int)((real)count + gw);
                    }
                }
            dst[y * dw + x] = sum / (real)count;
        }
}

/* verticesToDepthKernel, src/odom/utils.cu:526-537. */
void ORC(vertices_to_depth)(const float *v4, int w, int h, real cutoff, real *dst) {
    const size_t n = (size_t)w * h;
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < n; ++i) {
        real z = (real)v4[4 * i + 2];
        dst[i] = (z > cutoff || z <= 0) ? qnan() : z;
    }
}

/* projectPointsKernel, src/odom/utils.cu:640-658 (cloud as [h][w][3]). */
void ORC(project_cloud)(const real *depth, int w, int h, real inv_fx, real inv_fy, real cx, real cy, real *cloud) {
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            size_t i = (size_t)y * w + x;
            real z = depth[i];
            cloud[3 * i + 0] = ((real)x - cx) * z * inv_fx;
            cloud[3 * i + 1] = ((real)y - cy) * z * inv_fy;
            cloud[3 * i + 2] = z;
        }
}

/* ------------------------------------------------------------------ */
/* Reductions                                                           */
/* ------------------------------------------------------------------ */
/* Per-pixel products are summed pairwise within each row, then the row sums
 * pairwise: deterministic for any thread count.  The reference's summation
 * order (grid-stride + shuffle tree, src/odom/reduce.cu:90-255) depends on
 * its launch shape, so sums are compared to a tolerance. */
static void products7(real *p, const real *row, real found) {
    int s = 0;
    for (int i = 0; i < 7; ++i)
        for (int j = i; j < 7; ++j) p[s++] = row[i] * row[j];
    p[28] = found;
}

/* Pairwise (cascade) sum of n records of ncomp values each (record stride
 * `stride`), leaves of up to 8 records summed in order.  Deterministic and
 * with O(log n) error growth, close to the GPU's tree reductions. */
/* Summation-order perturbation (test infrastructure): when set, every
 * pairwise sum visits its records in reverse order -- the same error
 * structure in another order, as a GPU reduction tree of another shape. */
static int g_reverse_sums = 0; /* 0 pairwise halves, 1 the same reversed, 2 split at a third */
void ORC(set_reverse_sums)(int on) { g_reverse_sums = on; }

static void pairwise_sum(const real *v, int n, int stride, int ncomp, real *out) {
    if (n <= (g_reverse_sums == 2 ? 5 : 8)) {
        for (int k = 0; k < ncomp; ++k) out[k] = 0;
        for (int j = 0; j < n; ++j) {
            const int i = g_reverse_sums == 1 ? n - 1 - j : j;
            for (int k = 0; k < ncomp; ++k) out[k] += v[(size_t)i * stride + k];
        }
        return;
    }
    real a[32], b[32];
    int m = g_reverse_sums == 2 ? n / 3 : n / 2;
    pairwise_sum(v, m, stride, ncomp, a);
    pairwise_sum(v + (size_t)m * stride, n - m, stride, ncomp, b);
    for (int k = 0; k < ncomp; ++k) out[k] = g_reverse_sums == 1 ? b[k] + a[k] : a[k] + b[k];
}

/* ------------------------------------------------------------------ */
/* ICP (src/odom/reduce.cu:257-490)                                     */
/* ------------------------------------------------------------------ */
typedef struct {
    m33 Rcurr; v3 tcurr;
    const real *vmap_curr, *nmap_curr;
    m33 Rprev_inv; v3 tprev;
    real fx, fy, cx, cy;
    const real *vmap_g_prev, *nmap_g_prev;
    real distThres, angleThres;
    int cols, rows;
} icp_args;

/* ICPReduction::search, src/odom/reduce.cu:282-325.  Returns 1 on a
 * correspondence; *idx gets the gathered pixel (or -1) and *tie a flag when
 * the GPU's approximate division could decide otherwise. */
static int icp_search(const icp_args *a, int x, int y, v3 *n, v3 *d, v3 *s, int *idx, int *tie) {
    const size_t N = (size_t)a->cols * a->rows;
    const size_t p = (size_t)y * a->cols + x;
    *idx = -1; *tie = 0;
    v3 vcurr = mk(a->vmap_curr[p], a->vmap_curr[N + p], a->vmap_curr[2 * N + p]);
    if (isnan_r(vcurr.x)) return 0; /* GPU: NaN -> (0,0) gather, then dist is NaN -> reject */
    v3 vcurr_g = add(mv(&a->Rcurr, vcurr), a->tcurr);
    v3 vcurr_cp = mv(&a->Rprev_inv, sub(vcurr_g, a->tprev));
    real qx = vcurr_cp.x * a->fx / vcurr_cp.z + a->cx;
    real qy = vcurr_cp.y * a->fy / vcurr_cp.z + a->cy;
    int tq = 0;
    int ux = round_q(qx, &tq), uy = round_q(qy, &tq);
    if (tq) *tie |= 1;
    if (ux < 0 || uy < 0 || ux >= a->cols || uy >= a->rows || vcurr_cp.z < 0) return 0;
    const size_t q = (size_t)uy * a->cols + ux;
    v3 vprev_g = mk(a->vmap_g_prev[q], a->vmap_g_prev[N + q], a->vmap_g_prev[2 * N + q]);
    v3 ncurr = mk(a->nmap_curr[p], a->nmap_curr[N + p], a->nmap_curr[2 * N + p]);
    v3 ncurr_g = mv(&a->Rcurr, ncurr);
    v3 nprev_g = mk(a->nmap_g_prev[q], a->nmap_g_prev[N + q], a->nmap_g_prev[2 * N + q]);
    real dist = norm3(sub(vprev_g, vcurr_g));
    real sine = norm3(cross(ncurr_g, nprev_g));
    *n = nprev_g; *d = vprev_g; *s = vcurr_g;
    int tt = 0;
    const int sine_ok = decide(sine < a->angleThres, sine, a->angleThres, &tt);
    const int dist_ok = decide(dist <= a->distThres, dist, a->distThres, &tt);
    if (tt) *tie |= 2;
    int ok = (sine_ok && dist_ok && !isnan_r(ncurr.x) && !isnan_r(nprev_g.x));
    if (ok) *idx = (int)q;
    return ok;
}

/* ICPReduction::getProducts + icpStep unpacking, src/odom/reduce.cu:327-490.
 * out29 = 27 upper-triangle products of [n, s x n, n.(s-d)], residual^2,
 * inlier count.  assoc (optional) gets the gathered pixel or -1; tie
 * (optional) the per-pixel flag. */
void ORC(icp_step)(const real Rcurr[9], const real tcurr[3], const real *vmap_curr, const real *nmap_curr,
                   const real Rprev_inv[9], const real tprev[3], real fx, real fy, real cx, real cy,
                   const real *vmap_g_prev, const real *nmap_g_prev, real distThres, real angleThres, int cols,
                   int rows, double out29[29], int32_t *assoc, uint8_t *tie) {
    icp_args a;
    for (int i = 0; i < 3; ++i) {
        a.Rcurr.r[i] = mk(Rcurr[3 * i], Rcurr[3 * i + 1], Rcurr[3 * i + 2]);
        a.Rprev_inv.r[i] = mk(Rprev_inv[3 * i], Rprev_inv[3 * i + 1], Rprev_inv[3 * i + 2]);
    }
    a.tcurr = mk(tcurr[0], tcurr[1], tcurr[2]);
    a.tprev = mk(tprev[0], tprev[1], tprev[2]);
    a.vmap_curr = vmap_curr; a.nmap_curr = nmap_curr;
    a.vmap_g_prev = vmap_g_prev; a.nmap_g_prev = nmap_g_prev;
    a.fx = fx; a.fy = fy; a.cx = cx; a.cy = cy;
    a.distThres = distThres; a.angleThres = angleThres;
    a.cols = cols; a.rows = rows;
    real *part = (real *)calloc((size_t)rows * 29, sizeof(real));
#pragma omp parallel
    {
    real *rb = (real *)malloc(sizeof(real) * (size_t)cols * 29);
#pragma omp for schedule(static)
    for (int y = 0; y < rows; ++y) {
        for (int x = 0; x < cols; ++x) {
            v3 n, d, s;
            int idx, tf;
            int found = icp_search(&a, x, y, &n, &d, &s, &idx, &tf);
            if (assoc) assoc[(size_t)y * cols + x] = idx;
            if (tie) tie[(size_t)y * cols + x] = (uint8_t)tf;
            real row[7] = {0, 0, 0, 0, 0, 0, 0};
            if (found) {
                v3 s_cp = mv(&a.Rprev_inv, sub(s, a.tprev));
                v3 d_cp = mv(&a.Rprev_inv, sub(d, a.tprev));
                v3 n_cp = mv(&a.Rprev_inv, n);
                v3 c = cross(s_cp, n_cp);
                row[0] = n_cp.x; row[1] = n_cp.y; row[2] = n_cp.z;
                row[3] = c.x; row[4] = c.y; row[5] = c.z;
                row[6] = dot(n_cp, sub(s_cp, d_cp));
            }
            products7(rb + (size_t)x * 29, row, (real)found);
        }
        pairwise_sum(rb, cols, 29, 29, part + (size_t)y * 29);
    }
    free(rb);
    }
    real tot[29];
    pairwise_sum(part, rows, 29, 29, tot);
    for (int k = 0; k < 29; ++k) out29[k] = (double)tot[k];
    free(part);
}

/* ------------------------------------------------------------------ */
/* RGB residual (src/odom/reduce.cu:739-935)                           */
/* ------------------------------------------------------------------ */
/* RGBResidual::getProducts.  Returns {count, sigma} with the int32
 * wrap-around of the reference's int2 reduction. */
void ORC(rgb_residual)(real minScale, const int16_t *dIdx, const int16_t *dIdy, const real *lastDepth,
                       const real *nextDepth, const uint8_t *lastImage, const uint8_t *nextImage, int cols,
                       int rows, real maxDepthDelta, const real kt[3], const real krkinv[9],
                       orc_dataterm *corres, int32_t out2[2], uint8_t *tie) {
    uint32_t cnt = 0, sig = 0;
    const int N = cols * rows;
#pragma omp parallel for schedule(static) reduction(+ : cnt, sig)
    for (int k = 0; k < N; ++k) {
        int i = k / cols, j0 = k - i * cols;
        orc_dataterm c;
        memset(&c, 0, sizeof(c));
        c.valid = 0;
        uint8_t tf = 0;
        if (j0 < cols - 5 && i < rows - 1) {
            int valid = 1;
            int u1 = i + 2 < rows ? i + 2 : rows, v1 = j0 + 2 < cols ? j0 + 2 : cols;
            for (int u = (i - 2 > 0 ? i - 2 : 0); u < u1; u++)
                for (int v = (j0 - 2 > 0 ? j0 - 2 : 0); v < v1; v++) valid = valid && (nextImage[u * cols + v] > 0);
            if (valid) {
                int16_t valx = dIdx[i * cols + j0], valy = dIdy[i * cols + j0];
                real mTwo = (real)((int)valx * valx + (int)valy * valy);
                if (mTwo >= minScale) {
                    int y = i, x = j0;
                    real d1 = nextDepth[y * cols + x];
                    if (!isnan_r(d1)) {
                        real td1 = d1 * (krkinv[6] * (real)x + krkinv[7] * (real)y + krkinv[8]) + kt[2];
                        real qu = (d1 * (krkinv[0] * (real)x + krkinv[1] * (real)y + krkinv[2]) + kt[0]) / td1;
                        real qv = (d1 * (krkinv[3] * (real)x + krkinv[4] * (real)y + krkinv[5]) + kt[1]) / td1;
                        int tq = 0;
                        int u0 = round_q(qu, &tq), v0 = round_q(qv, &tq);
                        if (tq) tf |= 1;
                        if (u0 >= 0 && v0 >= 0 && u0 < cols && v0 < rows) {
                            real d0 = lastDepth[v0 * cols + u0];
                            int tt = 0;
                            const int near = d0 > 0 && decide(ABS(td1 - d0) <= maxDepthDelta, ABS(td1 - d0),
                                                               maxDepthDelta, &tt);
                            if (d0 > 0 && tt) tf |= 2;
                            if (near && lastImage[v0 * cols + u0] != 0) {
                                c.zero_x = (int16_t)u0; c.zero_y = (int16_t)v0;
                                c.one_x = (int16_t)x; c.one_y = (int16_t)y;
                                c.diff = (float)nextImage[y * cols + x] - (float)lastImage[v0 * cols + u0];
                                c.valid = 1;
                                cnt += 1;
                                sig += (uint32_t)(int32_t)(c.diff * c.diff);
                            }
                        }
                    }
                }
            }
        }
        if (corres) corres[k] = c;
        if (tie) tie[k] = tf;
    }
    out2[0] = (int32_t)cnt;
    out2[1] = (int32_t)sig;
}

/* RGBReduction::getProducts, src/odom/reduce.cu:494-619. */
void ORC(rgb_step)(const orc_dataterm *corres, real sigma, const real *cloud, real fx, real fy,
                   const int16_t *dIdx, const int16_t *dIdy, real sobelScale, int cols, int rows,
                   double out29[29]) {
    real *part = (real *)calloc((size_t)rows * 29, sizeof(real));
#pragma omp parallel
    {
    real *rb = (real *)malloc(sizeof(real) * (size_t)cols * 29);
#pragma omp for schedule(static)
    for (int y = 0; y < rows; ++y) {
        for (int x = 0; x < cols; ++x) {
            const orc_dataterm *c = &corres[(size_t)y * cols + x];
            real row[7] = {0, 0, 0, 0, 0, 0, 0};
            if (c->valid) {
                real w = sigma + ABS((real)c->diff);
                w = w > (real)FLT_EPSILON ? (real)1 / w : (real)1;
                if (sigma == -1) w = 1;
                row[6] = -w * (real)c->diff;
                size_t z = (size_t)c->zero_y * cols + c->zero_x;
                real px = cloud[3 * z], py = cloud[3 * z + 1], pz = cloud[3 * z + 2];
                real invz = (real)(1.0 / (double)pz);
                size_t o = (size_t)c->one_y * cols + c->one_x;
                real gx = w * sobelScale * (real)dIdx[o];
                real gy = w * sobelScale * (real)dIdy[o];
                real v0 = gx * fx * invz;
                real v1 = gy * fy * invz;
                real v2 = -(v0 * px + v1 * py) * invz;
                row[0] = v0; row[1] = v1; row[2] = v2;
                row[3] = -pz * v1 + py * v2;
                row[4] = pz * v0 - px * v2;
                row[5] = -py * v0 + px * v1;
            }
            products7(rb + (size_t)x * 29, row, (real)(c->valid != 0));
        }
        pairwise_sum(rb, cols, 29, 29, part + (size_t)y * 29);
    }
    free(rb);
    }
    real tot[29];
    pairwise_sum(part, rows, 29, 29, tot);
    for (int k = 0; k < 29; ++k) out29[k] = (double)tot[k];
    free(part);
}

/* ------------------------------------------------------------------ */
/* SO3 (src/odom/reduce.cu:937-1140)                                    */
/* ------------------------------------------------------------------ */
/* SO3Reduction::getGradient, src/odom/reduce.cu:953-969 */
static void so3_grad(const uint8_t *img, int cols, int x, int y, real *gx, real *gy) {
    real actu = (real)img[y * cols + x];
    real back = (real)img[y * cols + x - 1], fore = (real)img[y * cols + x + 1];
    *gx = ((back + actu) / (real)2) - ((fore + actu) / (real)2);
    back = (real)img[(y - 1) * cols + x]; fore = (real)img[(y + 1) * cols + x];
    *gy = ((back + actu) / (real)2) - ((fore + actu) / (real)2);
}

/* SO3Reduction::getProducts, src/odom/reduce.cu:971-1054.  out11 = 9
 * upper-triangle products of [J(3), r], residual^2, count. */
void ORC(so3_step)(const uint8_t *lastImage, const uint8_t *nextImage, int cols, int rows, const real H[9],
                   const real kinv[9], const real krlr[9], double out11[11]) {
    real *part = (real *)calloc((size_t)rows * 11, sizeof(real));
    m33 Hm, Ki;
    for (int i = 0; i < 3; ++i) {
        Hm.r[i] = mk(H[3 * i], H[3 * i + 1], H[3 * i + 2]);
        Ki.r[i] = mk(kinv[3 * i], kinv[3 * i + 1], kinv[3 * i + 2]);
    }
#pragma omp parallel
    {
    real *rb = (real *)malloc(sizeof(real) * (size_t)cols * 11);
#pragma omp for schedule(static)
    for (int y = 0; y < rows; ++y) {
        for (int x = 0; x < cols; ++x) {
            real *acc = rb + (size_t)x * 11;
            v3 p = mk((real)x, (real)y, 1);
            v3 wp = mv(&Hm, p);
            int tq = 0;
            int wx = round_q(wp.x / wp.z, &tq), wy = round_q(wp.y / wp.z, &tq);
            int found = wx >= 1 && wx < cols - 1 && wy >= 1 && wy < rows - 1 && x >= 1 && x < cols - 1 && y >= 1 &&
                        y < rows - 1;
            real row[4] = {0, 0, 0, 0};
            if (found) {
                real gnx, gny, glx, gly;
                so3_grad(nextImage, cols, wx, wy, &gnx, &gny);
                so3_grad(lastImage, cols, x, y, &glx, &gly);
                real gx = (gnx + glx) / (real)2, gy = (gny + gly) / (real)2;
                v3 point = mv(&Ki, p);
                real z2 = point.z * point.z;
                real a = krlr[0], b = krlr[1], c = krlr[2], d = krlr[3], e = krlr[4], f = krlr[5];
                real g = krlr[6], h = krlr[7], ii = krlr[8];
                real fy_ = (real)y, fx_ = (real)x;
                v3 lp = mk(((point.z * (d * gy + a * gx)) - (gy * g * fy_) - (gx * g * fx_)) / z2,
                           ((point.z * (e * gy + b * gx)) - (gy * h * fy_) - (gx * h * fx_)) / z2,
                           ((point.z * (f * gy + c * gx)) - (gy * ii * fy_) - (gx * ii * fx_)) / z2);
                v3 jr = cross(lp, point);
                row[0] = jr.x; row[1] = jr.y; row[2] = jr.z;
                row[3] = -((real)nextImage[wy * cols + wx] - (real)lastImage[y * cols + x]);
            }
            int s = 0;
            for (int i = 0; i < 4; ++i)
                for (int j = i; j < 4; ++j) acc[s++] = row[i] * row[j];
            acc[10] = (real)found;
        }
        pairwise_sum(rb, cols, 11, 11, part + (size_t)y * 11);
    }
    free(rb);
    }
    real tot[11];
    pairwise_sum(part, rows, 11, 11, tot);
    for (int k = 0; k < 11; ++k) out11[k] = (double)tot[k];
    free(part);
}

/* ------------------------------------------------------------------ */
/* Small dense linear algebra (Eigen restatements, see file header)     */
/* ------------------------------------------------------------------ */
/* LDLT with symmetric pivoting on the largest remaining |diagonal|;
 * solve with the pseudo-inverse of D.  n <= 6.  Precision: FP64. */
static void ldlt_solve_d(int n, const double *Ain, const double *b, double *x) {
    double A[36];
    int perm[6];
    memcpy(A, Ain, sizeof(double) * n * n);
    for (int i = 0; i < n; ++i) perm[i] = i;
    for (int k = 0; k < n; ++k) {
        int p = k;
        double best = fabs(A[k * n + k]);
        for (int i = k + 1; i < n; ++i)
            if (fabs(A[i * n + i]) > best) { best = fabs(A[i * n + i]); p = i; }
        if (p != k) {
            for (int j = 0; j < n; ++j) { double t = A[k * n + j]; A[k * n + j] = A[p * n + j]; A[p * n + j] = t; }
            for (int i = 0; i < n; ++i) { double t = A[i * n + k]; A[i * n + k] = A[i * n + p]; A[i * n + p] = t; }
            int t = perm[k]; perm[k] = perm[p]; perm[p] = t;
        }
        /* A(k,k) -= sum_j L(k,j)^2 D(j); L(i,k) = (A(i,k) - sum_j L(i,j) L(k,j) D(j)) / A(k,k) */
        double t[6];
        for (int j = 0; j < k; ++j) t[j] = A[k * n + j] * A[j * n + j];
        double s = 0;
        for (int j = 0; j < k; ++j) s += A[k * n + j] * t[j];
        A[k * n + k] -= s;
        double akk = A[k * n + k];
        for (int i = k + 1; i < n; ++i) {
            double r = 0;
            for (int j = 0; j < k; ++j) r += A[i * n + j] * t[j];
            A[i * n + k] -= r;
            if (fabs(akk) > 0) A[i * n + k] /= akk;
        }
    }
    double y[6];
    for (int i = 0; i < n; ++i) y[i] = b[perm[i]];
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < i; ++j) y[i] -= A[i * n + j] * y[j];
    for (int i = 0; i < n; ++i) y[i] = fabs(A[i * n + i]) > DBL_MIN ? y[i] / A[i * n + i] : 0.0;
    for (int i = n - 1; i >= 0; --i)
        for (int j = i + 1; j < n; ++j) y[i] -= A[j * n + i] * y[j];
    for (int i = 0; i < n; ++i) x[perm[i]] = y[i];
}

/* Same algorithm in FP32 (the reference's SO3 solve is Eigen LDLT<float>,
 * src/odom/RGBDOdometryef.cpp:366). */
static void ldlt_solve_f(int n, const float *Ain, const float *b, float *x) {
    float A[9];
    int perm[3];
    memcpy(A, Ain, sizeof(float) * n * n);
    for (int i = 0; i < n; ++i) perm[i] = i;
    for (int k = 0; k < n; ++k) {
        int p = k;
        float best = fabsf(A[k * n + k]);
        for (int i = k + 1; i < n; ++i)
            if (fabsf(A[i * n + i]) > best) { best = fabsf(A[i * n + i]); p = i; }
        if (p != k) {
            for (int j = 0; j < n; ++j) { float t = A[k * n + j]; A[k * n + j] = A[p * n + j]; A[p * n + j] = t; }
            for (int i = 0; i < n; ++i) { float t = A[i * n + k]; A[i * n + k] = A[i * n + p]; A[i * n + p] = t; }
            int t = perm[k]; perm[k] = perm[p]; perm[p] = t;
        }
        float t[3];
        for (int j = 0; j < k; ++j) t[j] = A[k * n + j] * A[j * n + j];
        float s = 0;
        for (int j = 0; j < k; ++j) s += A[k * n + j] * t[j];
        A[k * n + k] -= s;
        float akk = A[k * n + k];
        for (int i = k + 1; i < n; ++i) {
            float r = 0;
            for (int j = 0; j < k; ++j) r += A[i * n + j] * t[j];
            A[i * n + k] -= r;
            if (fabsf(akk) > 0) A[i * n + k] /= akk;
        }
    }
    float y[3];
    for (int i = 0; i < n; ++i) y[i] = b[perm[i]];
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < i; ++j) y[i] -= A[i * n + j] * y[j];
    for (int i = 0; i < n; ++i) y[i] = fabsf(A[i * n + i]) > FLT_MIN ? y[i] / A[i * n + i] : 0.0f;
    for (int i = n - 1; i >= 0; --i)
        for (int j = i + 1; j < n; ++j) y[i] -= A[j * n + i] * y[j];
    for (int i = 0; i < n; ++i) x[perm[i]] = y[i];
}

/* 3x3 inverse by cofactors (FP64). */
static void inv33_d(const double *m, double *o) {
    double c00 = m[4] * m[8] - m[5] * m[7], c01 = m[5] * m[6] - m[3] * m[8], c02 = m[3] * m[7] - m[4] * m[6];
    double det = m[0] * c00 + m[1] * c01 + m[2] * c02;
    double id = 1.0 / det;
    o[0] = c00 * id; o[1] = (m[2] * m[7] - m[1] * m[8]) * id; o[2] = (m[1] * m[5] - m[2] * m[4]) * id;
    o[3] = c01 * id; o[4] = (m[0] * m[8] - m[2] * m[6]) * id; o[5] = (m[2] * m[3] - m[0] * m[5]) * id;
    o[6] = c02 * id; o[7] = (m[1] * m[6] - m[0] * m[7]) * id; o[8] = (m[0] * m[4] - m[1] * m[3]) * id;
}
static void inv33_r(const real *m, real *o) {
    real c00 = m[4] * m[8] - m[5] * m[7], c01 = m[5] * m[6] - m[3] * m[8], c02 = m[3] * m[7] - m[4] * m[6];
    real det = m[0] * c00 + m[1] * c01 + m[2] * c02;
    real id = (real)1 / det;
    o[0] = c00 * id; o[1] = (m[2] * m[7] - m[1] * m[8]) * id; o[2] = (m[1] * m[5] - m[2] * m[4]) * id;
    o[3] = c01 * id; o[4] = (m[0] * m[8] - m[2] * m[6]) * id; o[5] = (m[2] * m[3] - m[0] * m[5]) * id;
    o[6] = c02 * id; o[7] = (m[1] * m[6] - m[0] * m[7]) * id; o[8] = (m[0] * m[4] - m[1] * m[3]) * id;
}
static void mm33_d(const double *a, const double *b, double *o) {
    double t[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) t[i * 3 + j] = a[i * 3] * b[j] + a[i * 3 + 1] * b[3 + j] + a[i * 3 + 2] * b[6 + j];
    memcpy(o, t, sizeof(t));
}
static void mm33_r(const real *a, const real *b, real *o) {
    real t[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) t[i * 3 + j] = a[i * 3] * b[j] + a[i * 3 + 1] * b[3 + j] + a[i * 3 + 2] * b[6 + j];
    memcpy(o, t, sizeof(t));
}

/* OdometryProvider::rodrigues, src/odom/utils.h:16-52 (FP64). */
static void rodrigues(const double *src, double *R) {
    for (int k = 0; k < 9; ++k) R[k] = (k % 4 == 0) ? 1.0 : 0.0;
    double rx = src[0], ry = src[1], rz = src[2];
    double theta = sqrt(rx * rx + ry * ry + rz * rz);
    if (theta >= DBL_EPSILON) {
        double c = cos(theta), s = sin(theta), c1 = 1. - c, it = theta ? 1. / theta : 0.;
        rx *= it; ry *= it; rz *= it;
        const double I[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        double rrt[9] = {rx * rx, rx * ry, rx * rz, rx * ry, ry * ry, ry * rz, rx * rz, ry * rz, rz * rz};
        double rx_[9] = {0, -rz, ry, rz, 0, -rx, -ry, rx, 0};
        for (int k = 0; k < 9; ++k) R[k] = c * I[k] + c1 * rrt[k] + s * rx_[k];
    }
}

/* Polar factor of a 3x3 (Eigen 3.3 Transform::rotation()). */
static void polar33(const real *Min, real *Rout) {
    double X[9];
    for (int k = 0; k < 9; ++k) X[k] = (double)Min[k];
    for (int it = 0; it < 2; ++it) {
        double Xi[9];
        inv33_d(X, Xi);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) X[i * 3 + j] = 0.5 * (X[i * 3 + j] + Xi[j * 3 + i]);
    }
    for (int k = 0; k < 9; ++k) Rout[k] = (real)X[k];
}

/* 6x6 inverse by LU with partial pivoting (getCovariance,
 * src/odom/RGBDOdometryef.cpp:597-600). */
void ORC(inverse6)(const double *Ain, double *inv) {
    double A[36];
    memcpy(A, Ain, sizeof(A));
    for (int i = 0; i < 36; ++i) inv[i] = (i % 7 == 0) ? 1.0 : 0.0;
    for (int k = 0; k < 6; ++k) {
        int p = k;
        for (int i = k + 1; i < 6; ++i)
            if (fabs(A[i * 6 + k]) > fabs(A[p * 6 + k])) p = i;
        if (p != k)
            for (int j = 0; j < 6; ++j) {
                double t = A[k * 6 + j]; A[k * 6 + j] = A[p * 6 + j]; A[p * 6 + j] = t;
                t = inv[k * 6 + j]; inv[k * 6 + j] = inv[p * 6 + j]; inv[p * 6 + j] = t;
            }
        double d = A[k * 6 + k];
        for (int j = 0; j < 6; ++j) { A[k * 6 + j] /= d; inv[k * 6 + j] /= d; }
        for (int i = 0; i < 6; ++i)
            if (i != k) {
                double f = A[i * 6 + k];
                for (int j = 0; j < 6; ++j) { A[i * 6 + j] -= f * A[k * 6 + j]; inv[i * 6 + j] -= f * inv[k * 6 + j]; }
            }
    }
}

void ORC(ldlt_solve6)(const double *A, const double *b, double *x) { ldlt_solve_d(6, A, b, x); }
void ORC(rodrigues)(const double *src, double *R) { rodrigues(src, R); }

/* ------------------------------------------------------------------ */
/* Tracker (RGBDOdometryef, src/odom/RGBDOdometryef.cpp)                */
/* ------------------------------------------------------------------ */
typedef struct {
    int width, height;
    float cx, cy, fx, fy;
    real distThres, angleThres;
    int dims_w[NUM_PYRS], dims_h[NUM_PYRS];
    uint16_t *depth_tmp[NUM_PYRS];
    float *vmaps_tmp, *nmaps_tmp; /* RGBA32F copies (w*h*4) */
    real *vmaps_g_prev[NUM_PYRS], *nmaps_g_prev[NUM_PYRS];
    real *vmaps_curr[NUM_PYRS], *nmaps_curr[NUM_PYRS];
    real *lastDepth[NUM_PYRS], *nextDepth[NUM_PYRS];
    uint8_t *lastImage[NUM_PYRS], *nextImage[NUM_PYRS], *lastNextImage[NUM_PYRS];
    int16_t *dIdx[NUM_PYRS], *dIdy[NUM_PYRS];
    orc_dataterm *corres[NUM_PYRS];
    real *cloud[NUM_PYRS];
    orc_stats st;
    double lastA[36], lastb[6];
    int so3_iters, iters_run[NUM_PYRS];
    /* schedule override (levels > 0): the reference's per-level iteration
     * counts (src/odom/RGBDOdometryef.cpp:382-384) restricted to the first
     * `sched_levels` levels, each replaced by sched[l] where that is > 0 --
     * how a batched pair with fewer pyramid levels or a short schedule runs */
    int sched_levels, sched[NUM_PYRS];
    /* keep_deriv != 0: the tracking call uses the derivative images already
     * in dIdx/dIdy (set through odo_buffer) instead of computing them */
    int keep_deriv;
    /* the loop's discrete decisions (SO3 convergence / divergence tests, the
     * rgbOnly early exit), numbered in the order taken: the smallest relative
     * margin between the compared values and its index, and the index of a
     * decision to take the other way (-1: none) */
    int ndec, flip_decision, min_margin_index;
    double min_margin;
    int nhist;
    double hist[32][9];
} orc_odo;

/* CameraModel::operator()(level), src/sensors/Camera.h:14-18 */
static void intr_level(const orc_odo *o, int l, float *fx, float *fy, float *cx, float *cy) {
    int div = 1 << l;
    *fx = o->fx / (float)div; *fy = o->fy / (float)div;
    *cx = o->cx / (float)div; *cy = o->cy / (float)div;
}

/* RGBDOdometryef::RGBDOdometryef, src/odom/RGBDOdometryef.cpp:21-111 */
orc_odo *ORC(odo_create)(int width, int height, float cx, float cy, float fx, float fy, float distThresh,
                         float angleThresh) {
    orc_odo *o = (orc_odo *)calloc(1, sizeof(orc_odo));
    o->flip_decision = -1;
    o->width = width; o->height = height;
    o->cx = cx; o->cy = cy; o->fx = fx; o->fy = fy;
    o->distThres = distThresh; o->angleThres = angleThresh;
    for (int l = 0; l < NUM_PYRS; ++l) {
        int w = width >> l, h = height >> l;
        size_t n = (size_t)w * h;
        o->dims_w[l] = w; o->dims_h[l] = h;
        o->depth_tmp[l] = (uint16_t *)calloc(n, 2);
        o->vmaps_g_prev[l] = (real *)calloc(3 * n, sizeof(real));
        o->nmaps_g_prev[l] = (real *)calloc(3 * n, sizeof(real));
        o->vmaps_curr[l] = (real *)calloc(3 * n, sizeof(real));
        o->nmaps_curr[l] = (real *)calloc(3 * n, sizeof(real));
        o->lastDepth[l] = (real *)calloc(n, sizeof(real));
        o->nextDepth[l] = (real *)calloc(n, sizeof(real));
        o->lastImage[l] = (uint8_t *)calloc(n, 1);
        o->nextImage[l] = (uint8_t *)calloc(n, 1);
        o->lastNextImage[l] = (uint8_t *)calloc(n, 1);
        o->dIdx[l] = (int16_t *)calloc(n, 2);
        o->dIdy[l] = (int16_t *)calloc(n, 2);
        o->corres[l] = (orc_dataterm *)calloc(n, sizeof(orc_dataterm));
        o->cloud[l] = (real *)calloc(3 * n, sizeof(real));
    }
    o->vmaps_tmp = (float *)calloc((size_t)width * height * 4, sizeof(float));
    o->nmaps_tmp = (float *)calloc((size_t)width * height * 4, sizeof(float));
    o->st.lastICPCount = o->st.lastRGBCount = o->st.lastSO3Count = (float)(width * height);
    return o;
}

void ORC(odo_destroy)(orc_odo *o) {
    if (!o) return;
    for (int l = 0; l < NUM_PYRS; ++l) {
        free(o->depth_tmp[l]); free(o->vmaps_g_prev[l]); free(o->nmaps_g_prev[l]);
        free(o->vmaps_curr[l]); free(o->nmaps_curr[l]); free(o->lastDepth[l]); free(o->nextDepth[l]);
        free(o->lastImage[l]); free(o->nextImage[l]); free(o->lastNextImage[l]);
        free(o->dIdx[l]); free(o->dIdy[l]); free(o->corres[l]); free(o->cloud[l]);
    }
    free(o->vmaps_tmp); free(o->nmaps_tmp);
    free(o);
}

/* initICP(depth), src/odom/RGBDOdometryef.cpp:118-142 */
void ORC(odo_init_icp_depth)(orc_odo *o, const uint16_t *depth, float depthCutoff) {
    memcpy(o->depth_tmp[0], depth, (size_t)o->width * o->height * 2);
    for (int l = 1; l < NUM_PYRS; ++l)
        orc_pyr_down_depth(o->depth_tmp[l - 1], o->dims_w[l - 1], o->dims_h[l - 1], o->depth_tmp[l]);
    for (int l = 0; l < NUM_PYRS; ++l) {
        float fx, fy, cx, cy;
        intr_level(o, l, &fx, &fy, &cx, &cy);
        /* createVMap passes 1.f / fx (src/odom/utils.cu:147) */
        ORC(create_vmap)(o->depth_tmp[l], o->dims_w[l], o->dims_h[l], (real)1 / (real)fx, (real)1 / (real)fy,
                         (real)cx, (real)cy, (real)depthCutoff, o->vmaps_curr[l]);
        ORC(create_nmap)(o->vmaps_curr[l], o->dims_w[l], o->dims_h[l], o->nmaps_curr[l]);
    }
}

static void load_maps(orc_odo *o, const float *v4, const float *n4, real **vm, real **nm) {
    size_t n4sz = (size_t)o->width * o->height * 4;
    memcpy(o->vmaps_tmp, v4, n4sz * sizeof(float));
    memcpy(o->nmaps_tmp, n4, n4sz * sizeof(float));
    ORC(copy_maps)(o->vmaps_tmp, o->nmaps_tmp, o->width, o->height, vm[0], nm[0]);
    for (int l = 1; l < NUM_PYRS; ++l) {
        ORC(resize_map)(vm[l - 1], o->dims_w[l - 1], o->dims_h[l - 1], vm[l], 0);
        ORC(resize_map)(nm[l - 1], o->dims_w[l - 1], o->dims_h[l - 1], nm[l], 1);
    }
}

/* initICP(vertices, normals), src/odom/RGBDOdometryef.cpp:144-167 */
void ORC(odo_init_icp_maps)(orc_odo *o, const float *v4, const float *n4, float depthCutoff) {
    (void)depthCutoff;
    load_maps(o, v4, n4, o->vmaps_curr, o->nmaps_curr);
}

/* initICPModel, src/odom/RGBDOdometryef.cpp:169-206.  pose: row-major 4x4
 * camera-to-world of the model prediction. */
void ORC(odo_init_icp_model)(orc_odo *o, const float *v4, const float *n4, float depthCutoff, const float pose[16]) {
    (void)depthCutoff;
    load_maps(o, v4, n4, o->vmaps_g_prev, o->nmaps_g_prev);
    real R[9] = {pose[0], pose[1], pose[2], pose[4], pose[5], pose[6], pose[8], pose[9], pose[10]};
    real t[3] = {pose[3], pose[7], pose[11]};
    for (int l = 0; l < NUM_PYRS; ++l)
        ORC(transform_maps)(o->vmaps_g_prev[l], o->nmaps_g_prev[l], o->dims_w[l], o->dims_h[l], R, t,
                            o->vmaps_g_prev[l], o->nmaps_g_prev[l]);
}

/* populateRGBDData, src/odom/RGBDOdometryef.cpp:208-235 (depth comes from
 * the last RGBA32F vertex map handed to initICP(maps)/initICPModel). */
static void populate(orc_odo *o, const uint8_t *rgba, real **depths, uint8_t **images) {
    ORC(vertices_to_depth)(o->vmaps_tmp, o->width, o->height, (real)6.0f, depths[0]);
    for (int l = 0; l + 1 < NUM_PYRS; ++l)
        ORC(pyr_down_gauss_f)(depths[l], o->dims_w[l], o->dims_h[l], depths[l + 1]);
    orc_bgr_to_intensity(rgba, o->width, o->height, images[0], NULL);
    for (int l = 0; l + 1 < NUM_PYRS; ++l)
        orc_pyr_down_uchar_gauss(images[l], o->dims_w[l], o->dims_h[l], images[l + 1], NULL);
}
void ORC(odo_init_rgb_model)(orc_odo *o, const uint8_t *rgba) { populate(o, rgba, o->lastDepth, o->lastImage); }
void ORC(odo_init_rgb)(orc_odo *o, const uint8_t *rgba) { populate(o, rgba, o->nextDepth, o->nextImage); }

/* initFirstRGB, src/odom/RGBDOdometryef.cpp:249-265 */
void ORC(odo_init_first_rgb)(orc_odo *o, const uint8_t *rgba) {
    orc_bgr_to_intensity(rgba, o->width, o->height, o->lastNextImage[0], NULL);
    for (int l = 0; l + 1 < NUM_PYRS; ++l)
        orc_pyr_down_uchar_gauss(o->lastNextImage[l], o->dims_w[l], o->dims_h[l], o->lastNextImage[l + 1], NULL);
}

static void unpack29(const double *h, real *A, real *b) {
    int shift = 0;
    for (int i = 0; i < 6; ++i)
        for (int j = i; j < 7; ++j) {
            real v = (real)h[shift++];
            if (j == 6) b[i] = v;
            else A[j * 6 + i] = A[i * 6 + j] = v;
        }
}

/* One loop decision `result` from comparing a with b: records its margin,
 * and reverses it when it is the decision chosen to be flipped. */
static int loop_decision(orc_odo *o, int result, double a, double b) {
    const double s = fabs(a) > fabs(b) ? fabs(a) : fabs(b);
    const double m = s > 0 ? fabs(a - b) / s : 0.0;
    const int k = o->ndec++;
    if (m < o->min_margin) { o->min_margin = m; o->min_margin_index = k; }
    return k == o->flip_decision ? !result : result;
}

/* getIncrementalTransformation, src/odom/RGBDOdometryef.cpp:267-595.
 * trans/rot: in = previous pose, out = new pose (rot row-major). */
void ORC(odo_track)(orc_odo *o, real trans[3], real rot[9], int rgbOnly, float icpWeight, int pyramid,
                    int fastOdom, int so3) {
    const int icp = !rgbOnly && icpWeight > 0;
    const int rgb = rgbOnly || icpWeight < 100;
    o->ndec = 0;
    o->min_margin = HUGE_VAL;
    o->min_margin_index = -1;
    real Rprev[9], tprev[3], Rcurr[9], tcurr[3];
    memcpy(Rprev, rot, sizeof(Rprev)); memcpy(tprev, trans, sizeof(tprev));
    memcpy(Rcurr, Rprev, sizeof(Rcurr)); memcpy(tcurr, tprev, sizeof(tcurr));
    const real sobelScale = (real)(1.0 / pow(2.0, 3));
    const real maxDepthDeltaRGB = (real)0.07f;
    const float minGrad[3] = {5, 3, 1};

    if (rgb && !o->keep_deriv)
        for (int l = 0; l < NUM_PYRS; ++l)
            orc_derivatives(o->nextImage[l], o->dims_w[l], o->dims_h[l], o->dIdx[l], o->dIdy[l], NULL);

    double resultR[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    o->so3_iters = 0;
    if (so3) {
        const int L = 2;
        float fx, fy, cx, cy;
        intr_level(o, L, &fx, &fy, &cx, &cy);
        real R_lr[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        double K[9] = {fx, 0, cx, 0, fy, cy, 0, 0, 1}, Kinv[9];
        inv33_d(K, Kinv);
        float lastError = FLT_MAX / 2, lastCount = FLT_MAX / 2;
        double lastResultR[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        for (int i = 0; i < 10; ++i) {
            double Hd[9], KR[9];
            mm33_d(K, resultR, KR);
            mm33_d(KR, Kinv, Hd);
            real H[9], ki[9], krlr[9];
            for (int k = 0; k < 9; ++k) { H[k] = (real)Hd[k]; ki[k] = (real)Kinv[k]; krlr[k] = (real)KR[k]; }
            double out11[11];
            ORC(so3_step)(o->lastNextImage[L], o->nextImage[L], o->dims_w[L], o->dims_h[L], H, ki, krlr, out11);
            o->so3_iters++;
            real jtj[9], jtr[3], res[2];
            {
                int shift = 0;
                for (int a = 0; a < 3; ++a)
                    for (int b = a; b < 4; ++b) {
                        real v = (real)out11[shift++];
                        if (b == 3) jtr[a] = v;
                        else jtj[b * 3 + a] = jtj[a * 3 + b] = v;
                    }
                res[0] = (real)out11[9]; res[1] = (real)out11[10];
            }
            o->st.lastSO3Error = (float)(SQRT(res[0]) / res[1]);
            o->st.lastSO3Count = (float)res[1];
            const int lower = loop_decision(o, o->st.lastSO3Error < lastError, o->st.lastSO3Error, lastError);
            if (lower && lastCount == o->st.lastSO3Count) break;
            else if (loop_decision(o, (double)o->st.lastSO3Error > (double)lastError + 0.001,
                                   (double)o->st.lastSO3Error, (double)lastError + 0.001)) {
                o->st.lastSO3Error = lastError; o->st.lastSO3Count = lastCount;
                memcpy(resultR, lastResultR, sizeof(resultR));
                break;
            }
            lastError = o->st.lastSO3Error; lastCount = o->st.lastSO3Count;
            memcpy(lastResultR, resultR, sizeof(resultR));
            double dd[3];
#ifdef ORC_REAL_F64
            {
                double A[9], bb[3];
                for (int k = 0; k < 9; ++k) A[k] = jtj[k];
                for (int k = 0; k < 3; ++k) bb[k] = jtr[k];
                ldlt_solve_d(3, A, bb, dd);
            }
#else
            {
                float delta[3];
                ldlt_solve_f(3, jtj, jtr, delta);
                for (int k = 0; k < 3; ++k) dd[k] = (double)delta[k];
            }
#endif
            double rotUpdate[9];
            rodrigues(dd, rotUpdate);
            real ru[9];
            for (int k = 0; k < 9; ++k) ru[k] = (real)rotUpdate[k];
            mm33_r(ru, R_lr, R_lr);
            for (int k = 0; k < 9; ++k) resultR[k] = (double)R_lr[k];
        }
    }

    int iterations[3] = {fastOdom ? 3 : 10, pyramid ? 5 : 0, pyramid ? 4 : 0};
    if (o->sched_levels > 0)
        for (int l = 0; l < NUM_PYRS; ++l)
            iterations[l] = l < o->sched_levels ? (o->sched[l] > 0 ? o->sched[l] : iterations[l]) : 0;
    o->nhist = 0;
    real Rprev_inv[9];
    inv33_r(Rprev, Rprev_inv);
    double resultRt[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    if (so3)
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) resultRt[a * 4 + b] = resultR[a * 3 + b];

    for (int l = NUM_PYRS - 1; l >= 0; --l) {
        float fx, fy, cx, cy;
        intr_level(o, l, &fx, &fy, &cx, &cy);
        const int w = o->dims_w[l], h = o->dims_h[l];
        o->iters_run[l] = 0;
        if (rgb)
            ORC(project_cloud)(o->lastDepth[l], w, h, (real)(1.0f / fx), (real)(1.0f / fy), (real)cx, (real)cy,
                               o->cloud[l]);
        double K[9] = {fx, 0, cx, 0, fy, cy, 0, 0, 1}, Kinv[9];
        inv33_d(K, Kinv);
        o->st.lastRGBError = FLT_MAX;
        for (int j = 0; j < iterations[l]; ++j) {
            /* Rt = resultRt^-1 (rigid) */
            double Rt_R[9], Rt_t[3];
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) Rt_R[a * 3 + b] = resultRt[b * 4 + a];
            for (int a = 0; a < 3; ++a)
                Rt_t[a] = -(Rt_R[a * 3] * resultRt[3] + Rt_R[a * 3 + 1] * resultRt[7] + Rt_R[a * 3 + 2] * resultRt[11]);
            double KR[9], KRKi[9];
            mm33_d(K, Rt_R, KR);
            mm33_d(KR, Kinv, KRKi);
            real krkInv[9], kt[3];
            for (int k = 0; k < 9; ++k) krkInv[k] = (real)KRKi[k];
            for (int a = 0; a < 3; ++a) kt[a] = (real)(K[a * 3] * Rt_t[0] + K[a * 3 + 1] * Rt_t[1] + K[a * 3 + 2] * Rt_t[2]);

            int sigma = 0, rgbSize = 0;
            if (rgb) {
                int32_t o2[2];
                real minScale = (real)(pow(minGrad[l], 2.0) / pow((double)sobelScale, 2.0));
                ORC(rgb_residual)(minScale, o->dIdx[l], o->dIdy[l], o->lastDepth[l], o->nextDepth[l],
                                  o->lastImage[l], o->nextImage[l], w, h, maxDepthDeltaRGB, kt, krkInv,
                                  o->corres[l], o2, NULL);
                rgbSize = o2[0]; sigma = o2[1];
            }
            /* src/odom/RGBDOdometryef.cpp:457-458, operator precedence kept */
            float sigmaVal = (float)sqrt((double)(((float)sigma / rgbSize == 0) ? 1 : rgbSize));
            float rgbError = (float)(sqrt((double)sigma) / (rgbSize == 0 ? 1 : rgbSize));
            if (rgbOnly && loop_decision(o, rgbError > o->st.lastRGBError, rgbError, o->st.lastRGBError)) break;
            o->st.lastRGBError = rgbError;
            o->st.lastRGBCount = (float)rgbSize;
            if (rgbOnly) sigmaVal = -1;

            double icp29[29] = {0}, rgb29[29] = {0};
            if (icp) {
                ORC(icp_step)(Rcurr, tcurr, o->vmaps_curr[l], o->nmaps_curr[l], Rprev_inv, tprev, (real)fx, (real)fy,
                              (real)cx, (real)cy, o->vmaps_g_prev[l], o->nmaps_g_prev[l], o->distThres,
                              o->angleThres, w, h, icp29, NULL, NULL);
                o->st.lastICPError = (float)(SQRT((real)icp29[27]) / (real)icp29[28]);
                o->st.lastICPCount = (float)icp29[28];
            }
            if (rgb)
                ORC(rgb_step)(o->corres[l], (real)sigmaVal, o->cloud[l], (real)fx, (real)fy, o->dIdx[l], o->dIdy[l],
                              sobelScale, w, h, rgb29);
            real Ai[36] = {0}, bi[6] = {0}, Ar[36] = {0}, br[6] = {0};
            unpack29(icp29, Ai, bi);
            unpack29(rgb29, Ar, br);
            double w_ = icpWeight;
            for (int k = 0; k < 36; ++k) {
                if (icp && rgb) o->lastA[k] = (double)Ar[k] + w_ * w_ * (double)Ai[k];
                else if (icp) o->lastA[k] = (double)Ai[k];
                else o->lastA[k] = (double)Ar[k];
            }
            for (int k = 0; k < 6; ++k) {
                if (icp && rgb) o->lastb[k] = (double)br[k] + w_ * (double)bi[k];
                else if (icp) o->lastb[k] = (double)bi[k];
                else o->lastb[k] = (double)br[k];
            }
            double result[6];
            ldlt_solve_d(6, o->lastA, o->lastb, result);
            if (o->nhist < 32) {
                double *hr = o->hist[o->nhist++];
                hr[0] = icp29[28];
                hr[1] = o->st.lastRGBCount;
                hr[2] = sigmaVal;
                for (int k = 0; k < 6; ++k) hr[3 + k] = result[k];
            }

            /* computeUpdateSE3, src/odom/utils.h:54-74 */
            double Rinc[9];
            rodrigues(result + 3, Rinc);
            double Rt4[16] = {Rinc[0], Rinc[1], Rinc[2], result[0], Rinc[3], Rinc[4], Rinc[5], result[1],
                              Rinc[6], Rinc[7], Rinc[8], result[2], 0, 0, 0, 1};
            double nr[16];
            for (int a = 0; a < 4; ++a)
                for (int b = 0; b < 4; ++b) {
                    double s = 0;
                    for (int k = 0; k < 4; ++k) s += Rt4[a * 4 + k] * resultRt[k * 4 + b];
                    nr[a * 4 + b] = s;
                }
            memcpy(resultRt, nr, sizeof(nr));
            /* rgbOdom: Isometry3f(rotation, translation) in the working precision */
            real oR[9], ot[3];
            for (int a = 0; a < 3; ++a) {
                for (int b = 0; b < 3; ++b) oR[a * 3 + b] = (real)resultRt[a * 4 + b];
                ot[a] = (real)resultRt[a * 4 + 3];
            }
            /* currentT = [Rprev|tprev] * rgbOdom^-1 */
            real iR[9], it[3];
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) iR[a * 3 + b] = oR[b * 3 + a];
            for (int a = 0; a < 3; ++a) it[a] = -(iR[a * 3] * ot[0] + iR[a * 3 + 1] * ot[1] + iR[a * 3 + 2] * ot[2]);
            real cR[9], ct[3];
            mm33_r(Rprev, iR, cR);
            for (int a = 0; a < 3; ++a)
                ct[a] = (Rprev[a * 3] * it[0] + Rprev[a * 3 + 1] * it[1] + Rprev[a * 3 + 2] * it[2]) + tprev[a];
            memcpy(tcurr, ct, sizeof(ct));
            polar33(cR, Rcurr);
            o->iters_run[l]++;
        }
    }
    if (rgb) {
        real dx = tcurr[0] - tprev[0], dy = tcurr[1] - tprev[1], dz = tcurr[2] - tprev[2];
        if ((double)SQRT(dx * dx + dy * dy + dz * dz) > 0.3) {
            memcpy(Rcurr, Rprev, sizeof(Rcurr));
            memcpy(tcurr, tprev, sizeof(tcurr));
        }
    }
    if (so3)
        for (int l = 0; l < NUM_PYRS; ++l) {
            uint8_t *t = o->lastNextImage[l]; o->lastNextImage[l] = o->nextImage[l]; o->nextImage[l] = t;
        }
    memcpy(trans, tcurr, sizeof(tcurr));
    memcpy(rot, Rcurr, sizeof(Rcurr));
    memcpy(o->st.lastA, o->lastA, sizeof(o->lastA));
    memcpy(o->st.lastb, o->lastb, sizeof(o->lastb));
}

/* Schedule override of the tracking loop (levels <= 0 restores the
 * reference's schedule); iters may be NULL (the reference's counts). */
void ORC(odo_set_schedule)(orc_odo *o, int levels, const int iters[3]) {
    o->sched_levels = levels > NUM_PYRS ? NUM_PYRS : levels;
    for (int l = 0; l < NUM_PYRS; ++l) o->sched[l] = iters ? iters[l] : 0;
}

void ORC(odo_set_keep_derivatives)(orc_odo *o, int keep) { o->keep_deriv = keep; }
void ORC(odo_set_flip_decision)(orc_odo *o, int index) { o->flip_decision = index; }
/* smallest relative margin of the last tracking call's loop decisions, and
 * its index (-1: no decision was taken) */
double ORC(odo_decision_margin)(orc_odo *o, int *index) {
    *index = o->min_margin_index;
    return o->min_margin;
}

/* getCovariance, src/odom/RGBDOdometryef.cpp:597-600 */
void ORC(odo_covariance)(orc_odo *o, double out[36]) { ORC(inverse6)(o->lastA, out); }
void ORC(odo_stats)(orc_odo *o, orc_stats *s) { *s = o->st; }
void ORC(odo_iters)(orc_odo *o, int out[4]) {
    out[0] = o->so3_iters; out[1] = o->iters_run[0]; out[2] = o->iters_run[1]; out[3] = o->iters_run[2];
}

/* Buffer access for the tests (which: 0 depth_tmp u16, 1 vmap_curr, 2 nmap_curr,
 * 3 vmap_g_prev, 4 nmap_g_prev, 5 lastDepth, 6 nextDepth, 7 lastImage u8,
 * 8 nextImage u8, 9 lastNextImage u8, 10 dIdx s16, 11 dIdy s16, 12 corres,
 * 13 cloud). */
void *ORC(odo_buffer)(orc_odo *o, int which, int level) {
    switch (which) {
    case 0: return o->depth_tmp[level];
    case 1: return o->vmaps_curr[level];
    case 2: return o->nmaps_curr[level];
    case 3: return o->vmaps_g_prev[level];
    case 4: return o->nmaps_g_prev[level];
    case 5: return o->lastDepth[level];
    case 6: return o->nextDepth[level];
    case 7: return o->lastImage[level];
    case 8: return o->nextImage[level];
    case 9: return o->lastNextImage[level];
    case 10: return o->dIdx[level];
    case 11: return o->dIdy[level];
    case 12: return o->corres[level];
    case 13: return o->cloud[level];
    }
    return NULL;
}
int ORC(real_size)(void) { return (int)sizeof(real); }
int ORC(odo_history)(orc_odo *o, double *out, int max_rows) {
    int n = o->nhist < max_rows ? o->nhist : max_rows;
    memcpy(out, o->hist, sizeof(double) * 9 * (size_t)n);
    return n;
}

#endif /* ORC_REAL_F32 || ORC_REAL_F64 */
