/* CPU oracle of the warm-start network (TEST INFRASTRUCTURE ONLY: used by
 * tests/ to check the GPU network's forward pass and gradients; never part of
 * the product path).
 *
 * The network has no counterpart in the reference; this file restates the
 * architecture and the training loss of the GPU implementation in plain C
 * with FP64 accumulation:
 *   input [B][120][160][8] FP16 NHWC, six 3x3 / stride 2 / pad 1 convolutions
 *   8->32->64->128->128->128->128 with ReLU,
 *   fc 768->768 ReLU, fc 768->6,
 *   loss = mean_b e^T M e, e = out - label, M a symmetric 6x6 metric.
 * rounding = 1 reproduces the GPU's rounding points (FP16 input and FP16
 * first-layer weights in the forward pass, BF16 weights, activations and
 * activation gradients elsewhere -- the first layer's weight gradient uses
 * the input rounded to BF16 --, FP32 sums, FP32 output / loss gradient);
 * rounding = 0 keeps everything in FP64 (for the finite-difference
 * check of the backward formulas).  Only the order of the FP32 accumulations
 * inside the tensor cores is not reproduced (sums are exact in FP64 here). */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define IN_H 120
#define IN_W 160
#define IN_C 8
#define NCONV 6
#define NLAYERS 8
#define FLAT 768
#define HIDDEN 768
#define NOUT 6

static const int CIN[NCONV] = {8, 32, 64, 128, 128, 128};
static const int COUT[NCONV] = {32, 64, 128, 128, 128, 128};
static const int HH[NCONV + 1] = {120, 60, 30, 15, 8, 4, 2};
static const int WW[NCONV + 1] = {160, 80, 40, 20, 10, 5, 3};
static const int KS[NCONV] = {3, 3, 3, 3, 3, 3};

static int w_rows(int l) { return l < NCONV ? COUT[l] : (l == NCONV ? HIDDEN : NOUT); }
static int w_cols(int l) { return l < NCONV ? KS[l] * KS[l] * CIN[l] : (l == NCONV ? FLAT : HIDDEN); }

/* parameter offsets: W then b per layer, each layer start rounded to 8 floats */
void cnn_layout(size_t w[NLAYERS], size_t b[NLAYERS], size_t *total) {
    size_t o = 0;
    for (int l = 0; l < NLAYERS; ++l) {
        w[l] = o;
        o += (size_t)w_rows(l) * w_cols(l);
        b[l] = o;
        o += (size_t)w_rows(l);
        o = (o + 7) & ~(size_t)7;
    }
    *total = o;
}

static int g_round = 1;
static double rf(double x) { return g_round ? (double)(float)x : x; }
static double rb(double x) {
    if (!g_round) return x;
    float f = (float)x;
    uint32_t u;
    memcpy(&u, &f, 4);
    if ((u & 0x7F800000u) != 0x7F800000u) u += 0x7FFFu + ((u >> 16) & 1u);
    u &= 0xFFFF0000u;
    memcpy(&f, &u, 4);
    return (double)f;
}
/* FP32 value -> nearest FP16 (ties to even, subnormals kept), as double */
static double rh(double x) {
    if (!g_round) return x;
    float f = (float)x;
    const double a = fabs((double)f);
    if (!(a < 65520.0)) return f > 0 ? INFINITY : -INFINITY;
    int e;
    frexp(a, &e);
    const double q = a >= ldexp(1.0, -14) ? ldexp(1.0, e - 11) : ldexp(1.0, -24);
    const double r = nearbyint(a / q) * q;
    return f < 0 ? -r : r;
}
static double half_to_double(uint16_t h) {
    const int s = (h >> 15) & 1, e = (h >> 10) & 31, m = h & 1023;
    double v;
    if (e == 0) v = ldexp((double)m, -24);
    else if (e == 31) v = m ? NAN : INFINITY;
    else v = ldexp((double)(m | 1024), e - 25);
    return s ? -v : v;
}

/* im2col source index of output position m (over B x Ho x Wo) and column k */
static long conv_src(int l, int B, int m, int k) {
    const int C = CIN[l], H = HH[l], W = WW[l], Ho = HH[l + 1], Wo = WW[l + 1];
    (void)B;
    const int ks = KS[l], pad = (ks - 1) / 2;
    const int tap = k / C, ci = k % C, ky = tap / ks, kx = tap % ks;
    const int ox = m % Wo, t = m / Wo, oy = t % Ho, b = t / Ho;
    const int iy = 2 * oy - pad + ky, ix = 2 * ox - pad + kx;
    if (iy < 0 || iy >= H || ix < 0 || ix >= W) return -1;
    return (((long)b * H + iy) * W + ix) * C + ci;
}

/* Forward, loss and (grad != NULL) backward.  params: FP32 parameter values
 * (as doubles); labels [B][6]; out [B][6]; grad in the parameter layout. */
int cnn_oracle_run(const double *params, const uint16_t *input, const double *labels, const double *metric, int B,
                   int rounding, double *out, double *loss, double *grad) {
    g_round = rounding;
    size_t wo[NLAYERS], bo[NLAYERS], total;
    cnn_layout(wo, bo, &total);
    double *w = malloc(total * sizeof(double));
    for (size_t i = 0; i < total; ++i) w[i] = rb(params[i]); /* BF16 weights (biases use params directly) */
    double *act[NCONV + 1];
    const size_t nin = (size_t)B * IN_H * IN_W * IN_C;
    act[0] = malloc(nin * sizeof(double));      /* BF16 view of the input (first-layer weight gradient) */
    double *in16 = malloc(nin * sizeof(double)); /* the FP16 input (first-layer forward product) */
    for (size_t i = 0; i < nin; ++i) {
        in16[i] = half_to_double(input[i]);
        act[0][i] = rb(in16[i]);
    }
    for (size_t i = 0; i < (size_t)COUT[0] * w_cols(0); ++i) w[wo[0] + i] = rh(params[wo[0] + i]);
    /* convolutions */
    for (int l = 0; l < NCONV; ++l) {
        const int M = B * HH[l + 1] * WW[l + 1], N = COUT[l], K = w_cols(l);
        act[l + 1] = malloc((size_t)M * N * sizeof(double));
        double *y = act[l + 1];
        const double *x = l == 0 ? in16 : act[l];
#pragma omp parallel for schedule(static)
        for (int m = 0; m < M; ++m)
            for (int n = 0; n < N; ++n) {
                double acc = 0;
                for (int k = 0; k < K; ++k) {
                    const long s = conv_src(l, B, m, k);
                    if (s >= 0) acc += x[s] * w[wo[l] + (size_t)n * K + k];
                }
                double f = rf(rf(acc) + rf(params[bo[l] + n]));
                y[(size_t)m * N + n] = rb(f > 0 ? f : 0);
            }
    }
    /* fc1 (ReLU) and fc2 */
    double *hid = malloc((size_t)B * HIDDEN * sizeof(double));
    const double *a6 = act[NCONV];
#pragma omp parallel for schedule(static)
    for (int bb = 0; bb < B; ++bb)
        for (int o = 0; o < HIDDEN; ++o) {
            double acc = 0;
            for (int i = 0; i < FLAT; ++i) acc += a6[(size_t)bb * FLAT + i] * w[wo[6] + (size_t)o * FLAT + i];
            double f = rf(rf(acc) + rf(params[bo[6] + o]));
            hid[(size_t)bb * HIDDEN + o] = rb(f > 0 ? f : 0);
        }
    for (int bb = 0; bb < B; ++bb)
        for (int o = 0; o < NOUT; ++o) {
            double acc = 0;
            for (int i = 0; i < HIDDEN; ++i) acc += hid[(size_t)bb * HIDDEN + i] * w[wo[7] + (size_t)o * HIDDEN + i];
            out[bb * NOUT + o] = rf(rf(acc) + rf(params[bo[7] + o]));
        }
    /* loss and its gradient */
    double *dout = malloc((size_t)B * NOUT * sizeof(double));
    double L = 0;
    for (int bb = 0; bb < B; ++bb) {
        double e[NOUT];
        for (int i = 0; i < NOUT; ++i) e[i] = rf(out[bb * NOUT + i] - labels[bb * NOUT + i]);
        for (int i = 0; i < NOUT; ++i) {
            double me = 0;
            for (int j = 0; j < NOUT; ++j) me = rf(me + rf(metric[i * NOUT + j]) * e[j]);
            L += e[i] * me;
            dout[bb * NOUT + i] = rf(rf(2.0 * me) / (double)B);
        }
    }
    *loss = L / B;
    if (!grad) goto done;
    memset(grad, 0, total * sizeof(double));
    {
        /* fc2 */
        for (int n = 0; n < NOUT; ++n) {
            double sb = 0;
            for (int bb = 0; bb < B; ++bb) sb += dout[bb * NOUT + n];
            grad[bo[7] + n] = rf(sb);
            for (int i = 0; i < HIDDEN; ++i) {
                double acc = 0;
                for (int bb = 0; bb < B; ++bb) acc += rb(dout[bb * NOUT + n]) * hid[(size_t)bb * HIDDEN + i];
                grad[wo[7] + (size_t)n * HIDDEN + i] = rf(acc);
            }
        }
        double *dh = malloc((size_t)B * HIDDEN * sizeof(double));
        for (int bb = 0; bb < B; ++bb)
            for (int i = 0; i < HIDDEN; ++i) {
                double acc = 0;
                for (int n = 0; n < NOUT; ++n) acc += rb(dout[bb * NOUT + n]) * w[wo[7] + (size_t)n * HIDDEN + i];
                dh[(size_t)bb * HIDDEN + i] = hid[(size_t)bb * HIDDEN + i] > 0 ? rb(rf(acc)) : 0;
            }
        /* fc1 */
#pragma omp parallel for schedule(static)
        for (int o = 0; o < HIDDEN; ++o) {
            double sb = 0;
            for (int bb = 0; bb < B; ++bb) sb += dh[(size_t)bb * HIDDEN + o];
            grad[bo[6] + o] = rf(sb);
            for (int i = 0; i < FLAT; ++i) {
                double acc = 0;
                for (int bb = 0; bb < B; ++bb) acc += dh[(size_t)bb * HIDDEN + o] * a6[(size_t)bb * FLAT + i];
                grad[wo[6] + (size_t)o * FLAT + i] = rf(acc);
            }
        }
        double *dpre = malloc((size_t)B * FLAT * sizeof(double));
#pragma omp parallel for schedule(static)
        for (int bb = 0; bb < B; ++bb)
            for (int i = 0; i < FLAT; ++i) {
                double acc = 0;
                for (int o = 0; o < HIDDEN; ++o) acc += dh[(size_t)bb * HIDDEN + o] * w[wo[6] + (size_t)o * FLAT + i];
                dpre[(size_t)bb * FLAT + i] = a6[(size_t)bb * FLAT + i] > 0 ? rb(rf(acc)) : 0;
            }
        free(dh);
        /* convolutions, last to first; dpre = gradient at conv l's pre-activation */
        for (int l = NCONV - 1; l >= 0; --l) {
            const int M = B * HH[l + 1] * WW[l + 1], Co = COUT[l], K = w_cols(l);
            const double *x = act[l];
#pragma omp parallel for schedule(static)
            for (int co = 0; co < Co; ++co) {
                double sb = 0;
                for (int m = 0; m < M; ++m) sb += dpre[(size_t)m * Co + co];
                grad[bo[l] + co] = rf(sb);
                for (int k = 0; k < K; ++k) {
                    double acc = 0;
                    for (int m = 0; m < M; ++m) {
                        const long s = conv_src(l, B, m, k);
                        if (s >= 0) acc += dpre[(size_t)m * Co + co] * x[s];
                    }
                    grad[wo[l] + (size_t)co * K + k] = rf(acc);
                }
            }
            if (l == 0) break;
            /* dcol, then col2im in the tap order (ky, kx) and the ReLU mask */
            double *dcol = malloc((size_t)M * K * sizeof(double));
#pragma omp parallel for schedule(static)
            for (int m = 0; m < M; ++m)
                for (int k = 0; k < K; ++k) {
                    double acc = 0;
                    for (int co = 0; co < Co; ++co) acc += dpre[(size_t)m * Co + co] * w[wo[l] + (size_t)co * K + k];
                    dcol[(size_t)m * K + k] = rf(acc);
                }
            const int H = HH[l], W = WW[l], C = CIN[l], Ho = HH[l + 1], Wo = WW[l + 1];
            double *dnew = malloc((size_t)B * H * W * C * sizeof(double));
#pragma omp parallel for schedule(static)
            for (long i = 0; i < (long)B * H * W * C; ++i) {
                const int ci = (int)(i % C);
                long t = i / C;
                const int ix = (int)(t % W);
                t /= W;
                const int iy = (int)(t % H), bb = (int)(t / H);
                double s = 0;
                for (int ky = 0; ky < 3; ++ky) {
                    const int ty = iy + 1 - ky;
                    if (ty < 0 || (ty & 1) || (ty >> 1) >= Ho) continue;
                    for (int kx = 0; kx < 3; ++kx) {
                        const int tx = ix + 1 - kx;
                        if (tx < 0 || (tx & 1) || (tx >> 1) >= Wo) continue;
                        s = rf(s + dcol[(((size_t)bb * Ho + (ty >> 1)) * Wo + (tx >> 1)) * K + (ky * 3 + kx) * C + ci]);
                    }
                }
                dnew[i] = x[i] > 0 ? rb(s) : 0;
            }
            free(dcol);
            free(dpre);
            dpre = dnew;
        }
        free(dpre);
    }
done:
    for (int l = 0; l <= NCONV; ++l) free(act[l]);
    free(in16);
    free(hid);
    free(dout);
    free(w);
    return 0;
}
