// Synthetic RGB-D scene generator: ray-cast box rooms / corridors with
// spheres and a seeded Perlin solid texture.
//
// Stands in for the reference's inputs (uint16 depth in mm + RGBA8 frames,
// src/inputs/*) and for its GL model prediction (RGBA32F camera-frame vertex
// and normal maps, src/gl/FillIn.cpp:22-42), which need a graphics stack.
// Deterministic for a given seed on any host (counter-based RNG, no libc
// rand); OpenMP over rows.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>

#include "synth_common.h"

namespace {

using synth::Rng;
using synth::splitmix64;
using synth::u01;

// Improved Perlin gradient noise (Perlin 2002) with a seeded permutation.
struct Perlin {
    int p[512];
    explicit Perlin(uint64_t seed) { synth::perlin_perm(seed, p); }
    static double fade(double t) { return t * t * t * (t * (t * 6 - 15) + 10); }
    static double lerp(double t, double a, double b) { return a + t * (b - a); }
    static double grad(int h, double x, double y, double z) {
        h &= 15;
        double u = h < 8 ? x : y, v = h < 4 ? y : (h == 12 || h == 14 ? x : z);
        return ((h & 1) ? -u : u) + ((h & 2) ? -v : v);
    }
    double operator()(double x, double y, double z) const {
        double fx = std::floor(x), fy = std::floor(y), fz = std::floor(z);
        int X = (int)fx & 255, Y = (int)fy & 255, Z = (int)fz & 255;
        x -= fx; y -= fy; z -= fz;
        double u = fade(x), v = fade(y), w = fade(z);
        int A = p[X] + Y, AA = p[A] + Z, AB = p[A + 1] + Z, B = p[X + 1] + Y, BA = p[B] + Z, BB = p[B + 1] + Z;
        return lerp(w,
                    lerp(v, lerp(u, grad(p[AA], x, y, z), grad(p[BA], x - 1, y, z)),
                         lerp(u, grad(p[AB], x, y - 1, z), grad(p[BB], x - 1, y - 1, z))),
                    lerp(v, lerp(u, grad(p[AA + 1], x, y, z - 1), grad(p[BA + 1], x - 1, y, z - 1)),
                         lerp(u, grad(p[AB + 1], x, y - 1, z - 1), grad(p[BB + 1], x - 1, y - 1, z - 1))));
    }
};

}  // namespace

extern "C" {

// A 6x4x3 m box room (x in [-3,3], y in [-1.5,1.5] (y down), z in [-2,2])
// with `nspheres` spheres of radius U(0.1, 0.5) kept clear of a 0.8 m ball
// around the origin, where cameras are placed.
int synth_make_room(uint64_t seed, int nspheres, synth_scene *s) {
    if (!s || nspheres < 0 || nspheres > SYNTH_MAX_SPH) return -1;
    std::memset(s, 0, sizeof(*s));
    Rng r(seed);
    const float bmin[3] = {-3.f, -1.5f, -2.f}, bmax[3] = {3.f, 1.5f, 2.f};
    for (int k = 0; k < 3; ++k) { s->bmin[k] = bmin[k]; s->bmax[k] = bmax[k]; }
    for (int f = 0; f < 6; ++f)
        for (int c = 0; c < 3; ++c) s->wall_col[f][c] = (float)r.uni(0.35, 0.95);
    int n = 0, tries = 0;
    while (n < nspheres && tries < 100000) {
        ++tries;
        float rad = (float)r.uni(0.1, 0.5);
        float c[3];
        for (int k = 0; k < 3; ++k) c[k] = (float)r.uni(bmin[k] + rad, bmax[k] - rad);
        float d = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
        if (d < rad + 0.8f) continue;
        for (int k = 0; k < 3; ++k) s->sph[n][k] = c[k];
        s->sph[n][3] = rad;
        for (int k = 0; k < 3; ++k) s->sph_col[n][k] = (float)r.uni(0.2, 1.0);
        ++n;
    }
    s->nsph = n;
    s->tex_freq = 4.0f;
    s->tex_amp = 0.85f;
    s->tex_seed = splitmix64(seed ^ 0x7e47u);
    return n == nspheres ? 0 : -2;
}

// A low-texture corridor 2 m wide (x), 3 m high (y, down) and 20 m long (z),
// with small clutter spheres against the side walls (cluttered fraction of
// the image is controlled by `nclutter`).
int synth_make_corridor(uint64_t seed, int nclutter, synth_scene *s) {
    if (!s || nclutter < 0 || nclutter > SYNTH_MAX_SPH) return -1;
    std::memset(s, 0, sizeof(*s));
    Rng r(seed);
    const float bmin[3] = {-1.f, -1.5f, -10.f}, bmax[3] = {1.f, 1.5f, 10.f};
    for (int k = 0; k < 3; ++k) { s->bmin[k] = bmin[k]; s->bmax[k] = bmax[k]; }
    for (int f = 0; f < 6; ++f)
        for (int c = 0; c < 3; ++c) s->wall_col[f][c] = (float)r.uni(0.55, 0.75);
    for (int n = 0; n < nclutter; ++n) {
        float rad = (float)r.uni(0.05, 0.15);
        int side = (r.uni() < 0.5) ? -1 : 1;
        s->sph[n][0] = side * (1.f - rad * 0.6f);
        s->sph[n][1] = (float)r.uni(-1.2, 1.2);
        s->sph[n][2] = (float)r.uni(-9.0, 9.0);
        s->sph[n][3] = rad;
        for (int k = 0; k < 3; ++k) s->sph_col[n][k] = (float)r.uni(0.3, 1.0);
    }
    s->nsph = nclutter;
    s->tex_freq = 1.5f;
    s->tex_amp = 0.12f;
    s->tex_seed = splitmix64(seed ^ 0xc0ffu);
    return 0;
}

// Ray-casts the scene from camera-to-world pose `pose_wc` (row-major 4x4;
// camera x right, y down, z forward) with a pinhole model.
//  depth_mm: uint16 depth in mm with Gaussian noise sigma = noise_k * z^2 (m),
//            a `dropout` fraction of zeros, and 0 outside [min_mm, max_mm];
//  rgba:     RGBA8 Perlin texture (A = 255);
//  vert4:    noise-free RGBA32F camera-frame vertices (w = 1), zero where no hit;
//  norm4:    RGBA32F camera-frame normals facing the camera (w = 1).
// Any output pointer may be NULL.
int synth_render(const synth_scene *s, const float pose_wc[16], int w, int h, float fx, float fy, float cx, float cy,
                 uint64_t noise_seed, float noise_k, float dropout, int min_mm, int max_mm, uint16_t *depth_mm,
                 uint8_t *rgba, float *vert4, float *norm4) {
    if (!s || !pose_wc || w <= 0 || h <= 0) return -1;
    Perlin perlin(s->tex_seed);
    double R[9], t[3];
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j) R[i * 3 + j] = pose_wc[i * 4 + j];
        t[i] = pose_wc[i * 4 + 3];
    }
#pragma omp parallel for schedule(dynamic, 8)
    for (int v = 0; v < h; ++v) {
        for (int u = 0; u < w; ++u) {
            const size_t pix = (size_t)v * w + u;
            double dc[3] = {(u - cx) / fx, (v - cy) / fy, 1.0};
            double d[3];
            for (int i = 0; i < 3; ++i) d[i] = R[i * 3] * dc[0] + R[i * 3 + 1] * dc[1] + R[i * 3 + 2] * dc[2];
            // exit distance of the box interior
            double tbest = 1e30;
            int hit = -1;  // 0..5 walls, 6+k sphere k
            const double taper = s->wall_taper;
            for (int k = 0; k < 3; ++k) {
                if (k == 0 && taper != 0) {
                    // tapered side walls x = bmax[0] + taper z, x = bmin[0] - taper z
                    const double dr = d[0] - taper * d[2], dl = d[0] + taper * d[2];
                    if (dr > 1e-12) {
                        const double tk = (s->bmax[0] + taper * t[2] - t[0]) / dr;
                        if (tk > 0 && tk < tbest) { tbest = tk; hit = 1; }
                    }
                    if (dl < -1e-12) {
                        const double tk = (s->bmin[0] - taper * t[2] - t[0]) / dl;
                        if (tk > 0 && tk < tbest) { tbest = tk; hit = 0; }
                    }
                    continue;
                }
                if (std::fabs(d[k]) < 1e-12) continue;
                double tk = ((d[k] > 0 ? s->bmax[k] : s->bmin[k]) - t[k]) / d[k];
                if (tk > 0 && tk < tbest) { tbest = tk; hit = 2 * k + (d[k] > 0 ? 1 : 0); }
            }
            for (int k = 0; k < s->nsph; ++k) {
                double oc[3] = {t[0] - s->sph[k][0], t[1] - s->sph[k][1], t[2] - s->sph[k][2]};
                double a = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
                double b = 2 * (oc[0] * d[0] + oc[1] * d[1] + oc[2] * d[2]);
                double c = oc[0] * oc[0] + oc[1] * oc[1] + oc[2] * oc[2] - (double)s->sph[k][3] * s->sph[k][3];
                double disc = b * b - 4 * a * c;
                if (disc <= 0) continue;
                double sq = std::sqrt(disc);
                double t0 = (-b - sq) / (2 * a);
                if (t0 > 1e-6 && t0 < tbest) { tbest = t0; hit = 6 + k; }
            }
            if (hit < 0) {
                if (depth_mm) depth_mm[pix] = 0;
                if (rgba) { rgba[4 * pix] = rgba[4 * pix + 1] = rgba[4 * pix + 2] = 0; rgba[4 * pix + 3] = 255; }
                if (vert4) std::memset(vert4 + 4 * pix, 0, 16);
                if (norm4) std::memset(norm4 + 4 * pix, 0, 16);
                continue;
            }
            double pw[3], nw[3];
            for (int i = 0; i < 3; ++i) pw[i] = t[i] + tbest * d[i];
            const float *base;
            if (hit < 6) {
                int ax = hit / 2;
                nw[0] = nw[1] = nw[2] = 0;
                nw[ax] = (hit & 1) ? -1.0 : 1.0;
                if (hit < 2 && taper != 0) {  // (-+1, 0, taper), unit length, facing the interior
                    const double inv = 1.0 / std::sqrt(1.0 + taper * taper);
                    nw[0] *= inv;
                    nw[2] = taper * inv;
                }
                base = s->wall_col[hit];
            } else {
                int k = hit - 6;
                for (int i = 0; i < 3; ++i) nw[i] = (pw[i] - s->sph[k][i]) / s->sph[k][3];
                base = s->sph_col[k];
            }
            // camera-frame point and normal; depth along the optical axis is tbest
            double pc[3] = {tbest * dc[0], tbest * dc[1], tbest};
            double nc[3];
            for (int i = 0; i < 3; ++i) nc[i] = R[i] * nw[0] + R[3 + i] * nw[1] + R[6 + i] * nw[2];
            if (rgba) {
                double f = s->tex_freq;
                double n1 = perlin(pw[0] * f, pw[1] * f, pw[2] * f);
                double n2 = perlin(pw[0] * f * 2.1 + 17.3, pw[1] * f * 2.1 + 5.1, pw[2] * f * 2.1 + 9.7);
                double n3 = perlin(pw[0] * f * 4.3 + 3.3, pw[1] * f * 4.3 + 41.1, pw[2] * f * 4.3 + 7.9);
                // contrast-stretched fractal noise: plateaus separated by
                // steep edges, so image gradients resemble real textures
                double nz = 0.5 + 3.0 * (0.6 * n1 + 0.3 * n2 + 0.1 * n3);
                nz = std::min(1.0, std::max(0.0, nz));
                double shade = (1.0 - s->tex_amp) + s->tex_amp * nz;
                for (int c = 0; c < 3; ++c) {
                    double val = 255.0 * base[c] * shade;
                    rgba[4 * pix + c] = (uint8_t)std::min(255.0, std::max(1.0, std::floor(val + 0.5)));
                }
                rgba[4 * pix + 3] = 255;
            }
            if (vert4) {
                vert4[4 * pix + 0] = (float)pc[0]; vert4[4 * pix + 1] = (float)pc[1];
                vert4[4 * pix + 2] = (float)pc[2]; vert4[4 * pix + 3] = 1.f;
            }
            if (norm4) {
                norm4[4 * pix + 0] = (float)nc[0]; norm4[4 * pix + 1] = (float)nc[1];
                norm4[4 * pix + 2] = (float)nc[2]; norm4[4 * pix + 3] = 1.f;
            }
            if (depth_mm) {
                uint64_t hsh = splitmix64(noise_seed ^ (pix * 0x9E3779B97F4A7C15ull));
                double ua = u01(hsh), ub = u01(splitmix64(hsh)), uc = u01(splitmix64(hsh ^ 0xabcdefull));
                double gauss = std::sqrt(-2.0 * std::log(std::max(ua, 1e-300))) * std::cos(6.283185307179586 * ub);
                double z = pc[2] + gauss * noise_k * pc[2] * pc[2];
                long mm = std::lround(z * 1000.0);
                if (uc < dropout || mm < min_mm || mm > max_mm) mm = 0;
                depth_mm[pix] = (uint16_t)mm;
            }
        }
    }
    return 0;
}

}  // extern "C"
