// GPU ray caster of the synthetic scenes (the CPU one is synth.cpp): many
// views rendered straight into device memory, for training-data and
// benchmark-input generation.  Same scene model, texture and depth-noise
// model as synth.cpp, evaluated in FP32 (the CPU renderer uses FP64, so
// images agree to rounding, not bit for bit).
#include <cuda_runtime.h>

#include <cstring>
#include <vector>

#include "../../include/slam_gb300.h"
#include "synth_common.h"

namespace {

struct ViewArgs {
    float R[9], t[3];
    uint64_t noise_seed;
    int scene;
};

__device__ __forceinline__ float fade(float t) { return t * t * t * (t * (t * 6.f - 15.f) + 10.f); }
__device__ __forceinline__ float lerpf(float t, float a, float b) { return a + t * (b - a); }
__device__ __forceinline__ float grad(int h, float x, float y, float z) {
    h &= 15;
    const float u = h < 8 ? x : y, v = h < 4 ? y : (h == 12 || h == 14 ? x : z);
    return ((h & 1) ? -u : u) + ((h & 2) ? -v : v);
}
__device__ float perlin(const int *p, float x, float y, float z) {
    const float fx = floorf(x), fy = floorf(y), fz = floorf(z);
    const int X = (int)fx & 255, Y = (int)fy & 255, Z = (int)fz & 255;
    x -= fx;
    y -= fy;
    z -= fz;
    const float u = fade(x), v = fade(y), w = fade(z);
    const int A = p[X] + Y, AA = p[A] + Z, AB = p[A + 1] + Z, B = p[X + 1] + Y, BA = p[B] + Z, BB = p[B + 1] + Z;
    return lerpf(w,
                 lerpf(v, lerpf(u, grad(p[AA], x, y, z), grad(p[BA], x - 1, y, z)),
                       lerpf(u, grad(p[AB], x, y - 1, z), grad(p[BB], x - 1, y - 1, z))),
                 lerpf(v, lerpf(u, grad(p[AA + 1], x, y, z - 1), grad(p[BA + 1], x - 1, y, z - 1)),
                       lerpf(u, grad(p[AB + 1], x, y - 1, z - 1), grad(p[BB + 1], x - 1, y - 1, z - 1))));
}

struct RenderArgs {
    int w, h;
    float fx, fy, cx, cy, noise_k, dropout;
    int min_mm, max_mm;
    uint16_t *depth;
    uint8_t *rgba;
    float *vert, *norm;
};

// One thread per pixel; blockIdx.z = view.
__global__ void k_render(const synth_scene *scenes, const int *perms, const ViewArgs *views, RenderArgs a) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x, v = blockIdx.y * blockDim.y + threadIdx.y;
    if (u >= a.w || v >= a.h) return;
    const ViewArgs &V = views[blockIdx.z];
    const synth_scene &s = scenes[V.scene];
    const int *perm = perms + 512 * V.scene;
    const size_t npx = (size_t)a.w * a.h;
    const size_t pix = (size_t)v * a.w + u;
    const size_t gpix = (size_t)blockIdx.z * npx + pix;
    const float dc[3] = {(u - a.cx) / a.fx, (v - a.cy) / a.fy, 1.f};
    float d[3];
    for (int i = 0; i < 3; ++i) d[i] = V.R[i * 3] * dc[0] + V.R[i * 3 + 1] * dc[1] + V.R[i * 3 + 2] * dc[2];
    float tbest = 1e30f;
    int hit = -1;
    const float taper = s.wall_taper;
    for (int k = 0; k < 3; ++k) {
        if (k == 0 && taper != 0.f) {
            // tapered side walls x = bmax[0] + taper z, x = bmin[0] - taper z
            const float dr = d[0] - taper * d[2], dl = d[0] + taper * d[2];
            if (dr > 1e-12f) {
                const float tk = (s.bmax[0] + taper * V.t[2] - V.t[0]) / dr;
                if (tk > 0 && tk < tbest) {
                    tbest = tk;
                    hit = 1;
                }
            }
            if (dl < -1e-12f) {
                const float tk = (s.bmin[0] - taper * V.t[2] - V.t[0]) / dl;
                if (tk > 0 && tk < tbest) {
                    tbest = tk;
                    hit = 0;
                }
            }
            continue;
        }
        if (fabsf(d[k]) < 1e-12f) continue;
        const float tk = ((d[k] > 0 ? s.bmax[k] : s.bmin[k]) - V.t[k]) / d[k];
        if (tk > 0 && tk < tbest) {
            tbest = tk;
            hit = 2 * k + (d[k] > 0 ? 1 : 0);
        }
    }
    for (int k = 0; k < s.nsph; ++k) {
        const float oc[3] = {V.t[0] - s.sph[k][0], V.t[1] - s.sph[k][1], V.t[2] - s.sph[k][2]};
        const float qa = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        const float qb = 2 * (oc[0] * d[0] + oc[1] * d[1] + oc[2] * d[2]);
        const float qc = oc[0] * oc[0] + oc[1] * oc[1] + oc[2] * oc[2] - s.sph[k][3] * s.sph[k][3];
        const float disc = qb * qb - 4 * qa * qc;
        if (disc <= 0) continue;
        const float t0 = (-qb - sqrtf(disc)) / (2 * qa);
        if (t0 > 1e-6f && t0 < tbest) {
            tbest = t0;
            hit = 6 + k;
        }
    }
    if (hit < 0) {
        if (a.depth) a.depth[gpix] = 0;
        if (a.rgba) reinterpret_cast<uchar4 *>(a.rgba)[gpix] = make_uchar4(0, 0, 0, 255);
        if (a.vert) reinterpret_cast<float4 *>(a.vert)[gpix] = make_float4(0, 0, 0, 0);
        if (a.norm) reinterpret_cast<float4 *>(a.norm)[gpix] = make_float4(0, 0, 0, 0);
        return;
    }
    float pw[3], nw[3];
    for (int i = 0; i < 3; ++i) pw[i] = V.t[i] + tbest * d[i];
    const float *base;
    if (hit < 6) {
        const int ax = hit / 2;
        nw[0] = nw[1] = nw[2] = 0;
        nw[ax] = (hit & 1) ? -1.f : 1.f;
        if (hit < 2 && taper != 0.f) {  // (-+1, 0, taper), unit length, facing the interior
            const float inv = rsqrtf(1.f + taper * taper);
            nw[0] *= inv;
            nw[2] = taper * inv;
        }
        base = s.wall_col[hit];
    } else {
        const int k = hit - 6;
        for (int i = 0; i < 3; ++i) nw[i] = (pw[i] - s.sph[k][i]) / s.sph[k][3];
        base = s.sph_col[k];
    }
    const float pc[3] = {tbest * dc[0], tbest * dc[1], tbest};
    float nc[3];
    for (int i = 0; i < 3; ++i) nc[i] = V.R[i] * nw[0] + V.R[3 + i] * nw[1] + V.R[6 + i] * nw[2];
    if (a.rgba) {
        const float f = s.tex_freq;
        const float n1 = perlin(perm, pw[0] * f, pw[1] * f, pw[2] * f);
        const float n2 = perlin(perm, pw[0] * f * 2.1f + 17.3f, pw[1] * f * 2.1f + 5.1f, pw[2] * f * 2.1f + 9.7f);
        const float n3 = perlin(perm, pw[0] * f * 4.3f + 3.3f, pw[1] * f * 4.3f + 41.1f, pw[2] * f * 4.3f + 7.9f);
        float nz = 0.5f + 3.0f * (0.6f * n1 + 0.3f * n2 + 0.1f * n3);
        nz = fminf(1.f, fmaxf(0.f, nz));
        const float shade = (1.f - s.tex_amp) + s.tex_amp * nz;
        uint8_t c3[3];
        for (int c = 0; c < 3; ++c) c3[c] = (uint8_t)fminf(255.f, fmaxf(1.f, floorf(255.f * base[c] * shade + 0.5f)));
        reinterpret_cast<uchar4 *>(a.rgba)[gpix] = make_uchar4(c3[0], c3[1], c3[2], 255);
    }
    if (a.vert) reinterpret_cast<float4 *>(a.vert)[gpix] = make_float4(pc[0], pc[1], pc[2], 1.f);
    if (a.norm) reinterpret_cast<float4 *>(a.norm)[gpix] = make_float4(nc[0], nc[1], nc[2], 1.f);
    if (a.depth) {
        const uint64_t hsh = synth::splitmix64(V.noise_seed ^ (pix * 0x9E3779B97F4A7C15ull));
        const float ua = (float)synth::u01(hsh), ub = (float)synth::u01(synth::splitmix64(hsh));
        const double uc = synth::u01(synth::splitmix64(hsh ^ 0xabcdefull));
        const float gauss = sqrtf(-2.f * logf(fmaxf(ua, 1e-30f))) * cospif(2.f * ub);
        const float z = pc[2] + gauss * a.noise_k * pc[2] * pc[2];
        long long mm = llrintf(z * 1000.f);
        if (uc < a.dropout || mm < a.min_mm || mm > a.max_mm) mm = 0;
        a.depth[gpix] = (uint16_t)mm;
    }
}

}  // namespace

extern "C" int odo_synth_render(const void *scenes_host, int nscenes, const int *view_scene, const float *poses,
                                const uint64_t *noise_seeds, int n, int w, int h, float fx, float fy, float cx,
                                float cy, float noise_k, float dropout, int min_mm, int max_mm, uint16_t *depth_dev,
                                uint8_t *rgba_dev, float *vert_dev, float *norm_dev, void *stream) {
    if (!scenes_host || nscenes < 1 || !view_scene || !poses || !noise_seeds || n < 1 || n > 65535 || w < 1 ||
        h < 1 || !(fx > 0) || !(fy > 0))
        return ODO_ERR_ARG;
    const synth_scene *sc = (const synth_scene *)scenes_host;
    std::vector<int> perms((size_t)512 * nscenes);
    for (int i = 0; i < nscenes; ++i) {
        if (sc[i].nsph < 0 || sc[i].nsph > SYNTH_MAX_SPH) return ODO_ERR_ARG;
        synth::perlin_perm(sc[i].tex_seed, perms.data() + 512 * i);
    }
    std::vector<ViewArgs> views(n);
    for (int i = 0; i < n; ++i) {
        if (view_scene[i] < 0 || view_scene[i] >= nscenes) return ODO_ERR_ARG;
        for (int r = 0; r < 3; ++r) {
            for (int c = 0; c < 3; ++c) views[i].R[r * 3 + c] = poses[16 * i + r * 4 + c];
            views[i].t[r] = poses[16 * i + r * 4 + 3];
        }
        views[i].noise_seed = noise_seeds[i];
        views[i].scene = view_scene[i];
    }
    cudaStream_t s = (cudaStream_t)stream;
    const size_t b_sc = sizeof(synth_scene) * nscenes, b_pe = perms.size() * sizeof(int), b_vi = sizeof(ViewArgs) * n;
    char *buf = nullptr;
    if (cudaMalloc(&buf, b_sc + b_pe + b_vi) != cudaSuccess) return ODO_ERR_OOM;
    cudaError_t e = cudaMemcpyAsync(buf, sc, b_sc, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(buf + b_sc, perms.data(), b_pe, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(buf + b_sc + b_pe, views.data(), b_vi, cudaMemcpyHostToDevice, s);
    RenderArgs a{w, h, fx, fy, cx, cy, noise_k, dropout, min_mm, max_mm, depth_dev, rgba_dev, vert_dev, norm_dev};
    if (e == cudaSuccess) {
        dim3 blk(16, 16), grid((w + 15) / 16, (h + 15) / 16, n);
        k_render<<<grid, blk, 0, s>>>((const synth_scene *)buf, (const int *)(buf + b_sc),
                                      (const ViewArgs *)(buf + b_sc + b_pe), a);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(buf);
    return e == cudaSuccess ? ODO_OK : ODO_ERR_CUDA;
}
