// Scene description and seeded generators shared by the CPU ray caster
// (synth.cpp) and the GPU ray caster (synth_gpu.cu).
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#define SYNTH_HD __host__ __device__
#else
#define SYNTH_HD
#endif

#define SYNTH_MAX_SPH 128

extern "C" {
typedef struct {
    float bmin[3], bmax[3];          // interior of the box (metres, world frame)
    int nsph;
    float sph[SYNTH_MAX_SPH][4];     // centre xyz, radius
    float sph_col[SYNTH_MAX_SPH][3]; // base colour 0..1
    float wall_col[6][3];
    float tex_freq;   // texture cycles per metre
    float tex_amp;    // 0..1 texture contrast
    uint64_t tex_seed;
    // the two x faces (side walls) tapered along z: x = bmax[0] + wall_taper z
    // and x = bmin[0] - wall_taper z (0: the box faces)
    float wall_taper;
} synth_scene;
}

namespace synth {

SYNTH_HD inline uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
SYNTH_HD inline double u01(uint64_t h) { return (double)(h >> 11) * (1.0 / 9007199254740992.0); }

struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(splitmix64(seed ^ 0x5eed5eedull)) {}
    double uni() { s = splitmix64(s); return u01(s); }
    double uni(double a, double b) { return a + (b - a) * uni(); }
};

// Seeded permutation table of the improved Perlin noise (Perlin 2002).
inline void perlin_perm(uint64_t seed, int p[512]) {
    int q[256];
    for (int i = 0; i < 256; ++i) q[i] = i;
    Rng r(seed);
    for (int i = 255; i > 0; --i) {
        int j = (int)(r.uni() * (i + 1));
        if (j > i) j = i;
        int t = q[i];
        q[i] = q[j];
        q[j] = t;
    }
    for (int i = 0; i < 512; ++i) p[i] = q[i & 255];
}

}  // namespace synth
