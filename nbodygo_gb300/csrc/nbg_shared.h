/*
 * nbg_shared.h - constants and the seeded fragment-position generator shared by
 * the CPU oracle and the GPU kernels.
 *
 * Constants restate cmd/body/body.go:18-24:
 *   G = 6.673e-11, at most 100 (+1) fragments emitted per cycle, 2000 in total.
 *
 * Fragment positions.  The reference draws them with util.GetVectorEven
 * (cmd/util/vectorutil.go:32-42): rejection sampling of a point in the unit
 * ball, x = rand.Float64()*2-1 (same for y, z) until x*x+y*y+z*z <= 1, then
 * center + radius*(x,y,z).  It reseeds math/rand from the wall clock on every
 * call, so its output cannot be reproduced.  Here every draw comes from a
 * counter-based generator instead: the SplitMix64 output function (Steele,
 * Lea & Flood, "Fast splittable pseudorandom number generators", OOPSLA 2014)
 * applied to a key built from (seed, parent id, cycle index) and a counter
 * built from (fragment index within this cycle, draw index).  The rejection
 * loop and the arithmetic of the reference are kept; after 85 rejected
 * attempts (probability ~1e-27) the offset (0,0,0) is used.
 */
#ifndef NBG_SHARED_H
#define NBG_SHARED_H

#include <stdint.h>

#if defined(__CUDACC__)
#define NBG_SFN __host__ __device__ static inline
#else
#define NBG_SFN static inline
#endif

#define NBG_G 6.673e-11
#define NBG_MAX_FRAGS_PER_CYCLE 100 /* body.go:21; the loop emits up to 101 */
#define NBG_MAX_FRAGS 2000.0        /* body.go:22 */
#define NBG_FRAG_MAX_ATTEMPTS 85

NBG_SFN uint64_t nbg_splitmix_out(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

/* Key of the stream that places the fragments one parent emits in one cycle. */
NBG_SFN uint64_t nbg_frag_key(uint64_t seed, int64_t parent_id, uint64_t cycle)
{
    uint64_t k = nbg_splitmix_out(seed + 0x9e3779b97f4a7c15ull);
    k = nbg_splitmix_out(k ^ ((uint64_t)parent_id * 0xd1b54a32d192ed03ull));
    k = nbg_splitmix_out(k ^ (cycle * 0xaef17502108ef2d9ull + 0x632be59bd9b4e019ull));
    return k;
}

/* Uniform double in [0, 1) with 53 random bits (draw `ctr` of stream `key`). */
NBG_SFN double nbg_frag_uniform(uint64_t key, uint64_t ctr)
{
    uint64_t u = nbg_splitmix_out(key + (ctr + 1ull) * 0x9e3779b97f4a7c15ull);
    return (double)(u >> 11) * 0x1p-53;
}

/* Position of fragment `cnt` (0-based within this cycle) of a parent. */
NBG_SFN void nbg_frag_point(uint64_t key, int cnt, double cx, double cy, double cz,
                            double radius, double *ox, double *oy, double *oz)
{
    double x = 0.0, y = 0.0, z = 0.0;
    uint64_t base = (uint64_t)cnt * 256ull;
    int accepted = 0;
    for (int a = 0; a < NBG_FRAG_MAX_ATTEMPTS; a++) {
        x = nbg_frag_uniform(key, base + 3ull * (uint64_t)a) * 2.0 - 1.0;
        y = nbg_frag_uniform(key, base + 3ull * (uint64_t)a + 1ull) * 2.0 - 1.0;
        z = nbg_frag_uniform(key, base + 3ull * (uint64_t)a + 2ull) * 2.0 - 1.0;
        double d = x * x + y * y + z * z;
        if (!(d > 1.0)) {
            accepted = 1;
            break;
        }
    }
    if (!accepted) x = y = z = 0.0;
    *ox = (x * radius) + cx;
    *oy = (y * radius) + cy;
    *oz = (z * radius) + cz;
}

#endif /* NBG_SHARED_H */
