/*
 * k_mixed.cu - mixed-precision force + collision detection.
 *
 * Computes the same force pass as calcForceFrom (cmd/body/body.go:214-225)
 * and the same collision set as Collided (body.go:192-208), with the pair
 * terms in FP32:
 *
 *  - bodies are visited in Morton order (k_sort.cu), so each 512-body i-tile
 *    is compact in space;
 *  - positions are held as hi/lo float pairs (x = hi + lo to ~2^-48 |x|);
 *    each work item re-centres positions on its i-tile's origin c with
 *    (x_hi - c) + x_lo, so the FP32 coordinates a pair subtracts carry an
 *    error of about 2^-24 |x - c|: small for the near pairs, where it matters;
 *  - pair terms m_j (x_j - x_i) / r^3 use packed f32x2 arithmetic (two j per
 *    instruction: FFMA2 / FADD2 / FMUL2) and the SFU reciprocal square root;
 *  - every 256 j the FP32 tile sum is folded into a (hi, lo) float pair with
 *    TwoSum (Knuth), so the accumulated rounding error stays that of a
 *    128-term sum; each item's total is written as FP64;
 *  - a pair closer than a conservative bound - the larger of r_i + r_max plus
 *    the FP32 error bound, and near_kappa times the body's offset from its
 *    i-tile's origin - takes a near-pair pass: dx from the difference of the
 *    hi/lo parts (error ~2^-24 |dx|), a Newton-refined reciprocal square
 *    root, and the term added to the compensated sums directly;
 *  - a near pair within 2^-10 of touching is re-evaluated in FP64 with the
 *    reference's exact expressions: that FP64 dist decides the overlap skip
 *    and the collision test, so the event set is the reference's.
 *
 * The pair work of a cycle, W units of (i-tile, one j-body), is cut into C
 * chunks, about 32 per resident CTA, whatever the sizes of the sims and
 * tiles; a chunk is a run of (i-tile, j-range) segments.  The cut is guided
 * (nbg_chunk_start): large chunks first, small ones last.  Persistent CTAs
 * take chunks from an atomic counter, so a CTA that meets many near pairs
 * simply takes fewer, and the small last chunks let the CTAs finish
 * together.  Each chunk writes its share of an i-tile to a slot of
 * its own, and k_mix_out adds the shares in chunk order, so results do not
 * depend on scheduling.
 */
#include <atomic>
#include <type_traits>

#include "nbg_internal.cuh"
#include "nbg_math.h"
#include "nbg_shared.h"

#define FULL_MASK 0xffffffffu
#define SENTINEL_POS 1.0e18f

__device__ __forceinline__ float rsqrt_sfu(float x)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

/* TwoSum: (hi, lo) += v with the rounding error of hi + v kept in lo. */
__device__ __forceinline__ void two_sum_add(float &hi, float &lo, float v)
{
    float s = hi + v;
    float bb = s - hi;
    float e = (hi - (s - bb)) + (v - bb);
    hi = s;
    lo += e;
}

/* A body whose position is not finite or whose radius is NaN interacts with
 * no other body in the reference's arithmetic except through NaN; the mixed
 * form keeps it out of every pair (massless, far away) and sets its own force
 * in k_mix_out. */
__device__ __forceinline__ bool is_special(double x, double y, double z, double r)
{
    return !(fabs(x) <= NBG_DBL_MAX && fabs(y) <= NBG_DBL_MAX && fabs(z) <= NBG_DBL_MAX) || r != r;
}

/* ---- per-cycle reductions: r_max, |x|_max, m_scale ------------------------ */

__global__ void k_mix_reduce(BodyArrays A, DevCtl *ctl, SimSegs seg)
{
    if (ctl->error) return;
    const ll n = ctl->n;
    float rmax = 0.f, xmax = 0.f;
    double mmax = 0.0;
    const ll stride = (ll)gridDim.x * blockDim.x;
    /* warp-uniform trip count: every lane takes part in the per-sim reduction */
    for (ll base = (ll)blockIdx.x * blockDim.x; base < n; base += stride) {
        const ll k = base + threadIdx.x;
        float xk = 0.f;
        int sim = -1;
        if (k < n) {
            const double x = A.x[k], y = A.y[k], z = A.z[k], r = A.rad[k];
            if (!is_special(x, y, z, r)) {
                rmax = fmaxf(rmax, (float)fmax(r, 0.0));
                xk = (float)fmax(fabs(x), fmax(fabs(y), fabs(z)));
                xmax = fmaxf(xmax, xk);
                if ((A.flags[k] & NBG_LIVE_MASK) == NBG_F_EXISTS) mmax = fmax(mmax, fabs(A.m[k]));
                sim = nbg_sim_of(seg.off, seg.nsims, k);
            }
        }
        if (seg.nsims > 1) {
            const unsigned peers = __match_any_sync(FULL_MASK, sim);
            const unsigned mx = __reduce_max_sync(peers, __float_as_uint(xk * (1.0f + 0x1p-20f)));
            if (sim >= 0 && (int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicMax(&seg.xmax_bits[sim], mx);
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        rmax = fmaxf(rmax, __shfl_xor_sync(FULL_MASK, rmax, o));
        xmax = fmaxf(xmax, __shfl_xor_sync(FULL_MASK, xmax, o));
        mmax = fmax(mmax, __shfl_xor_sync(FULL_MASK, mmax, o));
    }
    if ((threadIdx.x & 31) == 0) {
        /* rounding up keeps both bounds conservative */
        atomicMax(&ctl->rmax_bits, __float_as_uint(rmax * (1.0f + 0x1p-20f)));
        atomicMax(&ctl->xmax_bits, __float_as_uint(xmax * (1.0f + 0x1p-20f)));
        atomicMax((unsigned long long *)&ctl->m_scale, (ull)__double_as_longlong(mmax));
        if (seg.nsims == 1) atomicMax(&seg.xmax_bits[0], __float_as_uint(xmax * (1.0f + 0x1p-20f)));
    }
}

/* Packs body perm[p] at sorted position p:
 * jhi = (x_hi, y_hi, z_hi, m/m_scale), jlo = (x_lo, y_lo, z_lo, radius).
 * A special body (see is_special) gets a far sentinel position, no mass and
 * x_lo = NaN, which is how the kernels recognise it. */
__global__ void k_mix_pack(BodyArrays A, DevCtl *ctl, const unsigned *perm, float4 *jhi, float4 *jlo)
{
    if (ctl->error) return;
    const ll n = ctl->n;
    double ms = ctl->m_scale;
    if (!(ms > 0.0)) ms = 1.0;
    for (ll p = (ll)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (ll)gridDim.x * blockDim.x) {
        const ll k = perm[p];
        const double x = A.x[k], y = A.y[k], z = A.z[k], r = A.rad[k];
        if (is_special(x, y, z, r)) {
            jhi[p] = make_float4(SENTINEL_POS, SENTINEL_POS, SENTINEL_POS, 0.f);
            jlo[p] = make_float4(__int_as_float(0x7fc00000), 0.f, 0.f, 0.f);
            continue;
        }
        const float xh = (float)x, yh = (float)y, zh = (float)z;
        const float xl = (float)(x - (double)xh), yl = (float)(y - (double)yh), zl = (float)(z - (double)zh);
        const bool live = (A.flags[k] & NBG_LIVE_MASK) == NBG_F_EXISTS;
        const float m = live ? (float)(A.m[k] / ms) : 0.f;
        jhi[p] = make_float4(xh, yh, zh, m);
        jlo[p] = make_float4(xl, yl, zl, (float)r);
    }
}

__device__ __forceinline__ bool packed_special(const float4 &lo) { return lo.x != lo.x; }

/* origin of each i-tile: centre of the bounding box of its bodies */
#define TILES_BLOCK 128
__global__ void __launch_bounds__(TILES_BLOCK) k_mix_tiles(DevCtl *ctl, SimSegs seg, const float4 *jhi,
                                                           const float4 *jlo, float4 *tile_c, float *tile_t, int itile)
{
    __shared__ float red[6][TILES_BLOCK / 32];
    if (ctl->error) return;
    const ll ntiles = seg.mtile_off[seg.nsims];
    for (ll tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int sim = nbg_sim_of(seg.mtile_off, seg.nsims, tile);
    const ll base = seg.off[sim] + (tile - seg.mtile_off[sim]) * itile;
    const ll n = seg.off[sim + 1] < base + itile ? seg.off[sim + 1] : base + itile;
    float lo[3] = {3e38f, 3e38f, 3e38f}, hi[3] = {-3e38f, -3e38f, -3e38f};
    for (ll p = base + threadIdx.x; p < n; p += TILES_BLOCK) {
        if (packed_special(jlo[p])) continue;
        float4 h = jhi[p];
        lo[0] = fminf(lo[0], h.x);
        lo[1] = fminf(lo[1], h.y);
        lo[2] = fminf(lo[2], h.z);
        hi[0] = fmaxf(hi[0], h.x);
        hi[1] = fmaxf(hi[1], h.y);
        hi[2] = fmaxf(hi[2], h.z);
    }
    for (int o = 16; o > 0; o >>= 1)
        for (int c = 0; c < 3; c++) {
            lo[c] = fminf(lo[c], __shfl_xor_sync(FULL_MASK, lo[c], o));
            hi[c] = fmaxf(hi[c], __shfl_xor_sync(FULL_MASK, hi[c], o));
        }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0)
        for (int c = 0; c < 3; c++) {
            red[c][w] = lo[c];
            red[3 + c][w] = hi[c];
        }
    __syncthreads();
    if (threadIdx.x == 0) {
        float c3[3], e2 = 0.f, amax = 0.f;
        for (int c = 0; c < 3; c++) {
            float l = red[c][0], h = red[3 + c][0];
            for (int q = 1; q < TILES_BLOCK / 32; q++) {
                l = fminf(l, red[c][q]);
                h = fmaxf(h, red[3 + c][q]);
            }
            c3[c] = (l <= h) ? 0.5f * l + 0.5f * h : 0.f;
            const float e = l <= h ? fmaxf(h - c3[c], c3[c] - l) : 0.f;
            e2 += e * e;
            amax = fmaxf(amax, l <= h ? fmaxf(fabsf(l), fabsf(h)) : 0.f);
        }
        /* .w: a radius about the origin that holds every body of the tile,
         * rounded up past the FP32 arithmetic and the bodies' lo parts */
        const float rad = sqrtf(e2) * (1.0f + 0x1p-16f) + amax * 0x1p-20f;
        tile_c[tile] = make_float4(c3[0], c3[1], c3[2], rad);
        if (tile_t) tile_t[tile] = 0.f;
    }
    __syncthreads(); /* red[] is rewritten by the next tile */
    }
}

/* ---- the pair kernel ----------------------------------------------------- */

__device__ static int detect_event_mixed(unsigned bi, unsigned bj, double ri, double rj, double dist)
{
    bool ei = (bi == NBG_ELASTIC || bi == NBG_FRAGMENT);
    bool ej = (bj == NBG_ELASTIC || bj == NBG_FRAGMENT);
    if (ei && ej) return (int)NBG_EVT_COLL_IJ;
    if (bi == NBG_SUBSUME || bj == NBG_SUBSUME) {
        if (ri > rj && dist <= ri) return (int)NBG_EVT_SUB_IJ;
        if (rj > ri && dist <= rj) return (int)NBG_EVT_SUB_JI;
    }
    return -1;
}

/* A pair inside the candidate bound (body indices i, j): decide overlap and
 * collision in FP64 with the reference's expressions (no contraction:
 * explicit _rn intrinsics), return the force term if the pair does not
 * overlap (m_scale-normalised acceleration units), record the event. */
__device__ static void candidate_pair(const BodyArrays &A, DevCtl *ctl, ull *ev_keys, ll ev_cap, ll i, ll j,
                                      double inv_ms, double &tx, double &ty, double &tz)
{
    tx = ty = tz = 0.0;
    const unsigned fi = A.flags[i], fj = A.flags[j];
    const double xi = A.x[i], yi = A.y[i], zi = A.z[i], ri = A.rad[i];
    const double dx = __dsub_rn(A.x[j], xi);
    const double dy = __dsub_rn(A.y[j], yi);
    const double dz = __dsub_rn(A.z[j], zi);
    const double dist = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
    const double rj = A.rad[j];
    const double rr = __dadd_rn(ri, rj);
    const bool coll_i = (fi & NBG_F_COLLIDED) != 0;
    const bool live_j = (fj & NBG_LIVE_MASK) == NBG_F_EXISTS;
    if (live_j && (coll_i || dist > rr)) {
        const double w = (A.m[j] * inv_ms) / (dist * dist * dist);
        tx = w * dx;
        ty = w * dy;
        tz = w * dz;
    }
    const bool live_i = (fi & NBG_LIVE_MASK) == NBG_F_EXISTS;
    if (live_i && !coll_i && dist <= rr) {
        int type = detect_event_mixed(NBG_BEHAVIOR(fi), NBG_BEHAVIOR(fj), ri, rj, dist);
        if (type >= 0) {
            ll slot = (ll)atomicAdd((unsigned long long *)&ctl->ev_count, 1ull);
            if (slot < ev_cap) ev_keys[slot] = ((ull)i << 32) | ((ull)j << 2) | (ull)type;
        }
    }
}

__device__ __forceinline__ void fold64(float &hi, float &lo, double v)
{
    float vh = (float)v;
    float vl = (float)(v - (double)vh);
    two_sum_add(hi, lo, vh);
    lo += vl;
}

/* i-body at sorted position p (p >= n: none) re-centred on the tile origin
 * c, and its near-pair threshold t on r^2 (FP32, conservative): pairs closer
 * than max(r_i + r_max + the FP32 error bound, kappa |x - c|_max) take the
 * exact path.  A special body sits at the sentinel with t = -1. */
__device__ __forceinline__ void i_body_setup(const float4 *__restrict__ jhi, const float4 *__restrict__ jlo, ll p, ll n,
                                             const float4 &c, float rmax, float xmax, double kappa, float &xr,
                                             float &yr, float &zr, float &t)
{
    xr = yr = zr = 0.f;
    t = -1.f;
    if (p >= n) return;
    const float4 h = jhi[p], l = jlo[p];
    if (packed_special(l)) {
        xr = yr = zr = SENTINEL_POS;
        return;
    }
    xr = (h.x - c.x) + l.x;
    yr = (h.y - c.y) + l.y;
    zr = (h.z - c.z) + l.z;
    const double ri = (double)l.w + fabs((double)l.w) * 0x1p-22; /* rounded up */
    const double D = fmax(0.0, ri + (double)rmax);
    const double amax = (double)fmaxf(fabsf(xr), fmaxf(fabsf(yr), fabsf(zr)));
    const double eps = 0x1p-19 * (amax + D) + 0x1p-44 * (double)xmax + 0x1p-100;
    const double b = fmax(D + eps, kappa * amax) * (1.0 + 0x1p-18);
    t = __double2float_ru(b * b);
}

/* every i-body's re-centred position and near-pair threshold, once per
 * cycle; the pair kernel reads them for each chunk that covers the body */
__global__ void k_mix_iprep(DevCtl *ctl, SimSegs seg, const float4 *__restrict__ jhi,
                            const float4 *__restrict__ jlo, const float4 *__restrict__ tile_c, float4 *iprep,
                            float *tile_t, int itile)
{
    if (ctl->error) return;
    const ll n = ctl->n;
    const float rmax = __uint_as_float(ctl->rmax_bits);
    const float xmax = __uint_as_float(ctl->xmax_bits);
    const double kappa0 = (double)ctl->near_kappa;
    for (ll p = (ll)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (ll)gridDim.x * blockDim.x) {
        const int sim = nbg_sim_of(seg.off, seg.nsims, p);
        const ll s0 = seg.off[sim];
        /* In a small collection one or two tiles span it all, so a body's
         * offset from its tile origin is large next to its neighbours'
         * distances, and the neighbours carry much of its force: twice the
         * factor there.  Such collections hold a small share of the work. */
        const double kappa = seg.off[sim + 1] - s0 <= NBG_NEAR_SMALL_N ? 2.0 * kappa0 : kappa0;
        const ll tile = seg.mtile_off[sim] + (p - s0) / itile;
        const float4 c = tile_c[tile];
        float xr, yr, zr, t;
        i_body_setup(jhi, jlo, p, seg.off[sim + 1], c, rmax, xmax, kappa, xr, yr, zr, t);
        iprep[p] = make_float4(xr, yr, zr, t);
        /* the tile's largest near-pair threshold (positive floats order as
         * their bit patterns) */
        if (tile_t && t > 0.f) atomicMax((unsigned *)&tile_t[tile], __float_as_uint(t));
    }
}

/* One j of a near-pair pass for i-body p (raw i: hi_i, lo_i; re-centred
 * i: xi..zi; threshold thk): adds the FP32 term to (tx, ty, tz), or, for a
 * near pair, the term from the exact hi/lo difference, or, for a possible
 * overlap, the FP64 term folded into the (hi, lo) sums with the event
 * recorded.  xj..m are j's re-centred position and mass from the tile;
 * hj, lj its raw hi/lo (read only for a near pair, through get_raw). */
template <typename RAW>
__device__ __forceinline__ void near_pass_j(const BodyArrays &A, DevCtl *ctl, ull *ev_keys, ll ev_cap,
                                            const unsigned *__restrict__ perm, double inv_ms, ll i, ll q,
                                            const float4 &hi_i, const float4 &lo_i, float xi, float yi, float zi,
                                            float thk, float xj, float yj, float zj, float m, RAW get_raw, float &tx,
                                            float &ty, float &tz, float &fhx, float &flx, float &fhy, float &fly,
                                            float &fhz, float &flz)
{
    float dx = xj - xi, dy = yj - yi, dz = zj - zi;
    float r2 = dx * dx + dy * dy + dz * dz;
    if (r2 < thk) {
        /* near pair: difference of the hi/lo positions (error ~2^-24 |dx|) */
        float4 hj, lj;
        get_raw(q, hj, lj);
        dx = (hj.x - hi_i.x) + (lj.x - lo_i.x);
        dy = (hj.y - hi_i.y) + (lj.y - lo_i.y);
        dz = (hj.z - hi_i.z) + (lj.z - lo_i.z);
        r2 = dx * dx + dy * dy + dz * dz;
        const float rs = lo_i.w + lj.w;
        /* an overlap, or a pair within 2^-10 of the overlap distance, is
         * decided in FP64 */
        if (!(r2 > rs * rs * (1.0f + 0x1p-10f) && rs >= 0.f) || (lo_i.w < 0.f) || (lj.w < 0.f)) {
            double qx, qy, qz;
            candidate_pair(A, ctl, ev_keys, ev_cap, i, (ll)perm[q], inv_ms, qx, qy, qz);
            fold64(fhx, flx, qx);
            fold64(fhy, fly, qy);
            fold64(fhz, flz, qz);
            return;
        }
        /* A near pair can carry most of the body's force, so its term is
         * made as exact as FP32 allows: one Newton step on the SFU's
         * reciprocal square root (relative error 2^-22.9 -> ~2^-24), and
         * the term goes straight into the (hi, lo) sums rather than through
         * the tile's FP32 sum, whose roundings would be ulps of this term */
        float inv = rsqrt_sfu(r2);
        inv = inv * (1.5f - 0.5f * r2 * inv * inv);
        const float s = m * inv * inv * inv;
        two_sum_add(fhx, flx, s * dx);
        two_sum_add(fhy, fly, s * dy);
        two_sum_add(fhz, flz, s * dz);
        return;
    }
    const float inv = rsqrt_sfu(r2);
    const float s = m * inv * inv * inv;
    tx += s * dx;
    ty += s * dy;
    tz += s * dz;
}

/* ---- bulk copies into shared memory ----------------------------------------
 * cp.async.bulk (the copy engine, no registers) completing on an mbarrier:
 * the issuing thread arms the barrier with the bytes it expects, and every
 * thread waits for the barrier's phase.  Waits give up after about two
 * seconds of SM clock. */
__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(ull *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(ull *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

/* bytes (a multiple of 16, both addresses 16-byte aligned) from global src
 * to shared dst, completing on bar */
__device__ __forceinline__ void bulk_to_smem(void *dst, const void *src, unsigned bytes, ull *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(ull *bar, unsigned parity)
{
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_addr(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}

/* true once the phase of parity `parity` has completed; false after ~2^32
 * SM clocks */
__device__ __forceinline__ bool mbar_wait_bounded(ull *bar, unsigned parity)
{
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > (1ll << 32)) return false;
    return true;
}

/* Everything in this kernel is indexed by sorted position (p for i, q for
 * j); perm maps a position to the body index used by the FP64 arrays and the
 * event keys. */
template <int BLOCK, int K, int JT, int UNROLL, int MINB, bool SF, bool DB, bool BULK>
__global__ void __launch_bounds__(BLOCK, MINB)
k_pair_mixed(BodyArrays A, DevCtl *ctl, SimSegs seg, const float4 *__restrict__ jhi, const float4 *__restrict__ jlo,
             const float4 *__restrict__ tile_c, const float4 *__restrict__ iprep, const unsigned *__restrict__ perm,
             double *__restrict__ part, ull *ev_keys, ll ev_cap)
{
    constexpr int JP = JT / 2; /* j pairs per tile */
    constexpr int ITILE = BLOCK * K;
    static_assert(ITILE >= NBG_MIX_MIN_ITILE, "tile-origin buffer is sized for the smallest i-tile");
    static_assert(ITILE <= NBG_MIX_MAX_ITILE, "partial-sum buffer is sized for the largest i-tile");
    static_assert(!(DB && BULK), "one way of filling the tiles");
    /* DB: two tile buffers; the next tile's raw j is loaded into registers
     * while this tile is computed, and stored to the other buffer after it,
     * so a tile costs one barrier and its global loads are hidden.
     * BULK: two tile buffers too, and the raw j of the tiles after the next
     * are copied into two raw buffers by bulk copies issued ahead; each
     * tile re-centres the next one's raw j from shared memory. */
    __shared__ float4 sAb[DB || BULK ? 2 : 1][JP], sBb[DB || BULK ? 2 : 1][JP];
    __shared__ alignas(128) float4 rawH[BULK ? 2 : 1][BULK ? JT : 1], rawL[BULK ? 2 : 1][BULK ? JT : 1];
    __shared__ alignas(8) ull mbar[2];
    constexpr int PPT = (JP + BLOCK - 1) / BLOCK; /* j pairs a thread fills */
    float4 pre[DB ? PPT : 1][2][2];
    /* SF: each i-body's (hi, lo) sums and near-pair threshold live in shared
     * memory (only this thread touches them; read once per j-tile), which
     * frees seven registers per i-body for occupancy */
    __shared__ float sfold[6][SF ? ITILE : 1], sthr[SF ? ITILE : 1];
    float rfold[6][SF ? 1 : K], rthr[SF ? 1 : K];
#define FOLD(c, k) (SF ? sfold[c][(k) * BLOCK + tid] : rfold[c][SF ? 0 : (k)])
#define THR(k) (SF ? sthr[(k) * BLOCK + tid] : rthr[SF ? 0 : (k)])
    __shared__ ll s_chunk;
    if (ctl->error) return;
    const int C = ctl->splits;
    const ll W = ctl->work_total;
    double ms = ctl->m_scale;
    if (!(ms > 0.0)) ms = 1.0;
    const double inv_ms = 1.0 / ms;
    const float rmax = __uint_as_float(ctl->rmax_bits);
    const float xmax = __uint_as_float(ctl->xmax_bits);
    const double kappa = (double)ctl->near_kappa;
    const int tid = threadIdx.x;
    /* BULK: bit b of ph is the parity of mbar[b]'s next phase, bit b of pend
     * says a copy into raw buffer b is in flight (both the same in every
     * thread) */
    unsigned ph = 0, pend = 0;
    if (BULK) {
        if (tid == 0) {
            mbar_init(&mbar[0], 1);
            mbar_init(&mbar[1], 1);
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        __syncthreads();
    }

    for (;;) {
    if (tid == 0) s_chunk = (ll)atomicAdd((unsigned long long *)&ctl->work_next, 1ull);
    __syncthreads();
    const ll chunk = s_chunk;
    __syncthreads();
    if (chunk >= C) break;
    /* this chunk's units [U, U1): a run of (i-tile, j-range) segments */
    ll U = nbg_chunk_start(chunk, C, W);
    const ll U1 = nbg_chunk_start(chunk + 1, C, W);
    int sim = U < W ? nbg_sim_of(seg.item_off, seg.nsims, U) : 0;
    while (U < U1) {
        while (seg.item_off[sim + 1] <= U) sim++; /* past the end of a sim (or an empty one) */
        const ll s0 = seg.off[sim], n = seg.off[sim + 1];
        const ll ns = n - s0;
        const ll local = U - seg.item_off[sim];
        const ll t = local / ns;
        const ll j0 = local - t * ns;
        const ll len = ns - j0 < U1 - U ? ns - j0 : U1 - U;
        const ll g = seg.mtile_off[sim] + t;
        const ll ibase = s0 + t * ITILE;
        const float4 c = tile_c[g];

        float2 nx[K], ny[K], nz[K];
#pragma unroll
        for (int k = 0; k < K; k++) {
            const ll p = ibase + (ll)k * BLOCK + tid;
            float xr = 0.f, yr = 0.f, zr = 0.f, t = -1.f;
            if (p < n) {
                const float4 v = iprep[p];
                xr = v.x;
                yr = v.y;
                zr = v.z;
                t = v.w;
            }
            nx[k] = make_float2(-xr, -xr);
            ny[k] = make_float2(-yr, -yr);
            nz[k] = make_float2(-zr, -zr);
            THR(k) = t;
#pragma unroll
            for (int cc = 0; cc < 6; cc++) FOLD(cc, k) = 0.f;
        }

        const ll jb = s0 + j0;
        const ll je = jb + len;
        /* re-centred j pair (q, q + 1) of a tile: sentinels past je or for a
         * special body */
        auto pack = [&](const float4 (&h)[2], const float4 (&l)[2], ll q, float4 &oa, float4 &ob) {
            float v[2][4];
#pragma unroll
            for (int e = 0; e < 2; e++) {
                if (q + e < je && !packed_special(l[e])) {
                    v[e][0] = (h[e].x - c.x) + l[e].x;
                    v[e][1] = (h[e].y - c.y) + l[e].y;
                    v[e][2] = (h[e].z - c.z) + l[e].z;
                    v[e][3] = h[e].w;
                } else {
                    v[e][0] = v[e][1] = v[e][2] = SENTINEL_POS;
                    v[e][3] = 0.f;
                }
            }
            oa = make_float4(v[0][0], v[1][0], v[0][1], v[1][1]);
            ob = make_float4(v[0][2], v[1][2], v[0][3], v[1][3]);
        };
        auto load_raw = [&](ll jt2) {
#pragma unroll
            for (int r = 0; r < (DB ? PPT : 1); r++) {
                const int sp = tid + r * BLOCK;
#pragma unroll
                for (int e = 0; e < 2; e++) {
                    const ll q = jt2 + 2 * sp + e;
                    if (sp < JP && q < je) {
                        pre[r][e][0] = jhi[q];
                        pre[r][e][1] = jlo[q];
                    }
                }
            }
        };
        auto store_raw = [&](int buf, ll jt2) {
#pragma unroll
            for (int r = 0; r < (DB ? PPT : 1); r++) {
                const int sp = tid + r * BLOCK;
                if (sp < JP) {
                    const float4 h[2] = {pre[r][0][0], pre[r][1][0]}, l[2] = {pre[r][0][1], pre[r][1][1]};
                    pack(h, l, jt2 + 2 * sp, sAb[buf][sp], sBb[buf][sp]);
                }
            }
        };
        /* BULK: the segment's raw tile u (j from jb + u JT) goes to raw
         * buffer u & 1 through mbar[u & 1]; its re-centred pairs to tile
         * buffer u & 1 */
        auto issue = [&](ll q0, int b) {
            pend |= 1u << b;
            if constexpr (BULK) if (tid == 0) {
                const unsigned cnt = (unsigned)(je - q0 < JT ? je - q0 : JT);
                /* the buffer's last readers, before a barrier, read it
                 * through the generic proxy */
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                mbar_expect_tx(&mbar[b], 2u * 16u * cnt + ctl->test_tx_extra);
                bulk_to_smem(&rawH[b][0], jhi + q0, 16u * cnt, &mbar[b]);
                bulk_to_smem(&rawL[b][0], jlo + q0, 16u * cnt, &mbar[b]);
            }
        };
        /* waits for raw buffer b (the tile from q0) and re-centres it into
         * tile buffer b; false if the copy did not complete */
        auto unpack = [&](ll q0, int b) -> bool {
            if constexpr (BULK) {
                if (!mbar_wait_bounded(&mbar[b], (ph >> b) & 1u)) return false;
                ph ^= 1u << b;
                pend &= ~(1u << b);
                for (int sp = tid; sp < JP; sp += BLOCK) {
                    const float4 h[2] = {rawH[b][2 * sp], rawH[b][2 * sp + 1]};
                    const float4 l[2] = {rawL[b][2 * sp], rawL[b][2 * sp + 1]};
                    pack(h, l, q0 + 2 * sp, sAb[b][sp], sBb[b][sp]);
                }
            }
            return true;
        };
        /* a copy that did not complete: the cycle fails with NBG_E_TIMEOUT
         * after a second bounded wait for the copies still in flight */
        auto give_up = [&]() {
            if (tid == 0) {
                ctl->error = NBG_E_TIMEOUT;
                ctl->error_what = 8;
            }
            for (int b = 0; b < 2; b++)
                if (pend & (1u << b)) mbar_wait_bounded(&mbar[b], (ph >> b) & 1u);
        };
        int buf = 0;
        if (DB) {
            load_raw(jb);
            __syncthreads(); /* the previous segment's readers are done */
            store_raw(0, jb);
        }
        if (BULK) {
            /* the previous segment's readers of every buffer finished before
             * its last barrier */
            issue(jb, 0);
            if (jb + JT < je) issue(jb + JT, 1);
            const bool ok = unpack(jb, 0);
            if (__syncthreads_or(!ok)) {
                give_up();
                return;
            }
            if (jb + 2 * JT < je) issue(jb + 2 * JT, 0);
        }
        for (ll jt = jb; jt < je; jt += JT) {
            const float4 *sA = sAb[DB || BULK ? buf : 0], *sB = sBb[DB || BULK ? buf : 0];
            if (BULK) {
                /* this tile was re-centred before the last barrier */
            } else if (DB) {
                __syncthreads(); /* this tile is stored */
                if (jt + JT < je) load_raw(jt + JT);
            } else {
                __syncthreads();
                for (int sp = tid; sp < JP; sp += BLOCK) {
                    float4 h[2], l[2];
#pragma unroll
                    for (int e = 0; e < 2; e++) {
                        const ll q = jt + 2 * sp + e;
                        h[e] = q < je ? jhi[q] : make_float4(0.f, 0.f, 0.f, 0.f);
                        l[e] = q < je ? jlo[q] : make_float4(0.f, 0.f, 0.f, 0.f);
                    }
                    pack(h, l, jt + 2 * sp, sAb[0][sp], sBb[0][sp]);
                }
                __syncthreads();
            }

            float2 ax[K], ay[K], az[K];
            float mn[K];
#pragma unroll
            for (int k = 0; k < K; k++) {
                ax[k] = ay[k] = az[k] = make_float2(0.f, 0.f);
                mn[k] = 3.0e38f;
            }
            /* the j pairs this tile holds (a segment's last tile is short) */
            /* j pairs of this tile that hold bodies: JP, except in a
             * segment's short last tile */
            const int jpv = je - jt >= JT ? JP : (int)((je - jt + 1) / 2);
            auto pair_step = [&](int pp) {
                const float4 a = sA[pp], b = sB[pp];
                const float2 xj = make_float2(a.x, a.y), yj = make_float2(a.z, a.w);
                const float2 zj = make_float2(b.x, b.y), mj = make_float2(b.z, b.w);
#pragma unroll
                for (int k = 0; k < K; k++) {
                    const float2 dx = __fadd2_rn(xj, nx[k]);
                    const float2 dy = __fadd2_rn(yj, ny[k]);
                    const float2 dz = __fadd2_rn(zj, nz[k]);
                    float2 r2 = __fmul2_rn(dx, dx);
                    r2 = __ffma2_rn(dy, dy, r2);
                    r2 = __ffma2_rn(dz, dz, r2);
                    mn[k] = fminf(mn[k], fminf(r2.x, r2.y));
                    const float2 inv = make_float2(rsqrt_sfu(r2.x), rsqrt_sfu(r2.y));
                    const float2 t = __fmul2_rn(mj, inv);
                    const float2 inv2 = __fmul2_rn(inv, inv);
                    const float2 s = __fmul2_rn(t, inv2);
                    ax[k] = __ffma2_rn(s, dx, ax[k]);
                    ay[k] = __ffma2_rn(s, dy, ay[k]);
                    az[k] = __ffma2_rn(s, dz, az[k]);
                }
            };
            /* a full tile keeps a constant trip count for the unroller */
            if (jpv == JP) {
#pragma unroll UNROLL
                for (int pp = 0; pp < JP; pp++) pair_step(pp);
            } else {
                for (int pp = 0; pp < jpv; pp++) pair_step(pp);
            }
#pragma unroll
            for (int k = 0; k < K; k++) {
                const float thk = THR(k);
                if (mn[k] < thk) {
                    /* slow path: this tile holds a near or overlapping pair for i */
                    const ll p = ibase + (ll)k * BLOCK + tid;
                    const ll i = perm[p];
                    const float4 hi_i = jhi[p], lo_i = jlo[p];
                    float tx = 0.f, ty = 0.f, tz = 0.f;
                    const float xi = -nx[k].x, yi = -ny[k].x, zi = -nz[k].x;
                    for (int pp = 0; pp < jpv; pp++) {
                        const float4 a = sA[pp], b = sB[pp];
#pragma unroll
                        for (int e = 0; e < 2; e++) {
                            const ll q = jt + 2 * pp + e;
                            if (q >= je || q == p) continue;
                            near_pass_j(A, ctl, ev_keys, ev_cap, perm, inv_ms, i, q, hi_i, lo_i, xi, yi, zi, thk,
                                        e ? a.y : a.x, e ? a.w : a.z, e ? b.y : b.x, e ? b.w : b.z,
                                        [&](ll qq, float4 &hj, float4 &lj) {
                                            hj = jhi[qq];
                                            lj = jlo[qq];
                                        },
                                        tx, ty, tz, FOLD(0, k), FOLD(1, k), FOLD(2, k), FOLD(3, k), FOLD(4, k),
                                        FOLD(5, k));
                        }
                    }
                    ax[k] = make_float2(tx, 0.f);
                    ay[k] = make_float2(ty, 0.f);
                    az[k] = make_float2(tz, 0.f);
                }
                two_sum_add(FOLD(0, k), FOLD(1, k), ax[k].x + ax[k].y);
                two_sum_add(FOLD(2, k), FOLD(3, k), ay[k].x + ay[k].y);
                two_sum_add(FOLD(4, k), FOLD(5, k), az[k].x + az[k].y);
            }
            if (BULK) {
                /* tile buffer buf ^ 1 was last read by the previous tile,
                 * before the last barrier */
                const bool ok = jt + JT < je ? unpack(jt + JT, buf ^ 1) : true;
                if (__syncthreads_or(!ok)) {
                    give_up();
                    return;
                }
                if (jt + 3 * JT < je) issue(jt + 3 * JT, buf ^ 1);
                buf ^= 1;
            } else if (DB) {
                /* the other buffer's last readers finished the previous tile
                 * before this tile's barrier */
                if (jt + JT < je) store_raw(buf ^ 1, jt + JT);
                buf ^= 1;
            }
        }
        /* this chunk's share of i-tile g: slot g + chunk */
        double *o = part + (g + chunk) * 3 * ITILE;
#pragma unroll
        for (int k = 0; k < K; k++) {
            const int li = k * BLOCK + tid;
            o[li] = (double)FOLD(0, k) + (double)FOLD(1, k);
            o[ITILE + li] = (double)FOLD(2, k) + (double)FOLD(3, k);
            o[2 * ITILE + li] = (double)FOLD(4, k) + (double)FOLD(5, k);
        }
        U += len;
    }
    }
#undef FOLD
#undef THR
}

/* f = (G m_i m_scale) * the sum of the chunks' shares of body p's i-tile, in
 * chunk order, written to body perm[p]. */
__global__ void k_mix_out(BodyArrays A, DevCtl *ctl, SimSegs seg, const unsigned *perm, const double *part,
                          int itile)
{
    if (ctl->error) return;
    const ll n = ctl->n;
    const int C = ctl->splits;
    const ll W = ctl->work_total;
    double ms = ctl->m_scale;
    if (!(ms > 0.0)) ms = 1.0;
    for (ll p = (ll)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (ll)gridDim.x * blockDim.x) {
        const ll i = perm[p];
        const unsigned f = A.flags[i];
        if ((f & NBG_LIVE_MASK) != NBG_F_EXISTS) continue;
        const double x = A.x[i], y = A.y[i], z = A.z[i], r = A.rad[i];
        if (is_special(x, y, z, r)) {
            /* NaN position or radius: every dist comparison fails, no force;
             * an infinite coordinate makes the reference's terms NaN */
            const bool has_nan = x != x || y != y || z != z || r != r;
            const double v = has_nan ? 0.0 : nbg_nan();
            A.fx[i] = v;
            A.fy[i] = v;
            A.fz[i] = v;
            continue;
        }
        const int sim = nbg_sim_of(seg.off, seg.nsims, p);
        const ll s0 = seg.off[sim], ns = seg.off[sim + 1] - s0;
        const ll t = (p - s0) / itile;
        const int li = (int)(p - s0 - t * itile);
        const ll g = seg.mtile_off[sim] + t;
        const ll tu = seg.item_off[sim] + t * ns; /* the tile's first unit */
        const int c0 = nbg_work_chunk(tu, C, W), c1 = nbg_work_chunk(tu + ns - 1, C, W);
        double sx = 0, sy = 0, sz = 0;
        for (int c = c0; c <= c1; c++) {
            const double *o = part + (g + c) * 3 * itile;
            sx += o[li];
            sy += o[itile + li];
            sz += o[2 * itile + li];
        }
        const double gm = NBG_G * A.m[i] * ms;
        A.fx[i] = gm * sx;
        A.fy[i] = gm * sy;
        A.fz[i] = gm * sz;
    }
}

/* ---- the symmetric pair kernel ---------------------------------------------
 * Gravity is antisymmetric, f_ji = -f_ij, so each unordered pair is computed
 * once and its term added to both bodies: 16 FMA-pipe lane operations per
 * pair where the one-sided kernel spends 12 per direction, 24 per pair.
 *
 * Work.  A collection's sorted bodies form blocks of SYM_B (the i-tiles of
 * the one-sided kernel, with the same origins and i-body set-up).  The
 * units are the block pairs (a, b), a <= b, of each collection, row by row:
 * row a holds (a, a) .. (a, T-1).  They are cut into chunks like the
 * one-sided work; a chunk keeps block a's bodies in registers along a row.
 *
 * An off-diagonal unit (a < b).  Block b is staged in shared memory,
 * re-centred on block a's origin.  Each warp holds 128 i-bodies (4 per lane)
 * and takes block b in sub-blocks of 64 j: each lane loads two j (one packed
 * f32x2 pair) and the j-pairs rotate through the warp's lanes with
 * shuffles, 32 steps, carrying their force sums, so every lane meets every
 * pair and every j-pair returns home with the sum of its 128 i-terms.  The
 * per-warp sums of the j meet in shared memory and are added in warp order;
 * the unit writes them as its own slot of FP32 j-partials.
 *
 * A diagonal unit (a == a) is one-sided: every body of the block against
 * every other, i-sums only (both directions of each pair are in the block).
 *
 * Near pairs.  A pair closer than the i-body's near-pair threshold (the one
 * the one-sided kernel uses, from the i-side error bound, which the shared dx
 * carries to both directions) is masked out of both fast sums.  After the
 * unit, the lanes that met one re-evaluate their near pairs exactly in FP64
 * (candidate_pair: the reference's expressions, the overlap skip, the event
 * i -> j), and the owners of the j that were met re-evaluate the same pairs
 * from their side (the event j -> i and the j term).  Both sides decide
 * "near" with the same FP32 expression, so they agree pair by pair.  Every
 * sum is formed in a fixed order: results do not depend on scheduling.
 *
 * Sums.  i-sums fold into (hi, lo) pairs every 256 j and go to the one-sided
 * kernel's per-(row, chunk) FP64 slots; j-sums of a unit (128 terms per
 * warp, 4 warps) go to the unit's FP32 slot.  k_sym_out adds a body's row
 * slots in chunk order, then its column's unit slots in row order, in FP64. */

#define SYM_THREADS 128
#define SYM_KI 4
#define SYM_B (SYM_THREADS * SYM_KI) /* 512 bodies per block */
#define SYM_WARPS (SYM_THREADS / 32)
#define SYM_JP (SYM_B / 2)    /* j pairs per block */
#define SYM_NSUB (SYM_B / 64) /* 64-j sub-blocks a warp rotates through */
#define SYM_FOLD 4            /* sub-blocks between folds of the i-sums */
static_assert(SYM_B == NBG_MIX_ITILE, "blocks are the i-tiles of the default shape");
static_assert(SYM_NSUB % SYM_FOLD == 0, "whole folds per unit");

/* first unit of row a in a collection of T blocks (rows a .. T-1 wide) */
__host__ __device__ __forceinline__ ll sym_row_start(ll a, ll T) { return a * T - a * (a - 1) / 2; }

/* row of unit v (0 <= v < T (T + 1) / 2) */
__device__ __forceinline__ ll sym_row_of(ll v, ll T)
{
    const double b = 2.0 * (double)T + 1.0;
    ll a = (ll)((b - sqrt(fmax(b * b - 8.0 * (double)v, 0.0))) * 0.5);
    a = a < 0 ? 0 : (a > T - 1 ? T - 1 : a);
    while (a > 0 && sym_row_start(a, T) > v) a--;
    while (a < T - 1 && sym_row_start(a + 1, T) <= v) a++;
    return a;
}

__device__ __forceinline__ float2 shfl2(float2 v, int src)
{
    return make_float2(__shfl_sync(FULL_MASK, v.x, src), __shfl_sync(FULL_MASK, v.y, src));
}

/* the FP32 near-pair decision and squared distance of one pair, as the fast
 * loops form it (so the exact passes find exactly the masked pairs) */
__device__ __forceinline__ float sym_r2(float xj, float yj, float zj, float nxi, float nyi, float nzi)
{
    const float dx = __fadd_rn(xj, nxi), dy = __fadd_rn(yj, nyi), dz = __fadd_rn(zj, nzi);
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

template <int MINB>
__global__ void __launch_bounds__(SYM_THREADS, MINB)
k_pair_sym(BodyArrays A, DevCtl *ctl, SimSegs seg, const float4 *__restrict__ jhi, const float4 *__restrict__ jlo,
           const float4 *__restrict__ tile_c, const float *__restrict__ tile_t, const float4 *__restrict__ iprep,
           const unsigned *__restrict__ perm, double *__restrict__ part, float *__restrict__ jpart, ull *ev_keys,
           ll ev_cap)
{
    /* block b, re-centred on block a's origin: j pair pp is (x0, x1, y0, y1),
     * (z0, z1, m0, m1) */
    __shared__ float4 sA[SYM_JP], sB[SYM_JP];
    __shared__ float2 jacc[SYM_WARPS][3][SYM_JP]; /* per-warp j sums of the unit */
    __shared__ float sfold[6][SYM_B];             /* i sums: (hi, lo) per component */
    __shared__ unsigned char jnear[SYM_B];        /* j met a near pair in this unit */
    __shared__ ll s_chunk;
    if (ctl->error) return;
    const int C = ctl->splits;
    const ll W = ctl->work_total;
    double ms = ctl->m_scale;
    if (!(ms > 0.0)) ms = 1.0;
    const double inv_ms = 1.0 / ms;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int src = (lane + 1) & 31;

    for (;;) {
    if (tid == 0) s_chunk = (ll)atomicAdd((unsigned long long *)&ctl->work_next, 1ull);
    __syncthreads();
    const ll chunk = s_chunk;
    __syncthreads();
    if (chunk >= C) break;
    ll U = nbg_chunk_start(chunk, C, W);
    const ll U1 = nbg_chunk_start(chunk + 1, C, W);
    int sim = U < W ? nbg_sim_of(seg.item_off, seg.nsims, U) : 0;
    while (U < U1) {
        while (seg.item_off[sim + 1] <= U) sim++;
        const ll s0 = seg.off[sim], n = seg.off[sim + 1];
        const ll T = seg.mtile_off[sim + 1] - seg.mtile_off[sim];
        const ll v = U - seg.item_off[sim];
        const ll a = sym_row_of(v, T);
        const ll b0 = a + (v - sym_row_start(a, T));
        const ll cnt = T - b0 < U1 - U ? T - b0 : U1 - U; /* units of row a in this chunk */
        const ll g = seg.mtile_off[sim] + a;
        const ll ibase = s0 + a * SYM_B;
        const float4 c = tile_c[g];

        /* block a: re-centred positions (negated, duplicated for the packed
         * arithmetic), thresholds, and masses (negated) for the j terms;
         * slots past the collection sit at the sentinel, massless */
        float2 nx[SYM_KI], ny[SYM_KI], nz[SYM_KI], nm[SYM_KI];
        float thr[SYM_KI];
#pragma unroll
        for (int k = 0; k < SYM_KI; k++) {
            const ll p = ibase + (ll)k * SYM_THREADS + tid;
            float xr = SENTINEL_POS, yr = SENTINEL_POS, zr = SENTINEL_POS, t = -1.f, m = 0.f;
            if (p < n) {
                const float4 q = iprep[p];
                xr = q.x;
                yr = q.y;
                zr = q.z;
                t = q.w;
                m = jhi[p].w;
            }
            nx[k] = make_float2(-xr, -xr);
            ny[k] = make_float2(-yr, -yr);
            nz[k] = make_float2(-zr, -zr);
            nm[k] = make_float2(-m, -m);
            thr[k] = t;
#pragma unroll
            for (int cc = 0; cc < 6; cc++) sfold[cc][k * SYM_THREADS + tid] = 0.f;
        }

        for (ll bb = b0; bb < b0 + cnt; bb++) {
            const ll u = U + (bb - b0); /* this unit's global index */
            const ll jb = s0 + bb * SYM_B;
            const bool diag = bb == a;
            __syncthreads(); /* the previous unit's readers are done */
            for (int sp = tid; sp < SYM_JP; sp += SYM_THREADS) {
                float vv[2][4];
#pragma unroll
                for (int e = 0; e < 2; e++) {
                    const ll q = jb + 2 * sp + e;
                    float4 h = make_float4(0.f, 0.f, 0.f, 0.f), l = h;
                    if (q < n) {
                        h = jhi[q];
                        l = jlo[q];
                    }
                    if (q < n && !packed_special(l)) {
                        vv[e][0] = (h.x - c.x) + l.x;
                        vv[e][1] = (h.y - c.y) + l.y;
                        vv[e][2] = (h.z - c.z) + l.z;
                        vv[e][3] = h.w;
                    } else {
                        vv[e][0] = vv[e][1] = vv[e][2] = SENTINEL_POS;
                        vv[e][3] = 0.f;
                    }
                    jnear[2 * sp + e] = 0;
                }
                sA[sp] = make_float4(vv[0][0], vv[1][0], vv[0][1], vv[1][1]);
                sB[sp] = make_float4(vv[0][2], vv[1][2], vv[0][3], vv[1][3]);
            }
            __syncthreads();

            float2 ax[SYM_KI], ay[SYM_KI], az[SYM_KI];
            unsigned nearmask = 0; /* bit k: i-body k met a near pair (besides itself) */
            int selfnear[SYM_KI];
#pragma unroll
            for (int k = 0; k < SYM_KI; k++) {
                ax[k] = ay[k] = az[k] = make_float2(0.f, 0.f);
                selfnear[k] = 0;
            }
            auto fold = [&]() {
#pragma unroll
                for (int k = 0; k < SYM_KI; k++) {
                    const int li = k * SYM_THREADS + tid;
                    two_sum_add(sfold[0][li], sfold[1][li], ax[k].x + ax[k].y);
                    two_sum_add(sfold[2][li], sfold[3][li], ay[k].x + ay[k].y);
                    two_sum_add(sfold[4][li], sfold[5][li], az[k].x + az[k].y);
                    ax[k] = ay[k] = az[k] = make_float2(0.f, 0.f);
                }
            };
            /* A unit whose blocks' bounding spheres lie farther apart than
             * block a's largest near-pair radius holds no near pair: its
             * loop needs no mask (uniform over the CTA). */
            bool far = false;
            if (!diag) {
                const float4 cj = tile_c[seg.mtile_off[sim] + bb];
                const float ex = cj.x - c.x, ey = cj.y - c.y, ez = cj.z - c.z;
                const float gap = sqrtf(ex * ex + ey * ey + ez * ez) * (1.0f - 0x1p-18f) - c.w - cj.w;
                far = gap > 0.f && gap * gap > tile_t[g] * (1.0f + 0x1p-10f);
            }
            auto rotate = [&](auto masked) {
                constexpr bool MASK = decltype(masked)::value;
                /* symmetric: rotate 64-j sub-blocks through the warp */
                for (int r = 0; r < SYM_NSUB; r++) {
                    const int pp0 = ((w + r) % SYM_NSUB) * 32 + lane;
                    const float4 qa = sA[pp0], qb = sB[pp0];
                    float2 xj = make_float2(qa.x, qa.y), yj = make_float2(qa.z, qa.w);
                    float2 zj = make_float2(qb.x, qb.y), mj = make_float2(qb.z, qb.w);
                    float2 fx = make_float2(0.f, 0.f), fy = fx, fz = fx;
#pragma unroll 2
                    for (int s = 0; s < 32; s++) {
#pragma unroll
                        for (int k = 0; k < SYM_KI; k++) {
                            const float2 dx = __fadd2_rn(xj, nx[k]);
                            const float2 dy = __fadd2_rn(yj, ny[k]);
                            const float2 dz = __fadd2_rn(zj, nz[k]);
                            float2 r2 = __fmul2_rn(dx, dx);
                            r2 = __ffma2_rn(dy, dy, r2);
                            r2 = __ffma2_rn(dz, dz, r2);
                            const float2 inv = make_float2(rsqrt_sfu(r2.x), rsqrt_sfu(r2.y));
                            float2 inv3 = __fmul2_rn(__fmul2_rn(inv, inv), inv);
                            if (MASK) {
                                const bool n0 = r2.x < thr[k], n1 = r2.y < thr[k];
                                if (n0 | n1) nearmask |= 1u << k;
                                inv3.x = n0 ? 0.f : inv3.x;
                                inv3.y = n1 ? 0.f : inv3.y;
                            }
                            const float2 si = __fmul2_rn(mj, inv3);
                            const float2 sj = __fmul2_rn(nm[k], inv3);
                            ax[k] = __ffma2_rn(si, dx, ax[k]);
                            ay[k] = __ffma2_rn(si, dy, ay[k]);
                            az[k] = __ffma2_rn(si, dz, az[k]);
                            fx = __ffma2_rn(sj, dx, fx);
                            fy = __ffma2_rn(sj, dy, fy);
                            fz = __ffma2_rn(sj, dz, fz);
                        }
                        /* the next lane's pair, with its sums, moves here */
                        xj = shfl2(xj, src);
                        yj = shfl2(yj, src);
                        zj = shfl2(zj, src);
                        mj = shfl2(mj, src);
                        fx = shfl2(fx, src);
                        fy = shfl2(fy, src);
                        fz = shfl2(fz, src);
                    }
                    /* 32 steps: the pair is home with the sums of all 128 i */
                    jacc[w][0][pp0] = fx;
                    jacc[w][1][pp0] = fy;
                    jacc[w][2][pp0] = fz;
                    if ((r + 1) % SYM_FOLD == 0) fold();
                }
            };
            if (!diag) {
                if (far)
                    rotate(std::false_type{});
                else
                    rotate(std::true_type{});
            } else {
                /* diagonal: one-sided over the block, pairs broadcast */
                for (int pp = 0; pp < SYM_JP; pp++) {
                    const float4 qa = sA[pp], qb = sB[pp];
                    const float2 xj = make_float2(qa.x, qa.y), yj = make_float2(qa.z, qa.w);
                    const float2 zj = make_float2(qb.x, qb.y), mj = make_float2(qb.z, qb.w);
#pragma unroll
                    for (int k = 0; k < SYM_KI; k++) {
                        const float2 dx = __fadd2_rn(xj, nx[k]);
                        const float2 dy = __fadd2_rn(yj, ny[k]);
                        const float2 dz = __fadd2_rn(zj, nz[k]);
                        float2 r2 = __fmul2_rn(dx, dx);
                        r2 = __ffma2_rn(dy, dy, r2);
                        r2 = __ffma2_rn(dz, dz, r2);
                        const bool n0 = r2.x < thr[k], n1 = r2.y < thr[k];
                        selfnear[k] += (int)n0 + (int)n1;
                        const float2 inv = make_float2(rsqrt_sfu(r2.x), rsqrt_sfu(r2.y));
                        float2 inv3 = __fmul2_rn(__fmul2_rn(inv, inv), inv);
                        inv3.x = n0 ? 0.f : inv3.x;
                        inv3.y = n1 ? 0.f : inv3.y;
                        const float2 si = __fmul2_rn(mj, inv3);
                        ax[k] = __ffma2_rn(si, dx, ax[k]);
                        ay[k] = __ffma2_rn(si, dy, ay[k]);
                        az[k] = __ffma2_rn(si, dz, az[k]);
                    }
                    if ((pp + 1) % 128 == 0) fold();
                }
                /* a live body's own pair is near (distance 0); one more is a
                 * genuine near pair */
#pragma unroll
                for (int k = 0; k < SYM_KI; k++)
                    if (selfnear[k] > 1) nearmask |= 1u << k;
            }

            /* exact pass, i side: this thread's near pairs, j in block order */
#pragma unroll
            for (int k = 0; k < SYM_KI; k++) {
                if (!(nearmask & (1u << k))) continue;
                const int li = k * SYM_THREADS + tid;
                const ll p = ibase + li;
                const ll i = perm[p];
                for (int jj = 0; jj < SYM_B; jj++) {
                    const ll q = jb + jj;
                    if (q >= n || (diag && jj == li)) continue;
                    const float4 qa = sA[jj >> 1], qb = sB[jj >> 1];
                    const int e = jj & 1;
                    const float r2 = sym_r2(e ? qa.y : qa.x, e ? qa.w : qa.z, e ? qb.y : qb.x, nx[k].x, ny[k].x,
                                            nz[k].x);
                    if (!(r2 < thr[k])) continue;
                    double tx, ty, tz;
                    candidate_pair(A, ctl, ev_keys, ev_cap, i, (ll)perm[q], inv_ms, tx, ty, tz);
                    fold64(sfold[0][li], sfold[1][li], tx);
                    fold64(sfold[2][li], sfold[3][li], ty);
                    fold64(sfold[4][li], sfold[5][li], tz);
                    jnear[jj] = 1;
                }
            }
            if (diag) continue; /* a diagonal unit has no j slot */
            __syncthreads(); /* jacc and jnear complete */

            /* j side: the unit's sums in warp order, plus the exact terms of
             * the j that met a near pair, i in block order */
            float *jo = jpart + u * 3 * SYM_B;
            for (int jj = tid; jj < SYM_B; jj += SYM_THREADS) {
                const int pp = jj >> 1, e = jj & 1;
                float sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll
                for (int ww = 0; ww < SYM_WARPS; ww++) {
                    sx += e ? jacc[ww][0][pp].y : jacc[ww][0][pp].x;
                    sy += e ? jacc[ww][1][pp].y : jacc[ww][1][pp].x;
                    sz += e ? jacc[ww][2][pp].y : jacc[ww][2][pp].x;
                }
                const ll q = jb + jj;
                if (jnear[jj] && q < n) {
                    const float4 qa = sA[pp], qb = sB[pp];
                    const float xj = e ? qa.y : qa.x, yj = e ? qa.w : qa.z, zj = e ? qb.y : qb.x;
                    const ll j = perm[q];
                    double ex = 0.0, ey = 0.0, ez = 0.0;
                    for (int ii = 0; ii < SYM_B; ii++) {
                        const ll p = ibase + ii;
                        if (p >= n) break;
                        const float4 ip = iprep[p];
                        const float r2 = sym_r2(xj, yj, zj, -ip.x, -ip.y, -ip.z);
                        if (!(r2 < ip.w)) continue;
                        double tx, ty, tz;
                        candidate_pair(A, ctl, ev_keys, ev_cap, j, (ll)perm[p], inv_ms, tx, ty, tz);
                        ex += tx;
                        ey += ty;
                        ez += tz;
                    }
                    sx = (float)((double)sx + ex);
                    sy = (float)((double)sy + ey);
                    sz = (float)((double)sz + ez);
                }
                jo[jj] = sx;
                jo[SYM_B + jj] = sy;
                jo[2 * SYM_B + jj] = sz;
            }
        }
        /* this chunk's share of row a's i sums: slot g + chunk */
        __syncthreads();
        double *o = part + (g + chunk) * 3 * SYM_B;
#pragma unroll
        for (int k = 0; k < SYM_KI; k++) {
            const int li = k * SYM_THREADS + tid;
            o[li] = (double)sfold[0][li] + (double)sfold[1][li];
            o[SYM_B + li] = (double)sfold[2][li] + (double)sfold[3][li];
            o[2 * SYM_B + li] = (double)sfold[4][li] + (double)sfold[5][li];
        }
        U += cnt;
    }
    }
}

/* f = (G m_i m_scale) * (body p's row slots in chunk order, then its
 * column's unit slots in row order), written to body perm[p]. */
__global__ void k_sym_out(BodyArrays A, DevCtl *ctl, SimSegs seg, const unsigned *perm, const double *part,
                          const float *jpart)
{
    if (ctl->error) return;
    const ll n = ctl->n;
    const int C = ctl->splits;
    const ll W = ctl->work_total;
    double ms = ctl->m_scale;
    if (!(ms > 0.0)) ms = 1.0;
    for (ll p = (ll)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (ll)gridDim.x * blockDim.x) {
        const ll i = perm[p];
        const unsigned f = A.flags[i];
        if ((f & NBG_LIVE_MASK) != NBG_F_EXISTS) continue;
        const double x = A.x[i], y = A.y[i], z = A.z[i], r = A.rad[i];
        if (is_special(x, y, z, r)) {
            const bool has_nan = x != x || y != y || z != z || r != r;
            const double vv = has_nan ? 0.0 : nbg_nan();
            A.fx[i] = vv;
            A.fy[i] = vv;
            A.fz[i] = vv;
            continue;
        }
        const int sim = nbg_sim_of(seg.off, seg.nsims, p);
        const ll s0 = seg.off[sim];
        const ll T = seg.mtile_off[sim + 1] - seg.mtile_off[sim];
        const ll a = (p - s0) / SYM_B;
        const int li = (int)(p - s0 - a * SYM_B);
        const ll g = seg.mtile_off[sim] + a;
        const ll u0 = seg.item_off[sim] + sym_row_start(a, T);
        const int c0 = nbg_work_chunk(u0, C, W), c1 = nbg_work_chunk(u0 + (T - a) - 1, C, W);
        double sx = 0, sy = 0, sz = 0;
        for (int cc = c0; cc <= c1; cc++) {
            const double *o = part + (g + cc) * 3 * SYM_B;
            sx += o[li];
            sy += o[SYM_B + li];
            sz += o[2 * SYM_B + li];
        }
        /* the column's unit slots (aa, a), rows in order, as FP32 (hi, lo)
         * TwoSum pairs: a column holds up to T - 1 slots (2,047 for 2^20
         * bodies), and FP64 adds, at 1/64 of the FP32 rate, bound this loop.
         * Unit (aa, a) is row_start(aa) + a - aa, and row_start(aa + 1) =
         * row_start(aa) + T - aa. */
        float hx = 0.f, lx = 0.f, hy = 0.f, ly = 0.f, hz = 0.f, lz = 0.f;
        const float *q = jpart + (seg.item_off[sim] + a) * 3 * SYM_B + li;
#pragma unroll 4
        for (ll aa = 0; aa < a; aa++) {
            two_sum_add(hx, lx, q[0]);
            two_sum_add(hy, ly, q[SYM_B]);
            two_sum_add(hz, lz, q[2 * SYM_B]);
            q += (T - aa - 1) * 3 * SYM_B;
        }
        sx += (double)hx + (double)lx;
        sy += (double)hy + (double)ly;
        sz += (double)hz + (double)lz;
        const double gm = NBG_G * A.m[i] * ms;
        A.fx[i] = gm * sx;
        A.fy[i] = gm * sy;
        A.fz[i] = gm * sz;
    }
}

/* ---- kernel shapes ---------------------------------------------------------
 * (kind, threads per CTA, i-bodies per thread, j per shared-memory tile,
 * unroll of the j loop, CTAs per SM the register budget is set for).  Kind 0:
 * sums in registers; 1: sums in shared memory; 2: sums in shared memory and
 * two tile buffers filled from registers loaded a tile ahead; 3: sums in
 * shared memory and two tile buffers re-centred from raw tiles that bulk
 * copies bring into shared memory two tiles ahead.  Shapes 15 and 16 are
 * the symmetric kernel's.  Variant 0 is the default; the autotuner
 * (nbg_autotune) measures the others. */
#define MIX_VARIANTS(X)              \
    X(0, 0, 128, 4, 256, 2, 3)       \
    X(1, 0, 128, 4, 256, 1, 3)       \
    X(2, 0, 128, 2, 256, 2, 4)       \
    X(3, 0, 256, 2, 256, 2, 2)       \
    X(4, 0, 128, 4, 512, 2, 3)       \
    X(5, 0, 64, 4, 256, 2, 6)        \
    X(6, 0, 128, 2, 128, 4, 4)       \
    X(7, 1, 128, 2, 256, 2, 5)       \
    X(8, 1, 128, 3, 256, 2, 4)       \
    X(9, 1, 128, 4, 256, 2, 4)       \
    X(10, 1, 128, 4, 128, 4, 4)      \
    X(11, 2, 128, 2, 128, 4, 4)      \
    X(12, 2, 128, 2, 256, 2, 4)      \
    X(13, 2, 128, 2, 128, 2, 4)      \
    X(14, 2, 128, 4, 128, 2, 3)      \
    X(17, 3, 128, 2, 256, 2, 5)      \
    X(18, 3, 128, 4, 256, 2, 4)

/* the kernel of a shape */
#define MIX_KERNEL(kind, b, k, jt, u, mb) k_pair_mixed<b, k, jt, u, mb, (kind) >= 1, (kind) == 2, (kind) == 3>

/* the symmetric kernel's shapes: registers capped for 4 or 5 CTAs per SM */
#define SYM_MINB_A 4
#define SYM_MINB_B 5

MixVariantInfo nbg_mix_variant_info(int variant)
{
    switch (variant) {
#define X(id, kind, b, k, jt, u, mb) \
    case id: return MixVariantInfo{b, k, jt, u};
        MIX_VARIANTS(X)
#undef X
    case NBG_MIX_SYM:
    case NBG_MIX_SYM + 1: return MixVariantInfo{SYM_THREADS, SYM_KI, SYM_B, 2};
    default: return MixVariantInfo{0, 0, 0, 0};
    }
}

/* resident CTAs of each shape per device, filled on first use (relaxed
 * atomics: threads driving contexts at once store the same value) */
static std::atomic<int> g_mixed_slots_cache[64][NBG_MIX_VARIANTS];

int nbg_mixed_slots(int device, int variant)
{
    if (variant < 0 || variant >= NBG_MIX_VARIANTS) variant = 0;
    if (device >= 0 && device < 64) {
        const int cached = g_mixed_slots_cache[device][variant].load(std::memory_order_relaxed);
        if (cached > 0) return cached;
    }
    int per_sm = 0, sms = 0;
    switch (variant) {
#define X(id, kind, b, k, jt, u, mb) \
    case id: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, MIX_KERNEL(kind, b, k, jt, u, mb), b, 0); break;
        MIX_VARIANTS(X)
#undef X
    case NBG_MIX_SYM:
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pair_sym<SYM_MINB_A>, SYM_THREADS, 0);
        break;
    case NBG_MIX_SYM + 1:
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pair_sym<SYM_MINB_B>, SYM_THREADS, 0);
        break;
    }
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    int slots = per_sm * sms;
    if (slots < 1) slots = 1;
    if (device >= 0 && device < 64) g_mixed_slots_cache[device][variant].store(slots, std::memory_order_relaxed);
    return slots;
}


void nbg_launch_mixed_prep(const CycleBufs &cb, DevCtl *ctl, cudaStream_t st)
{
    const int fg = nbg_flat_grid(cb, cb.cap);
    k_mix_reduce<<<fg, 256, 0, st>>>(cb.a, ctl, cb.seg);
    nbg_launch_spatial_sort(cb, ctl, st);
    k_mix_pack<<<fg, 256, 0, st>>>(cb.a, ctl, cb.perm, cb.jhi, cb.jlo);
    const int itile = cb.itile > 0 ? cb.itile : NBG_MIX_ITILE;
    ll tiles = (cb.cap + itile - 1) / itile + cb.seg.nsims;
    if (tiles > (ll)(cb.sms > 0 ? cb.sms : 1) * 64) tiles = (ll)(cb.sms > 0 ? cb.sms : 1) * 64;
    k_mix_tiles<<<(int)tiles, TILES_BLOCK, 0, st>>>(ctl, cb.seg, cb.jhi, cb.jlo, cb.tile_c, cb.tile_t, itile);
    k_mix_iprep<<<fg, 256, 0, st>>>(ctl, cb.seg, cb.jhi, cb.jlo, cb.tile_c, cb.iprep, cb.tile_t, itile);
}

void nbg_launch_mixed_pair(const CycleBufs &cb, DevCtl *ctl, cudaStream_t st)
{
    switch (cb.mix_variant) {
#define X(id, kind, b, k, jt, u, mb)                                                                       \
    case id:                                                                                           \
        MIX_KERNEL(kind, b, k, jt, u, mb)<<<cb.slots, b, 0, st>>>(cb.a, ctl, cb.seg, cb.jhi, cb.jlo, cb.tile_c, \
                                                                  cb.iprep, cb.perm, cb.part, cb.ev_keys,   \
                                                                  cb.ev_cap);                                \
        break;
        MIX_VARIANTS(X)
#undef X
    case NBG_MIX_SYM:
        k_pair_sym<SYM_MINB_A><<<cb.slots, SYM_THREADS, 0, st>>>(cb.a, ctl, cb.seg, cb.jhi, cb.jlo, cb.tile_c,
                                                                 cb.tile_t, cb.iprep, cb.perm, cb.part, cb.jpart,
                                                                 cb.ev_keys, cb.ev_cap);
        break;
    case NBG_MIX_SYM + 1:
        k_pair_sym<SYM_MINB_B><<<cb.slots, SYM_THREADS, 0, st>>>(cb.a, ctl, cb.seg, cb.jhi, cb.jlo, cb.tile_c,
                                                                 cb.tile_t, cb.iprep, cb.perm, cb.part, cb.jpart,
                                                                 cb.ev_keys, cb.ev_cap);
        break;
    }
}

void nbg_launch_mixed_out(const CycleBufs &cb, DevCtl *ctl, cudaStream_t st)
{
    if (nbg_mix_is_sym(cb.mix_variant))
        k_sym_out<<<nbg_flat_grid(cb, cb.cap), 256, 0, st>>>(cb.a, ctl, cb.seg, cb.perm, cb.part, cb.jpart);
    else
        k_mix_out<<<nbg_flat_grid(cb, cb.cap), 256, 0, st>>>(cb.a, ctl, cb.seg, cb.perm, cb.part,
                                                             cb.itile > 0 ? cb.itile : NBG_MIX_ITILE);
}

/* units of the symmetric kernel's work for a collection of T blocks */
ll nbg_sym_units(ll T) { return T * (T + 1) / 2; }
