/*
 * k_sort.cu - spatial ordering of the i-tiles of the mixed pair kernel.
 *
 * Every few cycles (k_sort_decide) the bodies are ordered along a Morton
 * (Z-order) curve over a 1024^3 grid of the symmetric bounding box
 * [-x_max, x_max]^3, and compaction carries the order along in between
 * (k_order_carry in k_cycle.cu): 30-bit keys,
 * sorted with a stable LSD radix sort (8-bit digits, four passes) whose
 * ranking within a block uses warp match masks, so the order is the same on
 * every run.  Consecutive 512-body slices of the sorted order are compact in
 * space; the pair kernel re-centres FP32 coordinates on each slice's origin,
 * which keeps their error at 2^-24 of the slice size instead of the system
 * size.  Only the i side uses the order: which j a tile reads, and in which
 * order, does not matter to the sum's accuracy.
 *
 * Bodies with a non-finite position or NaN radius sort last (key 2^30).
 */
#include "nbg_internal.cuh"

#define RS_BLOCK 256
#define RS_ITEMS 16
#define RS_TILE (RS_BLOCK * RS_ITEMS)
#define RS_BINS 256

__device__ __forceinline__ unsigned spread10(unsigned v)
{
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__device__ __forceinline__ unsigned quant10(float x, float inv_span)
{
    float t = (x * inv_span + 0.5f) * 1024.0f;
    t = fminf(fmaxf(t, 0.0f), 1023.0f);
    return (unsigned)t;
}

/* Keys of the bodies 0..n-1 and the identity permutation.  One sim: a 30-bit
 * Morton key over [-x_max, x_max]^3.  Several sims: the sim index in the top
 * 11 bits and a 21-bit Morton key over the sim's own box, so every sim keeps
 * its range of positions and is ordered inside it. */
__global__ void k_morton_keys(BodyArrays A, DevCtl *ctl, SimSegs seg, unsigned *keys, unsigned *vals)
{
    if (ctl->error || !ctl->sort_now) return;
    const ll n = ctl->n;
    const bool multi = seg.nsims > 1;
    for (ll k = (ll)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (ll)gridDim.x * blockDim.x) {
        const double x = A.x[k], y = A.y[k], z = A.z[k], r = A.rad[k];
        const bool finite = fabs(x) <= 1.7976931348623157e308 && fabs(y) <= 1.7976931348623157e308 &&
                            fabs(z) <= 1.7976931348623157e308 && r == r;
        unsigned key;
        if (!multi) {
            const float xmax = __uint_as_float(ctl->xmax_bits);
            const float inv_span = xmax > 0.f ? 0.5f / xmax : 0.f;
            key = 1u << 30;
            if (finite)
                key = spread10(quant10((float)x, inv_span)) | (spread10(quant10((float)y, inv_span)) << 1) |
                      (spread10(quant10((float)z, inv_span)) << 2);
        } else {
            const int sim = nbg_sim_of(seg.off, seg.nsims, k);
            const float xmax = __uint_as_float(seg.xmax_bits[sim]);
            const float inv_span = xmax > 0.f ? 0.5f / xmax : 0.f;
            unsigned m = 0x1fffffu;
            if (finite)
                m = (spread10(quant10((float)x, inv_span) >> 3) | (spread10(quant10((float)y, inv_span) >> 3) << 1) |
                     (spread10(quant10((float)z, inv_span) >> 3) << 2));
            key = ((unsigned)sim << 21) | m;
        }
        keys[k] = key;
        vals[k] = (unsigned)k;
    }
}

/* What a radix pass sorts.  RS_MORTON: the bodies' Morton keys (32-bit,
 * with the permutation as values), in cycles that sort.  RS_EVENTS: the
 * detected events' 64-bit keys i<<32 | j<<2 | type, when there are more than
 * the one-block sort of k_cycle.cu holds.  The count comes from the control
 * block, so one captured graph serves every count: passes with nothing to
 * sort return at once. */
#define RS_MORTON 0
#define RS_EVENTS 1
#define RS_INCIDENCES 2 /* two (body, event) keys per event, for the resolution's links */

__device__ __forceinline__ ll rs_count(const DevCtl *ctl, int what)
{
    if (ctl->error) return 0;
    if (what == RS_MORTON) return ctl->sort_now ? ctl->n : 0;
    if (ctl->ev_count <= NBG_EV_BLOCK_SORT) return 0;
    return what == RS_EVENTS ? ctl->ev_count : 2 * ctl->ev_count;
}

/* per-block digit histogram, digit-major: hist[d * nb + b] */
template <typename K>
__global__ void __launch_bounds__(RS_BLOCK) k_rs_hist(DevCtl *ctl, int what, const K *keys, int shift, ll *hist)
{
    __shared__ unsigned cnt[RS_BINS];
    const ll n = rs_count(ctl, what);
    if (n == 0) return;
    const ll nb = (n + RS_TILE - 1) / RS_TILE;
    const ll b = blockIdx.x;
    if (b >= nb) return;
    for (int d = threadIdx.x; d < RS_BINS; d += RS_BLOCK) cnt[d] = 0;
    __syncthreads();
    const ll base = b * RS_TILE;
    for (int q = 0; q < RS_ITEMS; q++) {
        ll k = base + (ll)q * RS_BLOCK + threadIdx.x;
        if (k < n) atomicAdd(&cnt[(unsigned)(keys[k] >> shift) & 0xffu], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < RS_BINS; d += RS_BLOCK) hist[(ll)d * nb + b] = cnt[d];
}

/* Exclusive scan of the digit-major histogram in three launches: per-chunk
 * sums, a scan of those sums (one block), and the scan of each chunk from its
 * offset.  A chunk is RS_SCAN_CHUNK entries; the chunk sums sit after the
 * histogram in the same buffer. */
#define RS_SCAN_ITEMS 8
#define RS_SCAN_CHUNK (1024 * RS_SCAN_ITEMS)

__device__ __forceinline__ ll rs_hist_total(const DevCtl *ctl, int what)
{
    return ((rs_count(ctl, what) + RS_TILE - 1) / RS_TILE) * RS_BINS;
}

/* block-wide inclusive scan of one value per thread (1024 threads) */
__device__ __forceinline__ ll rs_block_incl(ll x, ll *warp_tot, ll *block_total)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 1; o < 32; o <<= 1) {
        const ll y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
        ll t = warp_tot[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const ll y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        warp_tot[lane] = t;
    }
    __syncthreads();
    const ll r = x + (w > 0 ? warp_tot[w - 1] : 0);
    *block_total = warp_tot[31];
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(1024) k_rs_scan_part(DevCtl *ctl, int what, ll *hist)
{
    __shared__ ll warp_tot[32];
    const ll total = rs_hist_total(ctl, what);
    if (total == 0) return;
    const ll c0 = (ll)blockIdx.x * RS_SCAN_CHUNK;
    if (c0 >= total) return;
    ll s = 0;
    for (int q = 0; q < RS_SCAN_ITEMS; q++) {
        const ll c = c0 + (ll)q * 1024 + threadIdx.x;
        if (c < total) s += hist[c];
    }
    ll tot;
    rs_block_incl(s, warp_tot, &tot);
    if (threadIdx.x == 0) hist[total + blockIdx.x] = tot;
}

__global__ void __launch_bounds__(1024) k_rs_scan_top(DevCtl *ctl, int what, ll *hist)
{
    __shared__ ll warp_tot[32];
    const ll total = rs_hist_total(ctl, what);
    if (total == 0) return;
    const ll nchunk = (total + RS_SCAN_CHUNK - 1) / RS_SCAN_CHUNK;
    ll *sums = hist + total;
    ll carry = 0;
    for (ll b0 = 0; b0 < nchunk; b0 += 1024) {
        const ll b = b0 + threadIdx.x;
        const ll v = b < nchunk ? sums[b] : 0;
        ll tot;
        const ll inc = rs_block_incl(v, warp_tot, &tot);
        if (b < nchunk) sums[b] = carry + inc - v;
        carry += tot;
    }
}

__global__ void __launch_bounds__(1024) k_rs_scan_fin(DevCtl *ctl, int what, ll *hist)
{
    __shared__ ll warp_tot[32];
    const ll total = rs_hist_total(ctl, what);
    if (total == 0) return;
    const ll c0 = (ll)blockIdx.x * RS_SCAN_CHUNK;
    if (c0 >= total) return;
    /* thread t takes RS_SCAN_ITEMS consecutive entries */
    const ll c = c0 + (ll)threadIdx.x * RS_SCAN_ITEMS;
    ll v[RS_SCAN_ITEMS], s = 0;
#pragma unroll
    for (int q = 0; q < RS_SCAN_ITEMS; q++) {
        v[q] = c + q < total ? hist[c + q] : 0;
        s += v[q];
    }
    ll tot;
    ll ex = rs_block_incl(s, warp_tot, &tot) - s + hist[total + blockIdx.x];
#pragma unroll
    for (int q = 0; q < RS_SCAN_ITEMS; q++) {
        if (c + q < total) hist[c + q] = ex;
        ex += v[q];
    }
}

/* stable scatter: element order within a block is kept per digit (vals
 * NULL: keys only) */
template <typename K>
__global__ void __launch_bounds__(RS_BLOCK) k_rs_scatter(DevCtl *ctl, int what, const K *keys_in,
                                                        const unsigned *vals_in, K *keys_out, unsigned *vals_out,
                                                        int shift, const ll *offs)
{
    __shared__ ll base[RS_BINS];
    __shared__ unsigned wcnt[RS_BLOCK / 32][RS_BINS];
    const ll n = rs_count(ctl, what);
    if (n == 0) return;
    const ll nb = (n + RS_TILE - 1) / RS_TILE;
    const ll b = blockIdx.x;
    if (b >= nb) return;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int d = threadIdx.x; d < RS_BINS; d += RS_BLOCK) base[d] = offs[(ll)d * nb + b];
    const unsigned lt = (1u << lane) - 1u;
    for (int q = 0; q < RS_ITEMS; q++) {
        for (int d = threadIdx.x; d < RS_BINS * (RS_BLOCK / 32); d += RS_BLOCK) (&wcnt[0][0])[d] = 0;
        __syncthreads();
        const ll k = b * RS_TILE + (ll)q * RS_BLOCK + threadIdx.x;
        const bool ok = k < n;
        const K key = ok ? keys_in[k] : (K)0;
        const unsigned d = ok ? (unsigned)(key >> shift) & 0xffu : RS_BINS; /* RS_BINS never matches a real digit */
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const unsigned rank = __popc(peers & lt);
        if (ok && rank == 0) wcnt[w][d] = __popc(peers);
        __syncthreads();
        if (ok) {
            ll pos = base[d] + rank;
            for (int v = 0; v < w; v++) pos += wcnt[v][d];
            keys_out[pos] = key;
            if (vals_in) vals_out[pos] = vals_in[k];
        }
        __syncthreads();
        for (int dd = threadIdx.x; dd < RS_BINS; dd += RS_BLOCK) {
            ll s = 0;
            for (int v = 0; v < RS_BLOCK / 32; v++) s += wcnt[v][dd];
            base[dd] += s;
        }
        __syncthreads();
    }
}

/* the histogram plus its chunk sums */
ll nbg_sort_scratch_hist(ll cap)
{
    const ll h = ((cap + RS_TILE - 1) / RS_TILE) * RS_BINS;
    return h + (h + RS_SCAN_CHUNK - 1) / RS_SCAN_CHUNK;
}

/* Whether this cycle sorts.  Bodies move a small fraction of a tile's size
 * per cycle, so an order a few cycles old still gives compact tiles; which i
 * a tile holds never changes a result's correctness, only its FP32 error
 * and the near-pair count.  An order is dropped (sort_valid = 0) whenever a
 * body changes index or the arrays are replaced: compaction, loads, edits,
 * reallocation, and a cycle that failed and is run again. */
__global__ void k_sort_decide(DevCtl *ctl)
{
    if (ctl->error) return;
    const int k = ctl->sort_interval > 0 ? ctl->sort_interval : NBG_SORT_INTERVAL_DEFAULT;
    const bool now = !ctl->sort_valid || ctl->cycle - ctl->sort_cycle >= (ull)k;
    ctl->sort_now = now;
    if (now) {
        ctl->sort_valid = 1;
        ctl->sort_cycle = ctl->cycle;
    }
}

/* Leaves the sorted permutation in cb.perm (when this cycle sorts). */
void nbg_launch_spatial_sort(const CycleBufs &cb, DevCtl *ctl, cudaStream_t st)
{
    k_sort_decide<<<1, 1, 0, st>>>(ctl);
    const int g = nbg_flat_grid(cb, cb.cap);
    k_morton_keys<<<g, 256, 0, st>>>(cb.a, ctl, cb.seg, cb.skey[0], cb.perm);
    const int nb = (int)((cb.cap + RS_TILE - 1) / RS_TILE);
    const int nchunk = (int)(((ll)nb * RS_BINS + RS_SCAN_CHUNK - 1) / RS_SCAN_CHUNK);
    unsigned *kin = cb.skey[0], *vin = cb.perm, *kout = cb.skey[1], *vout = cb.sval;
    for (int pass = 0; pass < 4; pass++) {
        const int shift = 8 * pass;
        k_rs_hist<unsigned><<<nb, RS_BLOCK, 0, st>>>(ctl, RS_MORTON, kin, shift, cb.shist);
        k_rs_scan_part<<<nchunk, 1024, 0, st>>>(ctl, RS_MORTON, cb.shist);
        k_rs_scan_top<<<1, 1024, 0, st>>>(ctl, RS_MORTON, cb.shist);
        k_rs_scan_fin<<<nchunk, 1024, 0, st>>>(ctl, RS_MORTON, cb.shist);
        k_rs_scatter<unsigned><<<nb, RS_BLOCK, 0, st>>>(ctl, RS_MORTON, kin, vin, kout, vout, shift, cb.shist);
        unsigned *t = kin;
        kin = kout;
        kout = t;
        t = vin;
        vin = vout;
        vout = t;
    }
    /* four passes: the result is back in skey[0] / perm */
}

/* Events beyond the one-block sort: a stable LSD radix sort of their keys
 * i<<32 | j<<2 | type on the bits that hold j (from bit 2) and i (from bit
 * 32), 8-bit digits, between the event list and its ping-pong buffer.  An
 * ordered pair (i, j) is detected once, so (i, j) decides the order and the
 * type bits need no pass.  Digits may overlap (the last j digit reaches into
 * i's bits): the lexicographic order over the passes is still the key order.
 * The two halves take the same number of passes, so the result ends in the
 * event list. */
void nbg_launch_event_radix(const CycleBufs &cb, DevCtl *ctl, cudaStream_t st)
{
    int kb = 1; /* bits of a body index */
    while (kb < 31 && ((ll)1 << kb) < cb.cap) kb++;
    const int per_half = (kb + 7) / 8;
    const int nb = (int)((cb.ev_cap + RS_TILE - 1) / RS_TILE);
    const int nchunk = (int)(((ll)nb * RS_BINS + RS_SCAN_CHUNK - 1) / RS_SCAN_CHUNK);
    ull *kin = cb.ev_keys, *kout = cb.ev_sort;
    for (int pass = 0; pass < 2 * per_half; pass++) {
        const int shift = pass < per_half ? 2 + 8 * pass : 32 + 8 * (pass - per_half);
        k_rs_hist<ull><<<nb, RS_BLOCK, 0, st>>>(ctl, RS_EVENTS, kin, shift, cb.ev_hist);
        k_rs_scan_part<<<nchunk, 1024, 0, st>>>(ctl, RS_EVENTS, cb.ev_hist);
        k_rs_scan_top<<<1, 1024, 0, st>>>(ctl, RS_EVENTS, cb.ev_hist);
        k_rs_scan_fin<<<nchunk, 1024, 0, st>>>(ctl, RS_EVENTS, cb.ev_hist);
        k_rs_scatter<ull><<<nb, RS_BLOCK, 0, st>>>(ctl, RS_EVENTS, kin, nullptr, kout, nullptr, shift, cb.ev_hist);
        ull *t = kin;
        kin = kout;
        kout = t;
    }
}

/* launches of the multi-block event sort and, when they fit one key, the
 * resolution's links (nbg_launch_after_pair) */
int nbg_event_radix_launches(const CycleBufs &cb)
{
    int kb = 1, ob = 1;
    while (kb < 31 && ((ll)1 << kb) < cb.cap) kb++;
    while (ob < 40 && ((ll)1 << ob) < cb.ev_cap) ob++;
    int n = 2 * ((kb + 7) / 8) * 5;
    if (kb + ob + 1 <= 64) n += 4 + ((kb + ob + 7) / 8) * 5;
    return n;
}

/* The (body, event) incidence keys of the resolution's links (k_cycle.cu),
 * sorted on their body and event bits: `bits` above the lowest (which tells
 * the event's side) in 8-bit digits.  Returns the buffer holding the
 * result: inc[0] after an even number of passes, inc[1] after an odd. */
ull *nbg_launch_incidence_radix(const CycleBufs &cb, DevCtl *ctl, int bits, cudaStream_t st)
{
    const ll cap2 = 2 * cb.ev_cap;
    const int nb = (int)((cap2 + RS_TILE - 1) / RS_TILE);
    const int nchunk = (int)(((ll)nb * RS_BINS + RS_SCAN_CHUNK - 1) / RS_SCAN_CHUNK);
    ull *kin = cb.inc[0], *kout = cb.inc[1];
    for (int shift = 1; shift < 1 + bits; shift += 8) {
        k_rs_hist<ull><<<nb, RS_BLOCK, 0, st>>>(ctl, RS_INCIDENCES, kin, shift, cb.inc_hist);
        k_rs_scan_part<<<nchunk, 1024, 0, st>>>(ctl, RS_INCIDENCES, cb.inc_hist);
        k_rs_scan_top<<<1, 1024, 0, st>>>(ctl, RS_INCIDENCES, cb.inc_hist);
        k_rs_scan_fin<<<nchunk, 1024, 0, st>>>(ctl, RS_INCIDENCES, cb.inc_hist);
        k_rs_scatter<ull><<<nb, RS_BLOCK, 0, st>>>(ctl, RS_INCIDENCES, kin, nullptr, kout, nullptr, shift,
                                                   cb.inc_hist);
        ull *t = kin;
        kin = kout;
        kout = t;
    }
    return kin;
}
