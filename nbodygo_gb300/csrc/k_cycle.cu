/*
 * k_cycle.cu - kernels of one compute cycle except the mixed-precision pair
 * kernel: the plain FP64 pair kernel, fragment emission, event ordering,
 * collision resolution, integration, compaction, and the cycle-boundary
 * edits (RemoveBodies, ModBody, GetBody).
 *
 * This file must be compiled with --fmad=false (and -DNBG_NO_FMAD): every
 * FP64 expression then rounds after each operation exactly like the
 * reference's Go code on amd64, which is what makes the plain path
 * bit-identical to the CPU oracle.
 */
#ifndef NBG_NO_FMAD
#error "k_cycle.cu must be compiled with --fmad=false -DNBG_NO_FMAD"
#endif

#include "nbg_internal.cuh"
#include "nbg_math.h"
#include "nbg_shared.h"

#define FULL_MASK 0xffffffffu

/* ------------------------------------------------------------------------ */
/* block-wide exclusive scan (blockDim.x == NBG_SCAN_BLOCK)                 */
/* ------------------------------------------------------------------------ */

__device__ static ll block_excl_scan(ll v, ll *total)
{
    __shared__ ll warp_tot[NBG_SCAN_BLOCK / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    ll x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        ll y = __shfl_up_sync(FULL_MASK, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
        ll t = warp_tot[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            ll y = __shfl_up_sync(FULL_MASK, t, o);
            if (lane >= o) t += y;
        }
        warp_tot[lane] = t;
    }
    __syncthreads();
    ll excl = x - v + (w > 0 ? warp_tot[w - 1] : 0);
    *total = warp_tot[NBG_SCAN_BLOCK / 32 - 1];
    __syncthreads();
    return excl;
}

/* Exclusive scan of f(0..ns-1) into out[0..ns-1], out[ns] = total, by one
 * block of NBG_SCAN_BLOCK threads; returns the total to every thread. */
template <typename F>
__device__ static ll block_scan_array(int ns, F f, ll *out)
{
    ll carry = 0;
    for (int s0 = 0; s0 < ns; s0 += NBG_SCAN_BLOCK) {
        const int s = s0 + (int)threadIdx.x;
        const ll v = s < ns ? f(s) : 0;
        ll tot;
        const ll ex = block_excl_scan(v, &tot);
        if (s < ns) out[s] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) out[ns] = carry;
    __syncthreads();
    return carry;
}

/* ------------------------------------------------------------------------ */
/* cycle start                                                              */
/* ------------------------------------------------------------------------ */

/* Per-cycle resets and the work layout of every sim: 64-body tiles of the
 * plain kernel; i-tiles and the pair work of the mixed kernel, and the chunks
 * it is cut into (C: NBG_MIX_CHUNKS_PER_CTA per resident CTA, or work_cap,
 * at least NBG_MIX_MIN_WORK units each, and few enough that the partial-sum
 * slots fit in part_doubles); the interaction count.  One block. */
__global__ void __launch_bounds__(NBG_SCAN_BLOCK) k_begin(DevCtl *ctl, SimSegs seg, int slots, int work_cap, int itile,
                                                          ll part_doubles, int sym, ll jpart_units)
{
    if (ctl->error) return;
    const int ns = seg.nsims;
    const ll *off = seg.off;
    for (int s = threadIdx.x; s < ns; s += NBG_SCAN_BLOCK) {
        seg.keep[s] = 0;
        seg.frag[s] = 0;
        seg.xmax_bits[s] = 0;
    }
    block_scan_array(ns, [&](int s) { return (off[s + 1] - off[s] + 63) / 64; }, seg.tile_off);
    const ll mtiles = block_scan_array(
        ns, [&](int s) { return (off[s + 1] - off[s] + itile - 1) / itile; }, seg.mtile_off);
    /* one-sided kernel: (i-tile, j-body) units; symmetric kernel: the
     * (block, block) pairs a <= b of each collection, T (T + 1) / 2 of them */
    const ll W = block_scan_array(
        ns,
        [&](int s) {
            const ll T = seg.mtile_off[s + 1] - seg.mtile_off[s];
            return sym ? T * (T + 1) / 2 : T * (off[s + 1] - off[s]);
        },
        seg.item_off);
    ll P = (ll)slots * NBG_MIX_CHUNKS_PER_CTA;
    if (work_cap > 0 && P > work_cap) P = work_cap;
    /* every chunk must hold work: the smallest guided chunk is W / (3 P) */
    if (P > W / (sym ? 4 : NBG_MIX_MIN_WORK)) P = W / (sym ? 4 : NBG_MIX_MIN_WORK);
    const ll part_slots = part_doubles / (3ll * itile);
    if (P > part_slots - mtiles + 1) P = part_slots - mtiles + 1;
    if (P < 1) P = 1;
    const bool part_short = mtiles + P - 1 > part_slots;
    /* interactions: sum of n_s (n_s - 1), reusing the keep_start array */
    const ll inter = block_scan_array(
        ns, [&](int s) { const ll m = off[s + 1] - off[s]; return m * (m > 0 ? m - 1 : 0); }, seg.keep_start);
    if (threadIdx.x == 0) {
        ll n = ctl->n;
        ctl->n_before = n;
        ctl->ev_count = 0;
        ctl->frag_total = 0;
        ctl->n_keep = n;
        ctl->rend_n = 0;
        ctl->last_ev_n = 0;
        ctl->rmax_bits = 0;
        ctl->xmax_bits = 0;
        ctl->m_scale = 0.0;
        ctl->splits = (int)P;
        ctl->work_total = W;
        ctl->work_next = 0;
        for (int c = 0; c < 3; c++) {
            ctl->bh_lo[c] = ~0ull;
            ctl->bh_hi[c] = 0ull;
        }
        ctl->bh_count = 0;
        ctl->bh_nodes = 0;
        ctl->bh_rmax = 0ull;
        ctl->bh_next = 0;
        ctl->cycle_interactions = inter;
        if (part_short) {
            ctl->error = NBG_E_OVERFLOW;
            ctl->error_what = 4;
            ctl->error_need = (mtiles + P - 1) * 3ll * itile;
        } else if (sym && W > jpart_units) {
            ctl->error = NBG_E_OVERFLOW;
            ctl->error_what = 6;
            ctl->error_need = W;
        }
    }
}

/* Fragments body k emits this cycle: Compute calls fragment() for a body that
 * exists and is fragmenting (body.go:148-154); the loop of fragcalc.go:96-111
 * emits min(fragments, 101) when fragments > 0. */
__device__ static ll frag_emit_count(const BodyArrays &A, ll k)
{
    unsigned f = A.flags[k];
    if ((f & NBG_LIVE_MASK) != NBG_LIVE_MASK) return 0;
    ll c = A.fr_cnt[k];
    if (c <= 0) return 0;
    return c < NBG_MAX_FRAGS_PER_CYCLE + 1 ? c : NBG_MAX_FRAGS_PER_CYCLE + 1;
}

/* Adds `v` to counter[sim] once per group of lanes that share `sim` (sim < 0:
 * nothing).  Every lane of the warp must call it. */
__device__ static void warp_add_per_sim(ll *counter, int sim, unsigned v)
{
    const unsigned peers = __match_any_sync(FULL_MASK, sim);
    const unsigned t = __reduce_add_sync(peers, v);
    if (sim >= 0 && (int)(threadIdx.x & 31) == __ffs(peers) - 1 && t != 0)
        atomicAdd((unsigned long long *)&counter[sim], (ull)t);
}

__global__ void __launch_bounds__(NBG_SCAN_BLOCK) k_frag_blocksum(BodyArrays A, DevCtl *ctl, SimSegs seg,
                                                                  ll *blk_sum)
{
    if (ctl->error) return;
    const ll n = ctl->n;
    const ll base = (ll)blockIdx.x * NBG_SCAN_TILE;
    if (base >= n) return;
    ll s = 0;
    for (int q = 0; q < NBG_SCAN_ITEMS; q++) {
        ll k = base + (ll)threadIdx.x * NBG_SCAN_ITEMS + q;
        if (k < n) {
            const ll c = frag_emit_count(A, k);
            s += c;
            if (c > 0) atomicAdd((unsigned long long *)&seg.frag[nbg_sim_of(seg.off, seg.nsims, k)], (ull)c);
        }
    }
    ll tot;
    block_excl_scan(s, &tot);
    if (threadIdx.x == 0) blk_sum[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(NBG_SCAN_BLOCK) k_keep_blocksum(BodyArrays A, DevCtl *ctl, SimSegs seg,
                                                                  ll *blk_sum)
{
    if (ctl->error) return;
    const ll n = ctl->n;
    const ll base = (ll)blockIdx.x * NBG_SCAN_TILE;
    if (base >= n) return;
    ll s = 0;
    for (int q = 0; q < NBG_SCAN_ITEMS; q++) {
        /* consecutive lanes take consecutive bodies so a warp mostly sees one sim */
        const ll k = base + (ll)q * NBG_SCAN_BLOCK + threadIdx.x;
        const bool keep = k < n && (A.flags[k] & NBG_F_EXISTS);
        s += keep ? 1 : 0;
        warp_add_per_sim(seg.keep, keep ? nbg_sim_of(seg.off, seg.nsims, k) : -1, keep ? 1 : 0);
    }
    ll tot;
    block_excl_scan(s, &tot);
    if (threadIdx.x == 0) blk_sum[blockIdx.x] = tot;
}

/* Single-block exclusive scan of the per-block sums, then the per-sim
 * layout.  mode 0: fragment counts, fragment and host-add starts per sim,
 * capacity checks.  mode 1: surviving bodies, keep starts and the layout
 * after Cycle: sim s gets [kept bodies][its fragments][its host adds].
 * mode 2: the block offsets alone. */
__global__ void __launch_bounds__(NBG_SCAN_BLOCK) k_scan_blocks(DevCtl *ctl, SimSegs seg, const ll *blk_sum,
                                                                ll *blk_off, int mode, ll cap, ll frag_cap)
{
    if (ctl->error) return;
    const ll n = ctl->n;
    const ll nb = (n + NBG_SCAN_TILE - 1) / NBG_SCAN_TILE;
    ll carry = 0;
    for (ll b0 = 0; b0 < nb; b0 += NBG_SCAN_BLOCK) {
        ll b = b0 + threadIdx.x;
        ll v = b < nb ? blk_sum[b] : 0;
        ll tot;
        ll ex = block_excl_scan(v, &tot);
        if (b < nb) blk_off[b] = carry + ex;
        carry += tot;
    }
    const int ns = seg.nsims;
    if (mode == 2) return; /* block offsets only (the carried order) */
    if (mode == 0) {
        block_scan_array(ns, [&](int s) { return seg.frag[s]; }, seg.frag_start);
        const ll hadds = block_scan_array(ns, [&](int s) { return seg.hadd[s]; }, seg.hadd_start);
        if (threadIdx.x == 0) {
            ctl->frag_total = carry;
            ctl->n_host_adds = hadds;
            ll need = n + carry + hadds;
            if (carry > frag_cap) {
                ctl->error = NBG_E_OVERFLOW;
                ctl->error_what = 3;
                ctl->error_need = carry;
            } else if (need > cap) {
                ctl->error = NBG_E_OVERFLOW;
                ctl->error_what = 1;
                ctl->error_need = need;
            }
        }
    } else {
        block_scan_array(ns, [&](int s) { return seg.keep[s]; }, seg.keep_start);
        block_scan_array(ns, [&](int s) { return seg.keep[s] + seg.frag[s] + seg.hadd[s]; }, seg.new_off);
        if (threadIdx.x == 0) ctl->n_keep = carry;
    }
}

/* ------------------------------------------------------------------------ */
/* K1: plain FP64 force + collision detection                              */
/* ------------------------------------------------------------------------ */

#define P64_BLOCK 64

/* Detection rule of Compute's second pass (body.go:172-186) for a pair with
 * Collided(i, j) true. Returns the event type or -1. */
/*
 * One thread per body i.  For each j in array order (tiles of P64_BLOCK staged
 * in shared memory) it evaluates exactly the reference's expressions
 * (calcForceFrom, body.go:214-225): the sum runs over j in ascending order,
 * so the result is bit-identical to the sequential loop.  The same dist
 * decides Collided (body.go:192-208); hits are appended to the event list.
 */
__global__ void __launch_bounds__(P64_BLOCK) k_pair_fp64(BodyArrays A, DevCtl *ctl, SimSegs seg, ull *ev_keys,
                                                          ll ev_cap)
{
    __shared__ double sx[P64_BLOCK], sy[P64_BLOCK], sz[P64_BLOCK], sm[P64_BLOCK], sr[P64_BLOCK];
    __shared__ unsigned sf[P64_BLOCK];
    if (ctl->error) return;
    const ll ntiles = seg.tile_off[seg.nsims];
    for (ll T = blockIdx.x; T < ntiles; T += gridDim.x) {
        /* tile T of sim s: i in [s0 + 64 t, ...), j over the sim [s0, s1) */
        const int sim = nbg_sim_of(seg.tile_off, seg.nsims, T);
        const ll s0 = seg.off[sim], n = seg.off[sim + 1];
        const ll i = s0 + (T - seg.tile_off[sim]) * P64_BLOCK + threadIdx.x;
        const bool valid = i < n;
        double xi = 0, yi = 0, zi = 0, mi = 0, ri = 0;
        unsigned fi = 0;
        if (valid) {
            xi = A.x[i];
            yi = A.y[i];
            zi = A.z[i];
            mi = A.m[i];
            ri = A.rad[i];
            fi = A.flags[i];
        }
        const bool live_i = valid && (fi & NBG_LIVE_MASK) == NBG_F_EXISTS;
        const bool coll_i = (fi & NBG_F_COLLIDED) != 0;
        const unsigned bi = NBG_BEHAVIOR(fi);
        const double gmi = NBG_G * mi;
        double fx = 0.0, fy = 0.0, fz = 0.0;
        for (ll j0 = s0; j0 < n; j0 += P64_BLOCK) {
            __syncthreads();
            const ll jl = j0 + threadIdx.x;
            if (jl < n) {
                sx[threadIdx.x] = A.x[jl];
                sy[threadIdx.x] = A.y[jl];
                sz[threadIdx.x] = A.z[jl];
                sm[threadIdx.x] = A.m[jl];
                sr[threadIdx.x] = A.rad[jl];
                sf[threadIdx.x] = A.flags[jl];
            }
            __syncthreads();
            if (!live_i) continue;
            const int cnt = (n - j0) < P64_BLOCK ? (int)(n - j0) : P64_BLOCK;
            /* unrolled: the divisions and square roots of later j overlap;
             * the sum still runs in j order */
#pragma unroll 4
            for (int t = 0; t < cnt; t++) {
                const ll j = j0 + t;
                const double dx = sx[t] - xi;
                const double dy = sy[t] - yi;
                const double dz = sz[t] - zi;
                const double dist = sqrt(dx * dx + dy * dy + dz * dz);
                const double rr = ri + sr[t];
                const unsigned fj = sf[t];
                const bool live_j = (fj & NBG_LIVE_MASK) == NBG_F_EXISTS;
                if (live_j && j != i && (coll_i || dist > rr)) {
                    const double force = gmi * sm[t] / (dist * dist);
                    fx += force * dx / dist;
                    fy += force * dy / dist;
                    fz += force * dz / dist;
                }
                if (!coll_i && dist <= rr && j != i) {
                    int type = nbg_detect_event(bi, NBG_BEHAVIOR(fj), ri, sr[t], dist);
                    if (type >= 0) nbg_emit_event(ctl, ev_keys, ev_cap, i, j, type);
                }
            }
        }
        if (live_i) {
            A.fx[i] = fx;
            A.fy[i] = fy;
            A.fz[i] = fz;
        }
    }
}

/* Small collections: one thread per body leaves most of the GPU idle (1,000
 * bodies fill 16 SMs), and FP64 runs at 1/64 of the FP32 rate.  So the pair
 * terms are computed for all (i, j) at once and stored, then each body adds
 * its terms in j order: the same expressions, the same additions in the same
 * order, so the result is bit-identical to k_pair_fp64.  A term that the
 * reference skips is stored as +0.0, and adding +0.0 changes no sum here
 * (the sum starts at +0.0 and can never be -0.0).  j runs in passes of jc;
 * the sums are carried between passes in acc.  One collection. */
/* P64_JS: j per block of k_p64_terms.  Many small blocks keep the FP64
 * pipes fed: 16 j (64 measured 2 % slower from 8,192 to 32,768 bodies), and
 * 4 for capacities up to 8,192, where the whole pass is only a few thousand
 * warps of long FP64 division chains. */
template <int P64_JS>
__global__ void __launch_bounds__(P64_BLOCK) k_p64_terms(BodyArrays A, DevCtl *ctl, double *T, ll cap, ll jc,
                                                         ll jbase, ull *ev_keys, ll ev_cap)
{
    __shared__ double sx[P64_JS], sy[P64_JS], sz[P64_JS], sm[P64_JS], sr[P64_JS];
    __shared__ unsigned sf[P64_JS];
    if (ctl->error) return;
    const ll n = ctl->n;
    /* this pass's j: to the end of the collection and of the pass */
    const ll jend = jbase + jc < n ? jbase + jc : n;
    if (jbase >= jend) return;
    /* work items (block of 64 i, block of P64_JS j) of the live bodies only:
     * a grid sized for the capacity would be mostly empty blocks */
    const ll nib = (n + P64_BLOCK - 1) / P64_BLOCK;
    const ll items = nib * ((jend - jbase + P64_JS - 1) / P64_JS);
    double *tx = T, *ty = T + jc * cap, *tz = T + 2 * jc * cap;
    for (ll w = blockIdx.x; w < items; w += gridDim.x) {
        const ll i = (w % nib) * P64_BLOCK + threadIdx.x;
        const ll j0 = jbase + (w / nib) * P64_JS;
        const ll jl = j0 + threadIdx.x;
        __syncthreads(); /* the previous item's readers are done */
        if (threadIdx.x < P64_JS && jl < jend) {
            sx[threadIdx.x] = A.x[jl];
            sy[threadIdx.x] = A.y[jl];
            sz[threadIdx.x] = A.z[jl];
            sm[threadIdx.x] = A.m[jl];
            sr[threadIdx.x] = A.rad[jl];
            sf[threadIdx.x] = A.flags[jl];
        }
        __syncthreads();
        if (i >= n) continue;
        const double xi = A.x[i], yi = A.y[i], zi = A.z[i], mi = A.m[i], ri = A.rad[i];
        const unsigned fi = A.flags[i];
        const bool live_i = (fi & NBG_LIVE_MASK) == NBG_F_EXISTS;
        const bool coll_i = (fi & NBG_F_COLLIDED) != 0;
        const unsigned bi = NBG_BEHAVIOR(fi);
        const double gmi = NBG_G * mi;
        const int cnt = (jend - j0) < P64_JS ? (int)(jend - j0) : P64_JS;
        for (int t = 0; t < cnt; t++) {
            const ll j = j0 + t;
            const ll slot = (j - jbase) * cap + i; /* a warp's stores are contiguous */
            double ex = 0.0, ey = 0.0, ez = 0.0;
            if (live_i) {
                const double dx = sx[t] - xi;
                const double dy = sy[t] - yi;
                const double dz = sz[t] - zi;
                const double dist = sqrt(dx * dx + dy * dy + dz * dz);
                const double rr = ri + sr[t];
                const unsigned fj = sf[t];
                const bool live_j = (fj & NBG_LIVE_MASK) == NBG_F_EXISTS;
                if (live_j && j != i && (coll_i || dist > rr)) {
                    const double force = gmi * sm[t] / (dist * dist);
                    ex = force * dx / dist;
                    ey = force * dy / dist;
                    ez = force * dz / dist;
                }
                if (!coll_i && dist <= rr && j != i) {
                    const int type = nbg_detect_event(bi, NBG_BEHAVIOR(fj), ri, sr[t], dist);
                    if (type >= 0) nbg_emit_event(ctl, ev_keys, ev_cap, i, j, type);
                }
            }
            tx[slot] = ex;
            ty[slot] = ey;
            tz[slot] = ez;
        }
    }
}

/* Each body adds its terms in j order.  A block takes 32 bodies: all its
 * threads load a tile of 32 j x 32 bodies x 3 components (coalesced rows of
 * 32 bodies), the next tile's loads go out while this one is added, and
 * three warps add the columns in j order, one force component each (FP64
 * adds run at 1/64 of the FP32 rate, so one warp adding all three left most
 * of the SM's FP64 units idle).  Each component's sum is formed exactly as
 * the sequential loop forms it. */
#define SUM_BODIES 32
#define SUM_J 32
#define SUM_THREADS 256
#define SUM_PER_THREAD (3 * SUM_J * SUM_BODIES / SUM_THREADS)
__global__ void __launch_bounds__(SUM_THREADS, 4) k_p64_sum(BodyArrays A, DevCtl *ctl, const double *T, double *acc,
                                                         ll cap, ll jc, ll jbase)
{
    __shared__ double tile[3][SUM_J][SUM_BODIES];
    if (ctl->error) return;
    const ll n = ctl->n;
    if (jbase >= n && jbase > 0) return;
    const ll je = jbase + jc < n ? jbase + jc : n;
    const ll cnt = je - jbase;
    const int tid = threadIdx.x;
    const int comp = tid / SUM_BODIES; /* warps 0-2: the component this thread adds */
    const bool adder = comp < 3;
    for (ll i0 = (ll)blockIdx.x * SUM_BODIES; i0 < n; i0 += (ll)gridDim.x * SUM_BODIES) {
        const ll i = i0 + (tid & (SUM_BODIES - 1));
        double f = 0.0;
        if (adder && jbase > 0 && i < n) f = acc[(ll)comp * cap + i];
        /* element e of a tile: component e / 1024, row (e / 32) % 32, body e % 32 */
        double r[SUM_PER_THREAD];
        auto load = [&](ll jt) {
#pragma unroll
            for (int q = 0; q < SUM_PER_THREAD; q++) {
                const int e = tid + q * SUM_THREADS;
                const int c = e / (SUM_J * SUM_BODIES), row = (e / SUM_BODIES) % SUM_J, b = e % SUM_BODIES;
                const ll j = jt + row, ib = i0 + b;
                r[q] = (j < cnt && ib < n) ? T[(ll)c * jc * cap + j * cap + ib] : 0.0;
            }
        };
        load(0);
        for (ll jt = 0; jt < cnt; jt += SUM_J) {
            __syncthreads(); /* the previous tile is added */
#pragma unroll
            for (int q = 0; q < SUM_PER_THREAD; q++) {
                const int e = tid + q * SUM_THREADS;
                tile[e / (SUM_J * SUM_BODIES)][(e / SUM_BODIES) % SUM_J][e % SUM_BODIES] = r[q];
            }
            __syncthreads();
            if (jt + SUM_J < cnt) load(jt + SUM_J);
            if (adder) {
                const int m = cnt - jt < SUM_J ? (int)(cnt - jt) : SUM_J;
                const int b = tid & (SUM_BODIES - 1);
                for (int t = 0; t < m; t++) f += tile[comp][t][b];
            }
        }
        if (adder && i < n) {
            if (je >= n) {
                if ((A.flags[i] & NBG_LIVE_MASK) == NBG_F_EXISTS) (comp == 0 ? A.fx : comp == 1 ? A.fy : A.fz)[i] = f;
            } else {
                acc[(ll)comp * cap + i] = f;
            }
        }
        __syncthreads(); /* the tile is free for the next bodies */
    }
}

/* ------------------------------------------------------------------------ */
/* K4: order the events (i ascending, then j)                               */
/* ------------------------------------------------------------------------ */

#define SORT_BLOCK 1024
#define SORT_SMEM NBG_EV_BLOCK_SORT

/* Orders the cycle's events by key (i, then j): up to SORT_SMEM in shared
 * memory by one block.  More are left to the multi-block radix sort that
 * follows when radix_follows is set; otherwise this block sorts them in
 * global memory (bitonic, slow but correct). */
__global__ void __launch_bounds__(SORT_BLOCK) k_sort_events(DevCtl *ctl, ull *keys, ll cap, int radix_follows)
{
    __shared__ ull s[SORT_SMEM];
    __shared__ int bail;
    if (threadIdx.x == 0) {
        bail = ctl->error != 0;
        if (!bail && ctl->ev_count > cap) {
            ctl->error = NBG_E_OVERFLOW;
            ctl->error_what = 2;
            ctl->error_need = ctl->ev_count;
            bail = 1;
        }
        if (!bail && ctl->ev_count > ctl->acc_ev_max) ctl->acc_ev_max = ctl->ev_count;
    }
    __syncthreads();
    if (bail) return;
    const ll cnt = ctl->ev_count;
    if (cnt <= 1 || (cnt > SORT_SMEM && radix_follows)) return;
    ll P = 1;
    while (P < cnt) P <<= 1;
    ull *d = keys;
    if (P <= SORT_SMEM) {
        d = s;
        for (ll k = threadIdx.x; k < P; k += SORT_BLOCK) s[k] = k < cnt ? keys[k] : ~0ull;
    } else {
        for (ll k = cnt + threadIdx.x; k < P; k += SORT_BLOCK) keys[k] = ~0ull;
    }
    __syncthreads();
    for (ll kk = 2; kk <= P; kk <<= 1) {
        for (ll jj = kk >> 1; jj > 0; jj >>= 1) {
            for (ll idx = threadIdx.x; idx < P; idx += SORT_BLOCK) {
                ll ixj = idx ^ jj;
                if (ixj > idx) {
                    bool asc = (idx & kk) == 0;
                    ull a = d[idx], b = d[ixj];
                    if ((a > b) == asc) {
                        d[idx] = b;
                        d[ixj] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
    if (P <= SORT_SMEM)
        for (ll k = threadIdx.x; k < cnt; k += SORT_BLOCK) keys[k] = s[k];
}

/* ------------------------------------------------------------------------ */
/* K8: fragment emission (fragcalc.go:94-117)                               */
/* ------------------------------------------------------------------------ */

__global__ void __launch_bounds__(NBG_SCAN_BLOCK) k_frag_emit(BodyArrays A, BodyArrays F, DevCtl *ctl, const ll *blk_off)
{
    if (ctl->error) return;
    const ll n = ctl->n;
    const ll base = (ll)blockIdx.x * NBG_SCAN_TILE;
    if (base >= n) return;
    ll c[NBG_SCAN_ITEMS];
    ll s = 0;
    for (int q = 0; q < NBG_SCAN_ITEMS; q++) {
        ll k = base + (ll)threadIdx.x * NBG_SCAN_ITEMS + q;
        c[q] = k < n ? frag_emit_count(A, k) : 0;
        s += c[q];
    }
    ll tot;
    ll off = block_excl_scan(s, &tot) + blk_off[blockIdx.x];
    const ll id0 = ctl->next_id;
    const ull seed = ctl->seed, cycle = ctl->cycle;
    for (int q = 0; q < NBG_SCAN_ITEMS; q++) {
        ll k = base + (ll)threadIdx.x * NBG_SCAN_ITEMS + q;
        if (k >= n) break;
        unsigned fk = A.flags[k];
        if ((fk & NBG_LIVE_MASK) != NBG_LIVE_MASK) continue;
        /* for (; fragments > 0;) { fragments--; emit; cnt++; if cnt > 100 break } */
        const ll parent = A.id[k];
        const ull key = nbg_frag_key(seed, parent, cycle);
        const double cx = A.fr_cx[k], cy = A.fr_cy[k], cz = A.fr_cz[k];
        const double rad9 = A.fr_rad[k] * .9;
        for (ll e = 0; e < c[q]; e++) {
            double px, py, pz;
            nbg_frag_point(key, (int)e, cx, cy, cz, rad9, &px, &py, &pz);
            const ll slot = off + e;
            F.id[slot] = id0 + slot;
            F.x[slot] = px;
            F.y[slot] = py;
            F.z[slot] = pz;
            F.vx[slot] = A.vx[k];
            F.vy[slot] = A.vy[k];
            F.vz[slot] = A.vz[k];
            F.m[slot] = A.fr_mass[k];
            F.rad[slot] = A.fr_newrad[k];
            F.fx[slot] = 0;
            F.fy[slot] = 0;
            F.fz[slot] = 0;
            F.ff[slot] = 0;
            F.fs[slot] = 0;
            F.rest[slot] = 0;
            F.fr_rad[slot] = 0;
            F.fr_newrad[slot] = 0;
            F.fr_mass[slot] = 0;
            F.fr_cx[slot] = 0;
            F.fr_cy[slot] = 0;
            F.fr_cz[slot] = 0;
            F.fr_cnt[slot] = 0;
            F.flags[slot] = NBG_F_EXISTS | ((unsigned)NBG_ELASTIC << NBG_BEHAVIOR_SHIFT);
        }
        off += c[q];
        ll left = A.fr_cnt[k] - c[q];
        A.fr_cnt[k] = left;
        if (left <= 0) A.flags[k] = fk & ~NBG_F_EXISTS;
    }
}

/* ------------------------------------------------------------------------ */
/* K5: collision resolution, one thread, newest event first                 */
/* ------------------------------------------------------------------------ */

struct ElasticOut {
    bool collided;
    double vx1, vy1, vz1, vx2, vy2, vz2, vx_cm, vy_cm, vz_cm;
};

/* calcElasticCollision, collisioncalc.go:42-186 (coll3d), on bodies b and o. */
__device__ static ElasticOut elastic_calc(const BodyArrays &A, ll b, ll o)
{
    ElasticOut res;
    res.collided = false;
    res.vx1 = res.vy1 = res.vz1 = res.vx2 = res.vy2 = res.vz2 = 0;
    res.vx_cm = res.vy_cm = res.vz_cm = 0;
    const double m1 = A.m[b], m2 = A.m[o], r1 = A.rad[b], r2 = A.rad[o];
    const double x1 = A.x[b], y1 = A.y[b], z1 = A.z[b];
    const double X2 = A.x[o], Y2 = A.y[o], Z2 = A.z[o];
    const double ux1 = A.vx[b], uy1 = A.vy[b], uz1 = A.vz[b];
    const double vx2 = A.vx[o], vy2 = A.vy[o], vz2 = A.vz[o];

    const double r12 = r1 + r2;
    const double m21 = m2 / m1;
    const double x21 = X2 - x1, y21 = Y2 - y1, z21 = Z2 - z1;
    const double vx21 = vx2 - ux1, vy21 = vy2 - uy1, vz21 = vz2 - uz1;
    const double vx_cm = (m1 * ux1 + m2 * vx2) / (m1 + m2);
    const double vy_cm = (m1 * uy1 + m2 * vy2) / (m1 + m2);
    const double vz_cm = (m1 * uz1 + m2 * vz2) / (m1 + m2);
    const double d = sqrt(x21 * x21 + y21 * y21 + z21 * z21);
    const double v = sqrt(vx21 * vx21 + vy21 * vy21 + vz21 * vz21);
    if (v == 0) return res;
    /* ball 1 at the origin, ball 2 at rest */
    const double px = x21, py = y21, pz = z21;
    const double wx = -vx21, wy = -vy21, wz = -vz21;
    const double theta2 = nbg_acos(pz / d);
    const double phi2 = (px == 0 && py == 0) ? 0.0 : nbg_atan2(py, px);
    const double st = nbg_sin(theta2), ct = nbg_cos(theta2);
    const double sp = nbg_sin(phi2), cp = nbg_cos(phi2);
    double vx1r = ct * cp * wx + ct * sp * wy - st * wz;
    double vy1r = cp * wy - sp * wx;
    double vz1r = st * cp * wx + st * sp * wy + ct * wz;
    double fvz1r = vz1r / v;
    if (fvz1r > 1)
        fvz1r = 1;
    else if (fvz1r < -1)
        fvz1r = -1;
    const double thetav = nbg_acos(fvz1r);
    const double phiv = (vx1r == 0 && vy1r == 0) ? 0.0 : nbg_atan2(vy1r, vx1r);
    const double dr = d * nbg_sin(thetav) / r12;
    if (thetav > NBG_PIO2_HI || fabs(dr) > 1) return res;
    const double alpha = nbg_asin(-dr);
    const double beta = phiv;
    const double sbeta = nbg_sin(beta), cbeta = nbg_cos(beta);
    const double a = nbg_tan(thetav + alpha);
    const double dvz2 = 2 * (vz1r + a * (cbeta * vx1r + sbeta * vy1r)) / ((1 + a * a) * (1 + m21));
    const double vz2r = dvz2;
    const double vx2r = a * cbeta * dvz2;
    const double vy2r = a * sbeta * dvz2;
    vz1r = vz1r - m21 * vz2r;
    vx1r = vx1r - m21 * vx2r;
    vy1r = vy1r - m21 * vy2r;
    res.collided = true;
    res.vx1 = ct * cp * vx1r - sp * vy1r + st * cp * vz1r + vx2;
    res.vy1 = ct * sp * vx1r + cp * vy1r + st * sp * vz1r + vy2;
    res.vz1 = ct * vz1r - st * vx1r + vz2;
    res.vx2 = ct * cp * vx2r - sp * vy2r + st * cp * vz2r + vx2;
    res.vy2 = ct * sp * vx2r + cp * vy2r + st * sp * vz2r + vy2;
    res.vz2 = ct * vz2r - st * vx2r + vz2;
    res.vx_cm = vx_cm;
    res.vy_cm = vy_cm;
    res.vz_cm = vz_cm;
    return res;
}

/* initiateFragmentation, fragcalc.go:67-85.  newRadius is always 1: Go
 * evaluates the exponent 1/3 as integer division (0) and Pow(x, 0) == 1. */
__device__ static void initiate_frag(BodyArrays &A, ll b, double fragFactor)
{
    const double ffb = A.ff[b];
    const double fragDelta = ffb > 10 ? 10.0 : fragFactor - ffb;
    const double fragments = nbg_go_min(fragDelta * A.fs[b], NBG_MAX_FRAGS);
    unsigned f = A.flags[b];
    if (fragments <= 1) {
        A.flags[b] = (f & ~(3u << NBG_BEHAVIOR_SHIFT)) | ((unsigned)NBG_FRAGMENT << NBG_BEHAVIOR_SHIFT);
        return;
    }
    A.flags[b] = f | NBG_F_FRAGMENTING;
    A.fr_rad[b] = A.rad[b];
    A.fr_newrad[b] = 1.0;
    A.fr_mass[b] = A.m[b] / fragments;
    A.fr_cnt[b] = fragments != fragments ? 0 : (ll)fragments; /* int(NaN): no fragment either way */
    A.fr_cx[b] = A.x[b];
    A.fr_cy[b] = A.y[b];
    A.fr_cz[b] = A.z[b];
}

/* ResolveCollision, body.go:248-264, with shouldFragment / doFragment /
 * doElastic (fragcalc.go:24-61, collisioncalc.go:26-35). */
__device__ static void resolve_collision(BodyArrays &A, ll b, ll o)
{
    const unsigned fb = A.flags[b], fo = A.flags[o];
    if (!(fb & NBG_F_EXISTS) || !(fo & NBG_F_EXISTS)) return;
    const unsigned bb = NBG_BEHAVIOR(fb), bo = NBG_BEHAVIOR(fo);
    if (!(bb == NBG_ELASTIC && (bo == NBG_ELASTIC || bo == NBG_FRAGMENT))) return;
    const ElasticOut r = elastic_calc(A, b, o);
    if (!r.collided) return;
    const double rb = A.rest[b];
    const double nvx1 = (r.vx1 - r.vx_cm) * rb + r.vx_cm;
    const double nvy1 = (r.vy1 - r.vy_cm) * rb + r.vy_cm;
    const double nvz1 = (r.vz1 - r.vz_cm) * rb + r.vz_cm;
    const double nvx2 = (r.vx2 - r.vx_cm) * rb + r.vx_cm;
    const double nvy2 = (r.vy2 - r.vy_cm) * rb + r.vy_cm;
    const double nvz2 = (r.vz2 - r.vz_cm) * rb + r.vz_cm;
    bool frag = false;
    double tf = 0, of = 0;
    if (bb == NBG_FRAGMENT || bo == NBG_FRAGMENT) {
        const double vThis = A.vx[b] + A.vy[b] + A.vz[b];
        const double dvThis = fabs(A.vx[b] - nvx1) + fabs(A.vy[b] - nvy1) + fabs(A.vz[b] - nvz1);
        const double thisFactor = dvThis / fabs(vThis);
        const double vOther = A.vx[o] + A.vy[o] + A.vz[o];
        const double dvOther = fabs(A.vx[o] - nvx2) + fabs(A.vy[o] - nvy2) + fabs(A.vz[o] - nvz2);
        const double otherFactor = dvOther / fabs(vOther);
        if ((bb == NBG_FRAGMENT && thisFactor > A.ff[b]) || (bo == NBG_FRAGMENT && otherFactor > A.ff[o])) {
            frag = true;
            tf = thisFactor;
            of = otherFactor;
        }
    }
    if (frag) {
        if (bb == NBG_FRAGMENT && tf > A.ff[b]) initiate_frag(A, b, tf);
        if (NBG_BEHAVIOR(A.flags[o]) == NBG_FRAGMENT && of > A.ff[o]) initiate_frag(A, o, of);
        return;
    }
    A.vx[b] = nvx1;
    A.vy[b] = nvy1;
    A.vz[b] = nvz1;
    A.vx[o] = nvx2;
    A.vy[o] = nvy2;
    A.vz[o] = nvz2;
    A.flags[b] |= NBG_F_COLLIDED;
    A.flags[o] |= NBG_F_COLLIDED;
}

/* ResolveSubsume, body.go:228-244 (no Exists checks, radius unchanged). */
__device__ static void resolve_subsume(BodyArrays &A, ll b, ll o)
{
    const double thisMass = A.m[b], otherMass = A.m[o];
    A.m[b] = thisMass + otherMass;
    A.m[o] = 0;
    A.flags[o] &= ~NBG_F_EXISTS;
}

/* first index of sorted keys[0..cnt) that is >= v */
__device__ static ll lower_bound_u64(const ull *keys, ll cnt, ull v)
{
    ll lo = 0, hi = cnt;
    while (lo < hi) {
        const ll mid = (lo + hi) >> 1;
        if (keys[mid] < v)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

/* ProcessMods (body_collection.go:213-235): each sim resolves its own events
 * newest first.  Events of one sim only touch that sim's bodies, and the
 * sorted keys are grouped by sim (i ranges).
 *
 * One CTA per sim.  Resolving an event reads and writes only its two bodies,
 * so the sequential order only matters between events that share a body:
 * the CTA resolves in rounds, and in each round every pending event that is
 * the oldest pending one (in processing order) on both of its bodies is
 * resolved, all such events in parallel.  Every body sees its events in the
 * sequential order, so the result is the sequential result bit for bit.
 * owner[] (one word per body; any contents on entry) holds, per round, the
 * smallest pending processing index that touches the body.  Once a round
 * resolves fewer than RESOLVE_MIN_ROUND events (a long chain through one
 * body, as when a large body absorbs many), one thread finishes the rest in
 * order.  ev_out holds the sims one after another, each in processing order;
 * its pad field marks pending events during the kernel and is 0 on return. */
#define RESOLVE_BLOCK 256
#define RESOLVE_MIN_ROUND 8 /* fewer events resolved in a round: finish sequentially */

__device__ static void event_bodies(ull key, ll &b1, ll &b2, unsigned &type)
{
    const ll i = (ll)(key >> 32);
    const ll j = (ll)((key >> 2) & 0x3fffffffull);
    type = (unsigned)(key & 3ull);
    b1 = i;
    b2 = j;
    if (type == NBG_EVT_SUB_JI) {
        b1 = j;
        b2 = i;
    }
}

__device__ static void resolve_one(BodyArrays &A, ull key, nbg_event *out)
{
    ll b1, b2;
    unsigned type;
    event_bodies(key, b1, b2, type);
    nbg_event e;
    e.id1 = A.id[b1];
    e.id2 = A.id[b2];
    e.type = type == NBG_EVT_COLL_IJ ? NBG_EV_COLLISION : NBG_EV_SUBSUME;
    e.pad = 0;
    if (type == NBG_EVT_COLL_IJ)
        resolve_collision(A, b1, b2);
    else
        resolve_subsume(A, b1, b2);
    *out = e;
}

/* ---- resolution links: the events of a busy cycle in dataflow order ------
 * ProcessMods resolves events one after another, newest first.  Two events
 * that share no body commute, so an event may be resolved as soon as every
 * earlier event on each of its bodies is: the per-body chains of events in
 * processing order are the only order that matters.  For cycles with more
 * events than the one-block sort holds, the chains are built from the sorted
 * (body, event) incidences, and k_resolve works through the ready events
 * round by round, touching only those - the result is the sequential one
 * bit for bit, however many events resolve at once. */

__device__ __forceinline__ bool links_on(const DevCtl *ctl)
{
    return ctl->error == 0 && ctl->ev_count > NBG_EV_BLOCK_SORT;
}

/* sim s holds the sorted events [ev_lo[s], ev_lo[s + 1]) */
__global__ void k_ev_ranges(DevCtl *ctl, SimSegs seg, const ull *keys, ll *ev_lo)
{
    if (!links_on(ctl)) return;
    const ll cnt = ctl->ev_count;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s <= seg.nsims; s += gridDim.x * blockDim.x)
        ev_lo[s] = s == seg.nsims ? cnt : (s == 0 ? 0 : lower_bound_u64(keys, cnt, (ull)seg.off[s] << 32));
}

/* The two incidences of the event at sorted position t, processing index o
 * (its sim's events in reverse key order): body << (ob + 1) | o << 1 | side */
__global__ void k_ev_incid(DevCtl *ctl, SimSegs seg, const ull *keys, const ll *ev_lo, ull *inc, int ob)
{
    if (!links_on(ctl)) return;
    const ll cnt = ctl->ev_count;
    for (ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x; t < cnt; t += (ll)gridDim.x * blockDim.x) {
        const ull key = keys[t];
        ll b1, b2;
        unsigned ty;
        event_bodies(key, b1, b2, ty);
        const int s = seg.nsims == 1 ? 0 : nbg_sim_of(seg.off, seg.nsims, (ll)(key >> 32));
        const ull o = (ull)(ev_lo[s] + ev_lo[s + 1] - 1 - t);
        inc[2 * t] = ((ull)b1 << (ob + 1)) | (o << 1);
        inc[2 * t + 1] = ((ull)b2 << (ob + 1)) | (o << 1) | 1ull;
    }
}

/* From the sorted incidences: each event's next event on each of its bodies
 * (link[2 o + side], -1: none) and previous one (pred[2 o + side]). */
__global__ void k_ev_links(DevCtl *ctl, const ull *inc, int ob, ll *link, ll *pred)
{
    if (!links_on(ctl)) return;
    const ll m2 = 2 * ctl->ev_count;
    const ull omask = (1ull << ob) - 1ull;
    for (ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x; t < m2; t += (ll)gridDim.x * blockDim.x) {
        const ull k = inc[t];
        const ull b = k >> (ob + 1);
        const ll slot = 2 * (ll)((k >> 1) & omask) + (ll)(k & 1ull);
        link[slot] = t + 1 < m2 && (inc[t + 1] >> (ob + 1)) == b ? (ll)((inc[t + 1] >> 1) & omask) : -1;
        pred[slot] = t > 0 && (inc[t - 1] >> (ob + 1)) == b ? (ll)((inc[t - 1] >> 1) & omask) : -1;
    }
}

/* unresolved predecessors of each event: one per body, once if both bodies'
 * previous event is the same */
__global__ void k_ev_pending(DevCtl *ctl, const ll *pred, int *pend)
{
    if (!links_on(ctl)) return;
    const ll m = ctl->ev_count;
    for (ll o = (ll)blockIdx.x * blockDim.x + threadIdx.x; o < m; o += (ll)gridDim.x * blockDim.x) {
        const ll p0 = pred[2 * o], p1 = pred[2 * o + 1];
        pend[o] = (p0 >= 0 ? 1 : 0) + (p1 >= 0 && p1 != p0 ? 1 : 0);
    }
}

/* Resolution of one sim's events through its links: round by round, every
 * ready event (all earlier events on its bodies resolved) at once. */
__device__ static void resolve_dataflow(BodyArrays &A, DevCtl *ctl, const ull *keys, nbg_event *ev_out, ll lo, ll hi,
                                        const ll *link, int *pend, ll *front, ll ev_cap)
{
    __shared__ ll s_n[2];
    __shared__ ll s_total;
    const int tid = threadIdx.x;
    ll *fr[2] = {front + lo, front + ev_cap + lo};
    if (tid == 0) {
        s_n[0] = s_n[1] = 0;
        s_total = 0;
    }
    __syncthreads();
    for (ll o = lo + tid; o < hi; o += RESOLVE_BLOCK)
        if (pend[o] == 0) fr[0][atomicAdd((unsigned long long *)&s_n[0], 1ull)] = o;
    __syncthreads();
    int cur = 0;
    ll done = 0;
    while (s_n[cur] > 0) {
        const ll nr = s_n[cur];
        if (nr == 1) {
            /* a chain (one body in every event): one thread follows it for
             * as long as each event readies exactly one successor, without
             * a barrier per event */
            if (tid == 0) {
                ll o = fr[cur][0];
                for (;;) {
                    resolve_one(A, keys[lo + hi - 1 - o], &ev_out[o]);
                    done++;
                    const ll n0 = link[2 * o], n1 = link[2 * o + 1];
                    ll rd[2];
                    int nready = 0;
                    if (n0 >= 0 && atomicSub(&pend[n0], 1) == 1) rd[nready++] = n0;
                    if (n1 >= 0 && n1 != n0 && atomicSub(&pend[n1], 1) == 1) rd[nready++] = n1;
                    if (nready == 1) {
                        o = rd[0];
                        continue;
                    }
                    for (int q = 0; q < nready; q++) fr[cur ^ 1][s_n[cur ^ 1]++] = rd[q];
                    break;
                }
            }
        } else
        for (ll x = tid; x < nr; x += RESOLVE_BLOCK) {
            const ll o = fr[cur][x];
            resolve_one(A, keys[lo + hi - 1 - o], &ev_out[o]);
            done++;
            const ll n0 = link[2 * o], n1 = link[2 * o + 1];
            if (n0 >= 0 && atomicSub(&pend[n0], 1) == 1)
                fr[cur ^ 1][atomicAdd((unsigned long long *)&s_n[cur ^ 1], 1ull)] = n0;
            if (n1 >= 0 && n1 != n0 && atomicSub(&pend[n1], 1) == 1)
                fr[cur ^ 1][atomicAdd((unsigned long long *)&s_n[cur ^ 1], 1ull)] = n1;
        }
        __syncthreads(); /* this round's bodies are written, the next frontier complete */
        if (tid == 0) s_n[cur] = 0;
        cur ^= 1;
        __syncthreads();
    }
    atomicAdd((unsigned long long *)&s_total, (ull)done);
    __syncthreads();
    /* every event has a chain of predecessors back to a ready one, so all
     * resolve; anything else is a broken invariant, reported as such */
    if (tid == 0 && s_total != (ull)(hi - lo)) {
        ctl->error = NBG_E_STATE;
        ctl->error_what = 7;
        ctl->error_need = hi - lo - (ll)s_total;
    }
}

__global__ void __launch_bounds__(RESOLVE_BLOCK) k_resolve(BodyArrays A, DevCtl *ctl, SimSegs seg, const ull *keys,
                                                           nbg_event *ev_out, unsigned *owner, int links,
                                                           const ll *ev_lo, const ll *link, int *pend, ll *front,
                                                           ll ev_cap)
{
    __shared__ int s_left, s_done;
    if (ctl->error) return;
    const ll cnt = ctl->ev_count;
    const int s = blockIdx.x;
    const int tid = threadIdx.x;
    if (s == 0 && tid == 0) {
        ctl->next_id += ctl->frag_total; /* fragments took ids next_id .. next_id+total-1 */
        ctl->last_ev_n = cnt;
        ctl->acc_events += cnt;
        ctl->acc_frags += ctl->frag_total;
    }
    if (s >= seg.nsims) return;
    if (links && cnt > NBG_EV_BLOCK_SORT) {
        const ll lo = ev_lo[s], hi = ev_lo[s + 1];
        if (hi > lo) resolve_dataflow(A, ctl, keys, ev_out, lo, hi, link, pend, front, ev_cap);
        return;
    }
    const ll lo = seg.nsims == 1 ? 0 : lower_bound_u64(keys, cnt, (ull)seg.off[s] << 32);
    const ll hi = seg.nsims == 1 ? cnt : lower_bound_u64(keys, cnt, (ull)seg.off[s + 1] << 32);
    const ll m = hi - lo;
    if (m <= 0) return;
    if (m == 1) {
        if (tid == 0) resolve_one(A, keys[lo], &ev_out[lo]);
        return;
    }
    /* processing index p is keys[hi - 1 - p], written to ev_out[lo + p] */
    for (ll p = tid; p < m; p += RESOLVE_BLOCK) ev_out[lo + p].pad = 1;
    if (tid == 0) s_left = (int)(m < 0x7fffffff ? m : 0x7fffffff);
    __syncthreads();
    for (ll round = 0; round < m; round++) {
        for (ll p = tid; p < m; p += RESOLVE_BLOCK) {
            if (ev_out[lo + p].pad) {
                ll b1, b2;
                unsigned ty;
                event_bodies(keys[hi - 1 - p], b1, b2, ty);
                owner[b1] = 0xffffffffu;
                owner[b2] = 0xffffffffu;
            }
        }
        __syncthreads();
        for (ll p = tid; p < m; p += RESOLVE_BLOCK) {
            if (ev_out[lo + p].pad) {
                ll b1, b2;
                unsigned ty;
                event_bodies(keys[hi - 1 - p], b1, b2, ty);
                atomicMin(&owner[b1], (unsigned)p);
                atomicMin(&owner[b2], (unsigned)p);
            }
        }
        if (tid == 0) s_done = 0;
        __syncthreads();
        int done = 0;
        for (ll p = tid; p < m; p += RESOLVE_BLOCK) {
            if (ev_out[lo + p].pad) {
                const ull key = keys[hi - 1 - p];
                ll b1, b2;
                unsigned ty;
                event_bodies(key, b1, b2, ty);
                if (owner[b1] == (unsigned)p && owner[b2] == (unsigned)p) {
                    resolve_one(A, key, &ev_out[lo + p]); /* clears pad */
                    done++;
                }
            }
        }
        if (done) atomicAdd(&s_done, done);
        __syncthreads();
        if (tid == 0) s_left -= s_done;
        __syncthreads();
        if (s_left <= 0) return;
        /* a chain of events on shared bodies: a round no longer pays for itself */
        if (s_done < RESOLVE_MIN_ROUND) break;
    }
    /* the rest in processing order, one thread: every pending event's
     * predecessors are resolved or come before it */
    if (tid == 0)
        for (ll p = 0; p < m; p++)
            if (ev_out[lo + p].pad) resolve_one(A, keys[hi - 1 - p], &ev_out[lo + p]);
}

/* ------------------------------------------------------------------------ */
/* K6: integration (Update, body.go:114-139) + renderables                 */
/* ------------------------------------------------------------------------ */

__global__ void k_integrate(BodyArrays A, DevCtl *ctl, nbg_renderable *rend, nbg_renderable *ring_rend, ll ring_cap,
                            int ring_slots)
{
    if (ctl->error) return;
    const ll n = ctl->n;
    const double dt = ctl->dt, R = ctl->R;
    ll nan_local = 0;
    /* this cycle's slot of the render ring, if one is attached */
    nbg_renderable *ring = ring_rend ? ring_rend + (ll)(ctl->cycle % (ull)ring_slots) * ring_cap : nullptr;
    for (ll k = (ll)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (ll)gridDim.x * blockDim.x) {
        unsigned f = A.flags[k];
        nbg_renderable r;
        r.id = A.id[k];
        if (!(f & NBG_F_EXISTS)) {
            r.x = r.y = r.z = 0.0f;
            r.flags = 0;
            r.radius = 0.0;
            rend[k] = r;
            if (ring && k < ring_cap) ring[k] = r;
            continue;
        }
        double vx = A.vx[k], vy = A.vy[k], vz = A.vz[k];
        if (!(f & NBG_F_COLLIDED)) {
            const double m = A.m[k];
            vx += dt * A.fx[k] / m;
            vy += dt * A.fy[k] / m;
            vz += dt * A.fz[k] / m;
            A.vx[k] = vx;
            A.vy[k] = vy;
            A.vz[k] = vz;
        }
        const double x = A.x[k] + dt * vx;
        const double y = A.y[k] + dt * vy;
        const double z = A.z[k] + dt * vz;
        A.x[k] = x;
        A.y[k] = y;
        A.z[k] = z;
        A.rest[k] = R;
        f &= ~NBG_F_COLLIDED;
        if (x != x || y != y || z != z) {
            f &= ~NBG_F_EXISTS;
            nan_local++;
        }
        A.flags[k] = f;
        r.x = (float)x;
        r.y = (float)y;
        r.z = (float)z;
        r.flags = f & (NBG_F_EXISTS | NBG_F_IS_SUN);
        r.radius = A.rad[k];
        if (!(f & NBG_F_EXISTS)) {
            r.x = r.y = r.z = 0.0f;
            r.flags = 0;
            r.radius = 0.0;
        }
        rend[k] = r;
        if (ring && k < ring_cap) ring[k] = r;
    }
    if (ring) __threadfence_system(); /* the slot's renderables before its header */
    if (nan_local) atomicAdd((unsigned long long *)&ctl->acc_nan, (ull)nan_local);
}

/* the header of this cycle's ring slot, after its renderables: count and
 * written, a system-wide fence, then the cycle */
__global__ void k_ring_header(DevCtl *ctl, nbg_ring_slot *head, ll ring_cap, int ring_slots)
{
    if (ctl->error) return;
    const ull cycle = ctl->cycle;
    const ll n = ctl->n;
    volatile nbg_ring_slot *h = head + cycle % (ull)ring_slots;
    __threadfence_system();
    h->count = n;
    h->written = n < ring_cap ? n : ring_cap;
    __threadfence_system();
    h->cycle = (ll)cycle;
    __threadfence_system();
}

/* ------------------------------------------------------------------------ */
/* K7: Cycle (body_collection.go:253-296): stable compaction + adds         */
/* ------------------------------------------------------------------------ */

__device__ static void copy_body(const BodyArrays &S, ll s, BodyArrays &D, ll d)
{
    D.x[d] = S.x[s];
    D.y[d] = S.y[s];
    D.z[d] = S.z[s];
    D.vx[d] = S.vx[s];
    D.vy[d] = S.vy[s];
    D.vz[d] = S.vz[s];
    D.m[d] = S.m[s];
    D.rad[d] = S.rad[s];
    D.fx[d] = S.fx[s];
    D.fy[d] = S.fy[s];
    D.fz[d] = S.fz[s];
    D.ff[d] = S.ff[s];
    D.fs[d] = S.fs[s];
    D.rest[d] = S.rest[s];
    D.fr_rad[d] = S.fr_rad[s];
    D.fr_newrad[d] = S.fr_newrad[s];
    D.fr_mass[d] = S.fr_mass[s];
    D.fr_cx[d] = S.fr_cx[s];
    D.fr_cy[d] = S.fr_cy[s];
    D.fr_cz[d] = S.fr_cz[s];
    D.fr_cnt[d] = S.fr_cnt[s];
    D.id[d] = S.id[s];
    D.flags[d] = S.flags[s];
}

__device__ static bool cycle_changes(const DevCtl *ctl)
{
    return ctl->n_keep != ctl->n || ctl->frag_total > 0 || ctl->n_host_adds > 0;
}

/* Kept body k of sim s goes to new_off[s] + (its rank among kept bodies -
 * keep_start[s]): the order inside each sim is preserved. */
#define NBG_GONE 0xffffffffu

__global__ void __launch_bounds__(NBG_SCAN_BLOCK) k_compact(BodyArrays A, BodyArrays Bt, DevCtl *ctl, SimSegs seg,
                                                            const ll *blk_off, unsigned *remap)
{
    if (ctl->error || !cycle_changes(ctl)) return;
    const ll n = ctl->n;
    const ll base = (ll)blockIdx.x * NBG_SCAN_TILE;
    if (base >= n) return;
    /* rows of NBG_SCAN_BLOCK consecutive bodies, so every field access of a
     * warp is coalesced; kept bodies keep their order */
    ll rank = blk_off[blockIdx.x];
    for (int q = 0; q < NBG_SCAN_ITEMS; q++) {
        const ll k = base + (ll)q * NBG_SCAN_BLOCK + threadIdx.x;
        const bool keep = k < n && (A.flags[k] & NBG_F_EXISTS);
        ll tot;
        const ll ex = block_excl_scan(keep ? 1 : 0, &tot);
        if (keep) {
            const int sim = nbg_sim_of(seg.off, seg.nsims, k);
            const ll d = seg.new_off[sim] + (rank + ex - seg.keep_start[sim]);
            copy_body(A, k, Bt, d);
            if (remap) remap[k] = (unsigned)d;
        } else if (remap && k < n) {
            remap[k] = NBG_GONE;
        }
        rank += tot;
    }
}

/* The mixed path's Morton order carried through compaction: the kept bodies
 * keep their sorted sequence under their new indices, and each sim's arrivals
 * (fragments, host adds) follow its kept bodies.  A sim's sorted positions
 * cover the same range as its indices, so the stable compaction over
 * positions uses the per-sim offsets of the body compaction.  Three steps:
 * kept positions per block, their block offsets (k_scan_blocks mode 2), and
 * the scatter into the scratch order; k_order_copy then installs it. */
__global__ void __launch_bounds__(NBG_SCAN_BLOCK) k_order_blocksum(DevCtl *ctl, const unsigned *perm,
                                                                   const unsigned *remap, ll *blk_sum)
{
    if (ctl->error || !cycle_changes(ctl)) return;
    const ll n = ctl->n;
    const ll base = (ll)blockIdx.x * NBG_SCAN_TILE;
    if (base >= n) return;
    ll s = 0;
    for (int q = 0; q < NBG_SCAN_ITEMS; q++) {
        const ll p = base + (ll)q * NBG_SCAN_BLOCK + threadIdx.x;
        s += p < n && remap[perm[p]] != NBG_GONE ? 1 : 0;
    }
    ll tot;
    block_excl_scan(s, &tot);
    if (threadIdx.x == 0) blk_sum[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(NBG_SCAN_BLOCK) k_order_carry(DevCtl *ctl, SimSegs seg, const unsigned *perm,
                                                                const unsigned *remap, const ll *blk_off,
                                                                unsigned *order)
{
    if (ctl->error || !cycle_changes(ctl)) return;
    const ll n = ctl->n;
    const ll base = (ll)blockIdx.x * NBG_SCAN_TILE;
    if (base >= n) return;
    ll rank = blk_off[blockIdx.x];
    for (int q = 0; q < NBG_SCAN_ITEMS; q++) {
        const ll p = base + (ll)q * NBG_SCAN_BLOCK + threadIdx.x;
        const unsigned to = p < n ? remap[perm[p]] : NBG_GONE;
        const bool keep = to != NBG_GONE;
        ll tot;
        const ll ex = block_excl_scan(keep ? 1 : 0, &tot);
        if (keep) {
            const int sim = nbg_sim_of(seg.off, seg.nsims, p);
            order[seg.new_off[sim] + (rank + ex - seg.keep_start[sim])] = to;
        }
        rank += tot;
    }
}

__global__ void k_order_copy(DevCtl *ctl, SimSegs seg, const unsigned *order, unsigned *perm)
{
    if (ctl->error || !cycle_changes(ctl)) return;
    const ll total = seg.new_off[seg.nsims];
    for (ll k = (ll)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (ll)gridDim.x * blockDim.x) {
        const int sim = nbg_sim_of(seg.new_off, seg.nsims, k);
        perm[k] = k - seg.new_off[sim] < seg.keep[sim] ? order[k] : (unsigned)k; /* arrivals: as they come */
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->order_carried = 1;
}

/* Appends each sim's adds after its kept bodies, newest first (the sim's
 * fragments of this cycle, then its host adds), each with r = R. */
__global__ void k_append_adds(BodyArrays Bt, BodyArrays F, BodyArrays H, DevCtl *ctl, SimSegs seg)
{
    if (ctl->error || !cycle_changes(ctl)) return;
    const ll nf = ctl->frag_total, nh = ctl->n_host_adds;
    const double R = ctl->R;
    const int ns = seg.nsims;
    for (ll k = (ll)blockIdx.x * blockDim.x + threadIdx.x; k < nf + nh; k += (ll)gridDim.x * blockDim.x) {
        ll d;
        if (k < nf) {
            const int s = nbg_sim_of(seg.frag_start, ns, k);
            d = seg.new_off[s] + seg.keep[s] + (seg.frag_start[s + 1] - 1 - k);
            copy_body(F, k, Bt, d);
        } else {
            const ll h = k - nf;
            const int s = nbg_sim_of(seg.hadd_start, ns, h);
            d = seg.new_off[s] + seg.keep[s] + seg.frag[s] + (seg.hadd_start[s + 1] - 1 - h);
            copy_body(H, h, Bt, d);
        }
        Bt.rest[d] = R;
    }
}

__global__ void k_copy_back(BodyArrays A, BodyArrays Bt, DevCtl *ctl, SimSegs seg)
{
    if (ctl->error || !cycle_changes(ctl)) return;
    const ll total = seg.new_off[seg.nsims];
    for (ll k = (ll)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (ll)gridDim.x * blockDim.x)
        copy_body(Bt, k, A, k);
}

__global__ void __launch_bounds__(NBG_SCAN_BLOCK) k_end(DevCtl *ctl, SimSegs seg)
{
    if (ctl->error) return;
    const int ns = seg.nsims;
    const bool changed = cycle_changes(ctl);
    for (int s = threadIdx.x; s <= ns; s += NBG_SCAN_BLOCK) {
        if (changed) seg.off[s] = seg.new_off[s];
        if (s < ns) seg.hadd[s] = 0;
    }
    if (threadIdx.x != 0) return;
    const ll n = ctl->n;
    ctl->rend_n = n;
    ctl->acc_removed += n - ctl->n_keep;
    ctl->acc_interactions += ctl->cycle_interactions;
    ctl->n = ctl->n_keep + ctl->frag_total + ctl->n_host_adds;
    ctl->n_host_adds = 0;
    /* bodies changed index: the order is stale unless it was carried along */
    if (changed && !ctl->order_carried) ctl->sort_valid = 0;
    ctl->order_carried = 0;
    ctl->cycle += 1;
    ctl->acc_steps += 1;
}

/* ------------------------------------------------------------------------ */
/* cycle-boundary edits                                                     */
/* ------------------------------------------------------------------------ */

/* Bodies [lo, hi) of collection sim (sim < 0: the whole array). */
__device__ __forceinline__ void sim_range(const DevCtl *ctl, const SimSegs &seg, int sim, ll &lo, ll &hi)
{
    lo = sim >= 0 ? seg.off[sim] : 0;
    hi = sim >= 0 ? seg.off[sim + 1] : ctl->n;
}

/* processDeletes, computation-runner.go:176-216 (sequential by nature), over
 * collection sim (sim < 0: the whole array, one collection). */
__global__ void k_remove(BodyArrays A, DevCtl *ctl, SimSegs seg, int sim, ll count, ll *removed)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    ll lo, hi;
    sim_range(ctl, seg, sim, lo, hi);
    const ll n = hi - lo;
    ll rem = 0;
    if (count == -1) {
        for (ll k = lo; k < hi; k++) {
            if (A.flags[k] & NBG_F_EXISTS) {
                A.m[k] = 0;
                A.flags[k] &= ~NBG_F_EXISTS;
                rem++;
            }
        }
    } else if (n > 0) {
        const ll step = count > n ? 1 : n / count;
        ll iter = 0;
        bool should = false;
        for (ll k = lo; k < hi; k++) {
            if (iter % step == 0) should = true;
            iter++;
            unsigned f = A.flags[k];
            if (should && !(f & NBG_F_PINNED) && (f & NBG_F_EXISTS)) {
                A.m[k] = 0;
                A.flags[k] = f & ~NBG_F_EXISTS;
                should = false;
                rem++;
            }
        }
    }
    *removed = rem;
}

/* ApplyMods for bodies matched by id (body.go:274-313, after parsing), in
 * collection sim (sim < 0: every collection). */
__global__ void k_edits(BodyArrays A, DevCtl *ctl, SimSegs seg, int sim, const nbg_edit *E, ll ne, int *results)
{
    ll lo, hi;
    sim_range(ctl, seg, sim, lo, hi);
    for (ll k = lo + (ll)blockIdx.x * blockDim.x + threadIdx.x; k < hi; k += (ll)gridDim.x * blockDim.x) {
        const ll id = A.id[k];
        for (ll q = 0; q < ne; q++) {
            const nbg_edit e = E[q];
            if (e.id != id) continue;
            atomicAdd(&results[q], 1);
            const unsigned m = e.mask;
            if (m & NBG_M_X) A.x[k] = e.x;
            if (m & NBG_M_Y) A.y[k] = e.y;
            if (m & NBG_M_Z) A.z[k] = e.z;
            if (m & NBG_M_VX) A.vx[k] = e.vx;
            if (m & NBG_M_VY) A.vy[k] = e.vy;
            if (m & NBG_M_VZ) A.vz[k] = e.vz;
            if (m & NBG_M_MASS) A.m[k] = e.mass;
            if (m & NBG_M_RADIUS) A.rad[k] = e.radius;
            if (m & NBG_M_FRAG_FACTOR) A.ff[k] = e.frag_factor;
            if (m & NBG_M_FRAG_STEP) A.fs[k] = e.frag_step;
            unsigned f = A.flags[k];
            if (m & NBG_M_COLLISION)
                f = (f & ~(3u << NBG_BEHAVIOR_SHIFT)) | (((unsigned)e.collision & 3u) << NBG_BEHAVIOR_SHIFT);
            if (m & NBG_M_TELEMETRY) f = e.telemetry ? (f | NBG_F_TELEMETRY) : (f & ~NBG_F_TELEMETRY);
            if (m & NBG_M_EXISTS) f = e.exists ? (f | NBG_F_EXISTS) : (f & ~NBG_F_EXISTS);
            A.flags[k] = f;
        }
    }
}

/* The first body with this id in collection sim (sim < 0: anywhere). */
__global__ void k_find(BodyArrays A, DevCtl *ctl, SimSegs seg, int sim, ll id, ll *idx)
{
    ll lo, hi;
    sim_range(ctl, seg, sim, lo, hi);
    for (ll k = lo + (ll)blockIdx.x * blockDim.x + threadIdx.x; k < hi; k += (ll)gridDim.x * blockDim.x)
        if (A.id[k] == id) atomicMin((long long *)idx, (long long)k);
}

/* dst[k] = src[index[k]] for k < n: every field of a body record. */
__global__ void k_gather_bodies(BodyArrays S, BodyArrays D, const ll *index, ll n)
{
    for (ll k = (ll)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (ll)gridDim.x * blockDim.x)
        copy_body(S, index[k], D, k);
}

/* Kinetic and pairwise potential energy plus momentum, per-block partials
 * (out[blockIdx*5 + 0..4]) summed on the host in block order. */
#define EN_BLOCK 128
__global__ void __launch_bounds__(EN_BLOCK) k_energy(BodyArrays A, DevCtl *ctl, SimSegs seg, double *out)
{
    __shared__ double red[5][EN_BLOCK];
    const ll n = ctl->n;
    double ke = 0, pe = 0, px = 0, py = 0, pz = 0;
    const ll i = (ll)blockIdx.x * EN_BLOCK + threadIdx.x;
    if (i < n && (A.flags[i] & NBG_F_EXISTS)) {
        const double m = A.m[i], vx = A.vx[i], vy = A.vy[i], vz = A.vz[i];
        ke = 0.5 * m * (vx * vx + vy * vy + vz * vz);
        px = m * vx;
        py = m * vy;
        pz = m * vz;
        const double xi = A.x[i], yi = A.y[i], zi = A.z[i];
        const ll end = seg.off[nbg_sim_of(seg.off, seg.nsims, i) + 1]; /* pairs within i's sim */
        for (ll j = i + 1; j < end; j++) {
            if (!(A.flags[j] & NBG_F_EXISTS)) continue;
            const double dx = A.x[j] - xi, dy = A.y[j] - yi, dz = A.z[j] - zi;
            const double r = sqrt(dx * dx + dy * dy + dz * dz);
            if (r > 0) pe -= NBG_G * m * A.m[j] / r;
        }
    }
    red[0][threadIdx.x] = ke;
    red[1][threadIdx.x] = pe;
    red[2][threadIdx.x] = px;
    red[3][threadIdx.x] = py;
    red[4][threadIdx.x] = pz;
    __syncthreads();
    for (int s = EN_BLOCK / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int q = 0; q < 5; q++) red[q][threadIdx.x] += red[q][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int q = 0; q < 5; q++) out[(ll)blockIdx.x * 5 + q] = red[q][0];
}

/* ------------------------------------------------------------------------ */
/* launchers                                                                */
/* ------------------------------------------------------------------------ */

static int scan_grid(ll cap) { return (int)((cap + NBG_SCAN_TILE - 1) / NBG_SCAN_TILE); }


void nbg_launch_begin(const CycleBufs &cb, DevCtl *ctl, cudaStream_t st)
{
    k_begin<<<1, NBG_SCAN_BLOCK, 0, st>>>(ctl, cb.seg, cb.slots, cb.work_cap, cb.itile > 0 ? cb.itile : NBG_MIX_ITILE,
                                          cb.part_doubles, nbg_mix_is_sym(cb.mix_variant), cb.jpart_units);
}

void nbg_launch_frag_count(const CycleBufs &cb, DevCtl *ctl, cudaStream_t st)
{
    int g = scan_grid(cb.cap);
    k_frag_blocksum<<<g, NBG_SCAN_BLOCK, 0, st>>>(cb.a, ctl, cb.seg, cb.blk_sum);
    k_scan_blocks<<<1, NBG_SCAN_BLOCK, 0, st>>>(ctl, cb.seg, cb.blk_sum, cb.blk_off, 0, cb.cap, cb.frag_cap);
}

int nbg_pair_fp64_grid(ll cap)
{
    ll g = (cap + P64_BLOCK - 1) / P64_BLOCK;
    return (int)(g < 1 ? 1 : (g > 65535 ? 65535 : g));
}

void nbg_launch_pair_fp64(const CycleBufs &cb, DevCtl *ctl, cudaStream_t st)
{
    if (cb.p64_terms && cb.seg.nsims == 1) {
        const ll jc = cb.p64_jc;
        /* a grid-stride loop over the live bodies' work items: at most 32
         * blocks of two warps per SM, fewer when the capacity is small */
        const int js = cb.cap <= 8192 ? 4 : 16;
        const ll want = ((cb.cap + P64_BLOCK - 1) / P64_BLOCK) * ((jc + js - 1) / js);
        const ll most = (ll)(cb.sms > 0 ? cb.sms : 1) * 32;
        const unsigned g = (unsigned)(want < most ? want : most);
        for (ll jbase = 0; jbase < cb.cap; jbase += jc) {
            if (js == 4)
                k_p64_terms<4><<<g, P64_BLOCK, 0, st>>>(cb.a, ctl, cb.p64_terms, cb.cap, jc, jbase, cb.ev_keys,
                                                         cb.ev_cap);
            else
                k_p64_terms<16><<<g, P64_BLOCK, 0, st>>>(cb.a, ctl, cb.p64_terms, cb.cap, jc, jbase, cb.ev_keys,
                                                          cb.ev_cap);
            /* 32 bodies per block, at most 8 blocks per SM */
            const ll sb = (cb.cap + SUM_BODIES - 1) / SUM_BODIES, smost = (ll)(cb.sms > 0 ? cb.sms : 1) * 8;
            k_p64_sum<<<(unsigned)(sb < smost ? sb : smost), SUM_THREADS, 0, st>>>(cb.a, ctl, cb.p64_terms,
                                                                                  cb.p64_acc, cb.cap, jc, jbase);
        }
        return;
    }
    k_pair_fp64<<<nbg_pair_fp64_grid(cb.cap), P64_BLOCK, 0, st>>>(cb.a, ctl, cb.seg, cb.ev_keys, cb.ev_cap);
}

int nbg_pair_fp64_launches(const CycleBufs &cb)
{
    return cb.p64_terms && cb.seg.nsims == 1 ? (int)(2 * ((cb.cap + cb.p64_jc - 1) / cb.p64_jc)) : 1;
}

/* everything after the pair kernel: order events, emit fragments, resolve,
 * integrate, Cycle */
void nbg_launch_after_pair(const CycleBufs &cb, DevCtl *ctl, cudaStream_t st, bool carry_order)
{
    const int sg = scan_grid(cb.cap);
    k_sort_events<<<1, SORT_BLOCK, 0, st>>>(ctl, cb.ev_keys, cb.ev_cap, cb.ev_radix);
    int links = 0;
    if (cb.ev_radix) {
        nbg_launch_event_radix(cb, ctl, st);
        /* the links, when a body index and an event index fit one key */
        int kb = 1, ob = 1;
        while (kb < 31 && ((ll)1 << kb) < cb.cap) kb++;
        while (ob < 40 && ((ll)1 << ob) < cb.ev_cap) ob++;
        if (kb + ob + 1 <= 64) {
            links = 1;
            const int eg = nbg_flat_grid(cb, 2 * cb.ev_cap);
            k_ev_ranges<<<(cb.seg.nsims + 256) / 256, 256, 0, st>>>(ctl, cb.seg, cb.ev_keys, cb.ev_lo);
            k_ev_incid<<<eg, 256, 0, st>>>(ctl, cb.seg, cb.ev_keys, cb.ev_lo, cb.inc[0], ob);
            const ull *sorted = nbg_launch_incidence_radix(cb, ctl, kb + ob, st);
            k_ev_links<<<eg, 256, 0, st>>>(ctl, sorted, ob, cb.ev_link, cb.ev_front);
            k_ev_pending<<<eg, 256, 0, st>>>(ctl, cb.ev_front, cb.ev_pend);
        }
    }
    k_frag_emit<<<sg, NBG_SCAN_BLOCK, 0, st>>>(cb.a, cb.frags, ctl, cb.blk_off);
    /* the radix-sort key buffer is free after the pair pass: per-body owner words */
    k_resolve<<<cb.seg.nsims, RESOLVE_BLOCK, 0, st>>>(cb.a, ctl, cb.seg, cb.ev_keys, cb.ev_out, cb.skey[1], links,
                                                      cb.ev_lo, cb.ev_link, cb.ev_pend, cb.ev_front, cb.ev_cap);
    k_integrate<<<nbg_flat_grid(cb, cb.cap), 256, 0, st>>>(cb.a, ctl, cb.rend, cb.ring_rend, cb.ring_cap, cb.ring_slots);
    if (cb.ring_head) k_ring_header<<<1, 1, 0, st>>>(ctl, cb.ring_head, cb.ring_cap, cb.ring_slots);
    k_keep_blocksum<<<sg, NBG_SCAN_BLOCK, 0, st>>>(cb.a, ctl, cb.seg, cb.blk_sum);
    k_scan_blocks<<<1, NBG_SCAN_BLOCK, 0, st>>>(ctl, cb.seg, cb.blk_sum, cb.blk_off, 1, cb.cap, cb.frag_cap);
    /* the radix value buffer is free after the sort: old -> new index */
    unsigned *remap = carry_order ? cb.sval : nullptr;
    k_compact<<<sg, NBG_SCAN_BLOCK, 0, st>>>(cb.a, cb.b, ctl, cb.seg, cb.blk_off, remap);
    k_append_adds<<<nbg_flat_grid(cb, cb.frag_cap + cb.adds_cap), 256, 0, st>>>(cb.b, cb.frags, cb.adds, ctl, cb.seg);
    k_copy_back<<<nbg_flat_grid(cb, cb.cap), 256, 0, st>>>(cb.a, cb.b, ctl, cb.seg);
    if (carry_order) {
        /* the sorted-key buffer is free after the sort: the scratch order */
        k_order_blocksum<<<sg, NBG_SCAN_BLOCK, 0, st>>>(ctl, cb.perm, remap, cb.blk_sum);
        k_scan_blocks<<<1, NBG_SCAN_BLOCK, 0, st>>>(ctl, cb.seg, cb.blk_sum, cb.blk_off, 2, cb.cap, cb.frag_cap);
        k_order_carry<<<sg, NBG_SCAN_BLOCK, 0, st>>>(ctl, cb.seg, cb.perm, remap, cb.blk_off, cb.skey[0]);
        k_order_copy<<<nbg_flat_grid(cb, cb.cap), 256, 0, st>>>(ctl, cb.seg, cb.skey[0], cb.perm);
    }
    k_end<<<1, NBG_SCAN_BLOCK, 0, st>>>(ctl, cb.seg);
}

void nbg_launch_remove(const CycleBufs &cb, DevCtl *ctl, int sim, ll count, ll *removed_dev, cudaStream_t st)
{
    k_remove<<<1, 32, 0, st>>>(cb.a, ctl, cb.seg, sim, count, removed_dev);
}

void nbg_launch_edits(const CycleBufs &cb, DevCtl *ctl, int sim, const nbg_edit *edits_dev, ll k, int *results_dev,
                      cudaStream_t st)
{
    k_edits<<<nbg_flat_grid(cb, cb.cap), 256, 0, st>>>(cb.a, ctl, cb.seg, sim, edits_dev, k, results_dev);
}

void nbg_launch_find(const CycleBufs &cb, DevCtl *ctl, int sim, ll id, ll *idx_dev, cudaStream_t st)
{
    k_find<<<nbg_flat_grid(cb, cb.cap), 256, 0, st>>>(cb.a, ctl, cb.seg, sim, id, idx_dev);
}

void nbg_launch_gather(const CycleBufs &cb, const BodyArrays &src, const BodyArrays &dst, const ll *index_dev, ll n,
                       cudaStream_t st)
{
    if (n > 0) k_gather_bodies<<<nbg_flat_grid(cb, n), 256, 0, st>>>(src, dst, index_dev, n);
}

void nbg_launch_energy(const CycleBufs &cb, DevCtl *ctl, double *out_dev, cudaStream_t st)
{
    int g = (int)((cb.cap + EN_BLOCK - 1) / EN_BLOCK);
    k_energy<<<g, EN_BLOCK, 0, st>>>(cb.a, ctl, cb.seg, out_dev);
}
