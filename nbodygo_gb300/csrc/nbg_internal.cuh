/*
 * nbg_internal.cuh - device-side layout of a context and the kernel entry
 * points shared between the translation units of libnbgpu.so.
 *
 * HBM layout (one context, capacity C bodies):
 *   BodyArrays: 20 FP64 arrays, 2 int64 arrays and 1 u32 flag array of C
 *   elements each (structure of arrays, 180 B per body).  A second BodyArrays
 *   set of the same size receives the compacted collection in Cycle and is
 *   copied back.  Flags hold NBG_F_* in bits 0..7 and the collision
 *   behaviour in bits 8..9.
 *   Mixed form only: jhi/jlo float4 per body (x_hi, y_hi, z_hi, m/m_scale)
 *   and (x_lo, y_lo, z_lo, radius) = 32 B per body, rebuilt every cycle; one
 *   float4 origin per 512-body i-tile; S x 3 x C FP64 partial sums.
 *   Events: one u64 key per detected (i, j) pair: i << 32 | j << 2 | type.
 */
#ifndef NBG_INTERNAL_CUH
#define NBG_INTERNAL_CUH

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/nbgpu.h"

typedef long long ll;
typedef unsigned long long ull;

#define NBG_BEHAVIOR_SHIFT 8
#define NBG_BEHAVIOR(flags) (((flags) >> NBG_BEHAVIOR_SHIFT) & 3u)
#define NBG_LIVE_MASK (NBG_F_EXISTS | NBG_F_FRAGMENTING)

/* event key type field */
#define NBG_EVT_COLL_IJ 0u /* collision(i, j)      */
#define NBG_EVT_SUB_IJ 1u  /* subsume(i absorbs j) */
#define NBG_EVT_SUB_JI 2u  /* subsume(j absorbs i) */

#define NBG_MAX_BODIES ((ll)1 << 30) /* event keys pack i and j in 30 bits */
#define NBG_MAX_SIMS 2048            /* Morton keys of several sims carry the sim in 11 bits */

#define NBG_NF64 20
struct BodyArrays {
    /* the FP64 fields, in this order, are f64[0..19] */
    double *x, *y, *z, *vx, *vy, *vz, *m, *rad, *fx, *fy, *fz, *ff, *fs, *rest;
    double *fr_rad, *fr_newrad, *fr_mass, *fr_cx, *fr_cy, *fr_cz;
    ll *fr_cnt, *id;
    unsigned *flags;
};

/* Control block in device memory; kernels of a cycle read and update it, so
 * a captured graph of one cycle can be replayed. */
struct DevCtl {
    ll n;            /* bodies in the array */
    ll next_id;      /* NextId counter */
    ull cycle;       /* cycle index (fragment generator key) */
    ull seed;
    double dt, R;
    int error;       /* sticky NBG_E_* raised by a kernel */
    int pad0;
    ll error_need;   /* for NBG_E_OVERFLOW: the size that would have fitted */
    int error_what;  /* 1 = bodies, 2 = events, 3 = fragments, 4 = partials, 5 = octree nodes,
                      * 6 = symmetric kernel j-partial units, 7 = inconsistent event links,
                      * 8 = a bulk copy into shared memory that did not complete */
    int splits;      /* mixed: chunks the pair work is cut into (C) */
    ll work_total;   /* mixed: pair work W in (i-tile, j-body) units */
    /* per-cycle values */
    ll ev_count;     /* detected events (may exceed capacity) */
    ll frag_total;   /* fragments emitted this cycle */
    ll n_keep;       /* bodies that survive Cycle */
    ll n_host_adds;  /* adds staged by the host for this cycle */
    ll n_before;     /* bodies at the start of the cycle */
    /* mixed-form reductions (float bits as unsigned for atomicMax) */
    unsigned rmax_bits, xmax_bits;
    double m_scale;
    /* mixed form: pairs closer than near_kappa * (extent of the i-tile around
     * its origin) are evaluated in FP64 (set by the host) */
    float near_kappa;
    /* test hook (NBG_OPT_TEST_WAIT_STALL): bytes the bulk-copy shapes add to
     * each mbarrier's expected count, so that no phase completes; 0 */
    unsigned test_tx_extra;
    /* accumulated over the cycles of one nbg_step call */
    ll acc_steps, acc_interactions, acc_events, acc_frags, acc_removed, acc_nan, acc_bh_terms;
    ll rend_n;       /* renderables written by the last cycle */
    ll last_ev_n;    /* resolved events recorded by the last cycle */
    ll cycle_interactions; /* sum over sims of n_s (n_s - 1) at the cycle start */
    ll acc_ev_max;   /* most events one cycle of this nbg_step call detected */
    ll work_next;    /* mixed: next chunk for the persistent CTAs */
    /* Barnes-Hut (k_bh.cu): bounds of the tree bodies as order-preserving
     * integer images of doubles, the tree body count, nodes built, and the
     * largest radius of any body (for the collision query) */
    ull bh_lo[3], bh_hi[3];
    ll bh_count;
    ll bh_nodes;
    ull bh_rmax;
    unsigned bh_next; /* the walk's next 32-body group (one per warp) */
    unsigned pad2;
    /* Morton order of the mixed path (perm): valid while no body changed
     * index; re-sorted when invalid or sort_interval cycles after the last
     * sort (0: NBG_SORT_INTERVAL_DEFAULT).  sort_now is this cycle's decision. */
    int sort_valid;
    int sort_now;
    int sort_interval;
    int order_carried; /* this cycle's compaction carried the order along */
    ull sort_cycle;
};

#define NBG_SORT_INTERVAL_DEFAULT 4

/* events sorted by one block in shared memory; more take the multi-block
 * radix sort (when the cycle's launches include it) */
#define NBG_EV_BLOCK_SORT 4096

/* mixed: pairs closer than this factor x the i-body's distance from its
 * tile origin take the near-pair pass (NBG_OPT_NEAR_PPM changes it) */
#define NBG_NEAR_KAPPA_DEFAULT 0.05f
/* collections of at most this many bodies use twice the near-pair factor */
#define NBG_NEAR_SMALL_N 2048

/* A collection may hold several independent simulations stored one after
 * another: sim s occupies bodies [off[s], off[s+1]) and bodies of different
 * sims never interact.  Events, fragments and adds stay inside their sim, so
 * each sim follows the reference's cycle exactly as if it were alone. */
struct SimSegs {
    int nsims;
    ll *off;         /* [nsims+1] */
    ll *tile_off;    /* [nsims+1] plain kernel: 64-body i-tiles before sim s */
    ll *mtile_off;   /* [nsims+1] mixed kernel: 512-body i-tiles before sim s */
    ll *item_off;    /* [nsims+1] mixed kernel: pair work before sim s, in (i-tile, j-body)
                      * units: sim s holds (its i-tiles) x n_s of them */
    ll *keep;        /* [nsims]   bodies of sim s that survive Cycle */
    ll *frag;        /* [nsims]   fragments sim s emits this cycle */
    ll *frag_start;  /* [nsims+1] */
    ll *hadd;        /* [nsims]   host adds staged for sim s */
    ll *hadd_start;  /* [nsims+1] */
    ll *keep_start;  /* [nsims+1] */
    ll *new_off;     /* [nsims+1] layout after Cycle */
    unsigned *xmax_bits; /* [nsims] mixed: |x| max of sim s (Morton grid) */
};

/* bytes of the SimSegs arrays for nsims sims (one allocation, carved by
 * nbg_seg_carve: 11 ll arrays and 2 32-bit arrays of nsims + 1) */
#define NBG_SEG_BYTES(ns) ((size_t)((ns) + 1) * 8 * 11 + (size_t)((ns) + 1) * 4 * 2 + 256)

static inline SimSegs nbg_seg_carve(void *base, int nsims)
{
    SimSegs s;
    const size_t m = (size_t)nsims + 1;
    ll *p = (ll *)base;
    s.nsims = nsims;
    s.off = p;
    s.tile_off = p + m;
    s.mtile_off = p + 2 * m;
    s.item_off = p + 3 * m;
    s.keep = p + 4 * m;
    s.frag = p + 5 * m;
    s.frag_start = p + 6 * m;
    s.hadd = p + 7 * m;
    s.hadd_start = p + 8 * m;
    s.keep_start = p + 9 * m;
    s.new_off = p + 10 * m;
    s.xmax_bits = (unsigned *)(p + 11 * m) + m; /* the first 32-bit array is spare */
    return s;
}

/* sim holding position k of a segmented array: the largest s with
 * off[s] <= k (empty sims are skipped) */
__device__ __forceinline__ int nbg_sim_of(const ll *off, int nsims, ll k)
{
    int lo = 0, hi = nsims - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= k)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

/* Barnes-Hut octree of one collection, nodes in depth-first order */
struct BhTree {
    ull *key[2];        /* octant-path keys (radix ping-pong) */
    unsigned *val[2];   /* body index (ping-pong partner) */
    ll *hist;           /* radix digit histogram */
    ll *base;           /* nodes starting at each sorted position, then their scan */
    ll *blk;            /* per-block sums of that scan */
    double *mass, *mx, *my, *mz, *cmx, *cmy, *cmz, *cx, *cy, *cz, *half;
    float4 *fa, *fb;    /* mixed walk: (cm hi xyz, mass / root mass), (cm lo xyz, opening r^2) */
    int4 *fc;           /* mixed walk: (skip, start, end, flags) */
    float4 *fd;         /* collision query: the node's cube (centre xyz, half) in FP32 */
    int *skip, *start, *end, *first;
    unsigned char *level, *flags;
    /* one tree per collection, all in one depth-first node array: per
     * collection s its bounding box (sbox[6 s ..]: lo xyz, hi xyz as
     * order-preserving integers), tree bodies (scount), first sorted
     * position (stree, [nsims + 1]), root node (sroot, [nsims + 1]: the nodes
     * of s are [sroot[s], sroot[s + 1])) and first 32-body walk group (sgrp,
     * [nsims + 1]) */
    ull *sbox;
    ll *scount, *stree, *sroot, *sgrp;
    ll node_cap;
};

struct CycleBufs {
    SimSegs seg;
    BodyArrays a;       /* the collection */
    BodyArrays b;       /* compaction target */
    BodyArrays adds;    /* host adds staged for the next Cycle (arrival order) */
    BodyArrays frags;   /* fragments emitted this cycle (arrival order) */
    ll cap, frag_cap, adds_cap;
    ull *ev_keys;
    ull *ev_sort;       /* ping-pong partner of ev_keys for the multi-block event sort */
    ll *ev_hist;        /* its digit histogram and chunk sums (nbg_sort_scratch_hist(ev_cap)) */
    ll ev_cap;
    int ev_radix;       /* this cycle's launches include the multi-block event sort and the
                         * resolution's links (dataflow order) */
    /* resolution links, for cycles beyond the one-block sort: incidence keys
     * (ping-pong, 2 ev_cap each) and their histogram; per event (processing
     * index) the next event on each of its bodies, the count of unresolved
     * predecessors, and the frontier lists (2 ev_cap); each sim's event range */
    ull *inc[2];
    ll *inc_hist;
    ll *ev_link;
    int *ev_pend;
    ll *ev_front;
    ll *ev_lo;
    nbg_event *ev_out;  /* resolved events of the last cycle */
    nbg_renderable *rend;
    ll *blk_sum;        /* per-block counts for the scans */
    ll *blk_off;
    ll nblk_cap;
    /* mixed form (indexed by sorted position) */
    float4 *jhi, *jlo;
    float4 *tile_c;     /* per i-tile: origin (xyz) and a radius holding its bodies (w) */
    float *tile_t;      /* per i-tile: the largest near-pair threshold of its bodies (NULL: not kept) */
    float4 *iprep;      /* per sorted position: re-centred x, y, z and near-pair threshold */
    double *part;
    unsigned *perm;     /* sorted position -> body index */
    unsigned *skey[2];  /* radix-sort keys (ping-pong) */
    unsigned *sval;     /* radix-sort values (ping-pong partner of perm) */
    ll *shist;          /* radix-sort digit histogram / offsets */
    ll part_doubles;    /* size of part */
    int work_cap;       /* most CTAs the mixed pair work is divided among (0 = slots) */
    int slots;          /* resident CTAs of the mixed kernel on this device */
    int mix_variant;    /* shape of the mixed pair kernel (see nbg_mix_variant_info) */
    float *jpart;       /* symmetric kernel: FP32 j sums per unit, 3 x itile each */
    ll jpart_units;     /* units jpart holds */
    int itile;          /* i-bodies per work item of that shape */
    /* render ring in mapped host memory (device addresses; NULL: none) */
    nbg_ring_slot *ring_head;
    nbg_renderable *ring_rend;
    ll ring_cap;
    int ring_slots;
    /* plain form, small collections: pair terms (3 x p64_jc x cap) and the
     * sums carried between passes (3 x cap); NULL when cap is too large */
    double *p64_terms, *p64_acc;
    ll p64_jc;
    int bh;             /* forces from the Barnes-Hut octree */
    int bh_shape;       /* register cap of the mixed walk: 0, 1, 2 = 3, 4, 5 CTAs per SM */
    int sms;            /* streaming multiprocessors of the device */
    BhTree t;
};

/* Grid of a grid-stride kernel over `items` items, 256 threads per CTA:
 * one CTA per 256 items, at most `per_sm` CTAs per streaming multiprocessor
 * of the device the buffers live on. */
static inline int nbg_flat_grid(const CycleBufs &cb, ll items, int per_sm = 16)
{
    const ll most = (ll)(cb.sms > 0 ? cb.sms : 1) * per_sm;
    ll g = (items + 255) / 256;
    if (g > most) g = most;
    return (int)(g < 1 ? 1 : g);
}

/* Shapes of the mixed pair kernel the autotuner chooses from. */
struct MixVariantInfo {
    int block, k, jt, unroll;
};
#define NBG_MIX_VARIANTS NBG_MIX_SHAPES
/* the symmetric kernel (each unordered pair once, k_pair_sym): shapes 15
 * and 16 (registers capped for 4 and 5 CTAs per SM) */
#define NBG_MIX_SYM 15
__host__ __device__ __forceinline__ bool nbg_mix_is_sym(int variant)
{
    return variant == NBG_MIX_SYM || variant == NBG_MIX_SYM + 1;
}
#define NBG_MIX_MIN_ITILE 256
#define NBG_MIX_MAX_ITILE 512
/* fewest (i-tile, j-body) units of pair work in a chunk, and chunks per
 * resident CTA */
#define NBG_MIX_MIN_WORK 2048
#define NBG_MIX_CHUNKS_PER_CTA 32

/* floor(a b / c) for 0 <= a, 0 < c, without forming a b */
__host__ __device__ __forceinline__ ll nbg_mul_div(ll a, ll b, ll c)
{
    return a * (b / c) + a * (b % c) / c;
}

/* The mixed pair work of a cycle is W units, (i-tile, j-body) pairs in sim,
 * i-tile, j order, cut into C chunks that persistent CTAs take from an
 * atomic counter.  The cut is guided: the first C/4 chunks split the first
 * three quarters of the work evenly and the other chunks the last quarter,
 * so the chunks still running when the counter runs out are a ninth of the
 * first ones and the CTAs finish close together.  The boundaries depend on
 * C and W alone, never on timing.  With C >= 4 and W >= 2048 C every chunk
 * holds work.  This is the first unit of chunk c (c = C gives W). */
__host__ __device__ __forceinline__ ll nbg_chunk_start(ll c, int C, ll W)
{
    const int C1 = C / 4;
    const ll W1 = C1 > 0 ? W - W / 4 : 0;
    if (c <= C1) return C1 > 0 ? nbg_mul_div(c, W1, C1) : 0;
    return W1 + nbg_mul_div(c - C1, W - W1, C - C1);
}

/* the chunk that holds unit u (0 <= u < W) */
__host__ __device__ __forceinline__ int nbg_work_chunk(ll u, int C, ll W)
{
    const int C1 = C / 4;
    const ll W1 = C1 > 0 ? W - W / 4 : 0;
    ll c0, c1;
    if (u < W1) {
        c0 = (ll)((double)u * C1 / (double)W1);
        c0 = c0 < 0 ? 0 : (c0 > C1 - 1 ? C1 - 1 : c0);
        c1 = C1 - 1;
    } else {
        c0 = C1 + (ll)((double)(u - W1) * (C - C1) / (double)(W - W1));
        c0 = c0 < C1 ? C1 : (c0 > C - 1 ? C - 1 : c0);
        c1 = C - 1;
    }
    /* the estimate is off by at most one either way */
    while (c0 > 0 && nbg_chunk_start(c0, C, W) > u) c0--;
    while (c0 < c1 && nbg_chunk_start(c0 + 1, C, W) <= u) c0++;
    return (int)c0;
}

/* Partial sums of the mixed pair kernel: chunk c's share of i-tile g (global
 * tile index) is slot g + c, 3 x itile doubles; no two (tile, chunk) pairs
 * that both hold work share a slot, since chunks are contiguous and ordered.
 * Slots needed: tiles + C - 1, tiles <= cap / itile + sims. */
#define NBG_PART_DOUBLES(cap, chunks, itile) \
    (3 * ((ll)(cap) + (ll)(itile) * ((ll)(chunks) + NBG_MAX_SIMS + 2)))

#define NBG_SCAN_BLOCK 1024
#define NBG_SCAN_ITEMS 4
#define NBG_SCAN_TILE (NBG_SCAN_BLOCK * NBG_SCAN_ITEMS)

#define NBG_MIX_BLOCK 128
#define NBG_MIX_K 4
#define NBG_MIX_ITILE (NBG_MIX_BLOCK * NBG_MIX_K)
#define NBG_MIX_JT 256

/* The reference's event rules (body.go:174-184): the event type for bodies
 * i, j with behaviours bi, bj, radii ri, rj at distance dist, or -1. */
__device__ static inline int nbg_detect_event(unsigned bi, unsigned bj, double ri, double rj, double dist)
{
    const bool ei = (bi == NBG_ELASTIC || bi == NBG_FRAGMENT);
    const bool ej = (bj == NBG_ELASTIC || bj == NBG_FRAGMENT);
    if (ei && ej) return (int)NBG_EVT_COLL_IJ;
    if (bi == NBG_SUBSUME || bj == NBG_SUBSUME) {
        if (ri > rj && dist <= ri) return (int)NBG_EVT_SUB_IJ;
        if (rj > ri && dist <= rj) return (int)NBG_EVT_SUB_JI;
    }
    return -1;
}

/* appends event (i, j, type) to the list (the count may pass the capacity:
 * the host grows the list and re-runs the cycle) */
__device__ static inline void nbg_emit_event(DevCtl *ctl, ull *keys, ll cap, ll i, ll j, int type)
{
    const ll slot = (ll)atomicAdd((unsigned long long *)&ctl->ev_count, 1ull);
    if (slot < cap) keys[slot] = ((ull)i << 32) | ((ull)j << 2) | (ull)type;
}

/* k_bh.cu (compiled with --fmad=false) */
int nbg_bh_alloc(BhTree &t, ll cap, ll node_cap);
void nbg_bh_free(BhTree &t);
void nbg_launch_bh(const CycleBufs &cb, DevCtl *ctl, cudaStream_t st, bool mixed);
int nbg_bh_launches(const CycleBufs &cb, bool mixed); /* kernels nbg_launch_bh launches */

/* k_cycle.cu (compiled with --fmad=false) */
void nbg_launch_begin(const CycleBufs &cb, DevCtl *ctl, cudaStream_t st);
void nbg_launch_frag_count(const CycleBufs &cb, DevCtl *ctl, cudaStream_t st);
void nbg_launch_pair_fp64(const CycleBufs &cb, DevCtl *ctl, cudaStream_t st);
void nbg_launch_after_pair(const CycleBufs &cb, DevCtl *ctl, cudaStream_t st, bool carry_order);
/* sim < 0: every collection (the whole array) */
void nbg_launch_remove(const CycleBufs &cb, DevCtl *ctl, int sim, ll count, ll *removed_dev, cudaStream_t st);
void nbg_launch_edits(const CycleBufs &cb, DevCtl *ctl, int sim, const nbg_edit *edits_dev, ll k, int *results_dev,
                      cudaStream_t st);
void nbg_launch_energy(const CycleBufs &cb, DevCtl *ctl, double *out_dev, cudaStream_t st);
void nbg_launch_find(const CycleBufs &cb, DevCtl *ctl, int sim, ll id, ll *idx_dev, cudaStream_t st);
/* dst[k] = src[index[k]], k < n, every field (index on the device) */
void nbg_launch_gather(const CycleBufs &cb, const BodyArrays &src, const BodyArrays &dst, const ll *index_dev, ll n,
                       cudaStream_t st);
int nbg_pair_fp64_grid(ll cap);
int nbg_pair_fp64_launches(const CycleBufs &cb);
/* largest capacity the plain form stores its pair terms for */
#define NBG_P64_SPLIT_MAX_CAP 65536
#define NBG_P64_SPLIT_JC 2048

/* k_mixed.cu */
void nbg_launch_mixed_prep(const CycleBufs &cb, DevCtl *ctl, cudaStream_t st);
void nbg_launch_mixed_pair(const CycleBufs &cb, DevCtl *ctl, cudaStream_t st);
void nbg_launch_mixed_out(const CycleBufs &cb, DevCtl *ctl, cudaStream_t st);
int nbg_mixed_slots(int device, int variant);
ll nbg_sym_units(ll blocks);
MixVariantInfo nbg_mix_variant_info(int variant);

/* k_sort.cu */
void nbg_launch_spatial_sort(const CycleBufs &cb, DevCtl *ctl, cudaStream_t st);
void nbg_launch_event_radix(const CycleBufs &cb, DevCtl *ctl, cudaStream_t st);
ull *nbg_launch_incidence_radix(const CycleBufs &cb, DevCtl *ctl, int bits, cudaStream_t st);
int nbg_event_radix_launches(const CycleBufs &cb);
ll nbg_sort_scratch_hist(ll cap);

/* k_probe.cu */
int nbg_run_probes(int device, double *fp32, double *fp64, double *mhz);

#endif
