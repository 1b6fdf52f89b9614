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
    int error_what;  /* 1 = bodies, 2 = events, 3 = fragments, 4 = partials */
    int splits;      /* mixed: j-range splits per i-tile for this cycle */
    ll work_next;    /* mixed: next work item for the persistent CTAs */
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
    int pad1;
    /* accumulated over the cycles of one nbg_step call */
    ll acc_steps, acc_interactions, acc_events, acc_frags, acc_removed, acc_nan;
    ll rend_n;       /* renderables written by the last cycle */
    ll last_ev_n;    /* resolved events recorded by the last cycle */
};

struct CycleBufs {
    BodyArrays a;       /* the collection */
    BodyArrays b;       /* compaction target */
    BodyArrays adds;    /* host adds staged for the next Cycle (arrival order) */
    BodyArrays frags;   /* fragments emitted this cycle (arrival order) */
    ll cap, frag_cap, adds_cap;
    ull *ev_keys;
    ull *ev_sort;       /* scratch for sorting when the count exceeds shared memory */
    ll ev_cap;
    nbg_event *ev_out;  /* resolved events of the last cycle */
    nbg_renderable *rend;
    ll *blk_sum;        /* per-block counts for the scans */
    ll *blk_off;
    ll nblk_cap;
    /* mixed form (indexed by sorted position) */
    float4 *jhi, *jlo;
    float4 *tile_c;
    double *part;
    unsigned *perm;     /* sorted position -> body index */
    unsigned *skey[2];  /* radix-sort keys (ping-pong) */
    unsigned *sval;     /* radix-sort values (ping-pong partner of perm) */
    ll *shist;          /* radix-sort digit histogram / offsets */
    int split_cap;
    int slots;          /* resident CTAs of the mixed kernel on this device */
};

#define NBG_SCAN_BLOCK 1024
#define NBG_SCAN_ITEMS 4
#define NBG_SCAN_TILE (NBG_SCAN_BLOCK * NBG_SCAN_ITEMS)

#define NBG_MIX_BLOCK 128
#define NBG_MIX_K 4
#define NBG_MIX_ITILE (NBG_MIX_BLOCK * NBG_MIX_K)
#define NBG_MIX_JT 256

/* k_cycle.cu (compiled with --fmad=false) */
void nbg_launch_begin(const CycleBufs &cb, DevCtl *ctl, cudaStream_t st);
void nbg_launch_frag_count(const CycleBufs &cb, DevCtl *ctl, cudaStream_t st);
void nbg_launch_pair_fp64(const CycleBufs &cb, DevCtl *ctl, cudaStream_t st);
void nbg_launch_after_pair(const CycleBufs &cb, DevCtl *ctl, cudaStream_t st);
void nbg_launch_remove(const CycleBufs &cb, DevCtl *ctl, ll count, ll *removed_dev, cudaStream_t st);
void nbg_launch_edits(const CycleBufs &cb, DevCtl *ctl, const nbg_edit *edits_dev, ll k, int *results_dev, cudaStream_t st);
void nbg_launch_energy(const CycleBufs &cb, DevCtl *ctl, double *out_dev, cudaStream_t st);
void nbg_launch_find(const CycleBufs &cb, DevCtl *ctl, ll id, ll *idx_dev, cudaStream_t st);
int nbg_pair_fp64_grid(ll cap);

/* k_mixed.cu */
void nbg_launch_mixed_prep(const CycleBufs &cb, DevCtl *ctl, cudaStream_t st);
void nbg_launch_mixed_pair(const CycleBufs &cb, DevCtl *ctl, cudaStream_t st);
void nbg_launch_mixed_out(const CycleBufs &cb, DevCtl *ctl, cudaStream_t st);
int nbg_mixed_slots(int device);

/* k_sort.cu */
void nbg_launch_spatial_sort(const CycleBufs &cb, DevCtl *ctl, cudaStream_t st);
ll nbg_sort_scratch_hist(ll cap);

/* k_probe.cu */
int nbg_run_probes(int device, double *fp32, double *fp64, double *mhz);

#endif
