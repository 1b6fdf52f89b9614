/*
 * k_bh.cu - the Barnes-Hut force pass (cmd/body/octree.go) on the GPU.
 *
 * The reference builds a point-region octree by inserting the bodies that
 * exist and are not fragmenting, in array order, into a cube centred on
 * their bounding box (half = max extent / 2 * 1.05, octree.go:136-188); a
 * leaf holds one body, and an occupied leaf that receives another splits
 * into eight children.  Which node each body ends in depends only on the
 * comparisons x >= cx, y >= cy, z >= cz down the tree (octantOf,
 * octree.go:53-65), so the tree is built here without insertion:
 *
 *   1. every tree body descends BH_LEVELS levels with the reference's own
 *      centre arithmetic (cx +- half / 2, half / 2) and records its octant
 *      path, 3 bits a level, as a 63-bit key;
 *   2. the keys are sorted (LSD radix, stable);
 *   3. a node is a key prefix shared by at least one body whose parent holds
 *      two or more: the nodes that start at sorted position p run from the
 *      first level where key p differs from key p - 1 down to the level
 *      where it parts from key p + 1, so their count comes from the two
 *      neighbouring keys, and one scan numbers every node in depth-first
 *      order (position, then level).  That order makes the first child of a
 *      node the next node and the end of its subtree the first node starting
 *      at the end of its body range (the skip pointer), so the force pass
 *      walks the tree without a stack;
 *   4. masses and centres of mass are summed bottom-up, level by level, over
 *      the children in octant order.
 *
 * The force pass (accumForce, octree.go:265-305) walks the tree for every
 * body with the reference's expressions, softening 1e-4 and opening angle
 * 0.3; a sun sums every body directly (CalcForce, octree.go:236-263).  The
 * collision pass (Compute's second loop, body.go:171-186) becomes a range
 * query on the same tree: nodes whose cube lies farther than r_i + r_max are
 * skipped, and every body that remains is tested with the reference's exact
 * dist <= r_i + r_j, so the event set is the O(N^2) loop's.  Bodies outside
 * the tree (not existing, fragmenting, or not finite) are tested one by one.
 *
 * Against the reference's tree:
 *  - the tree and the opening decisions are the same; a node's centre of
 *    mass is sum(m x) / sum(m) instead of the reference's running update,
 *    which differs in the last bits (a one-body leaf is x * m / m, as in the
 *    reference).  The reference's node whose first inserted body is massless
 *    has a NaN centre (0 / 0) and is therefore always opened; that is kept;
 *  - keys have 21 levels; bodies that share a node at that depth (closer
 *    than 2^-20 of the root cube) stay together in one leaf and each acts as
 *    a leaf of its own, where the reference keeps splitting (and recurses
 *    without end for two bodies at one position);
 *  - the sun's direct sum is a parallel reduction, not array order.
 *
 * Several collections (nbg_set_collections): one tree per collection, each
 * exactly the tree a context holding that collection alone builds.  Every
 * collection gets its own bounding box and root cube; after the key passes
 * the sort takes two more stable passes on the collection index (tree
 * bodies; the others go last), so each collection's tree bodies are one run
 * of sorted positions, in key order.  Node boundaries are found within each
 * run, the depth-first numbering then puts each collection's nodes in one
 * range with its root first, and the walks, the suns' sums and the collision
 * query stay inside the body's own collection.  Walk groups of 32 bodies
 * start at each collection's first sorted position, as they would alone.
 */
#include "nbg_internal.cuh"
#include "nbg_math.h"
#include "nbg_shared.h"

#define BH_THETA 0.3
#define BH_SOFTENING 1e-4
#define BH_LEVELS 21
#define BH_BLOCK 256
#define BH_RS_BLOCK 256
#define BH_RS_ITEMS 16
#define BH_RS_TILE (BH_RS_BLOCK * BH_RS_ITEMS)
#define BH_RS_BINS 256
#define BH_SCAN_BLOCK 1024
#define BH_SCAN_ITEMS 4
#define BH_SCAN_TILE (BH_SCAN_BLOCK * BH_SCAN_ITEMS)
#define BH_F_LEAF 1u
#define BH_F_NAN_CM 2u
#define FULL_MASK 0xffffffffu

/* order-preserving integer image of a double (for atomicMin / atomicMax) */
__device__ __forceinline__ ull dbl_ord(double v)
{
    const ull b = (ull)__double_as_longlong(v);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double ord_dbl(ull o)
{
    const ull b = (o >> 63) ? (o & 0x7fffffffffffffffull) : ~o;
    return __longlong_as_double((long long)b);
}

__device__ __forceinline__ bool tree_body(const BodyArrays &A, ll k)
{
    if ((A.flags[k] & NBG_LIVE_MASK) != NBG_F_EXISTS) return false;
    const double x = A.x[k], y = A.y[k], z = A.z[k];
    return fabs(x) <= NBG_DBL_MAX && fabs(y) <= NBG_DBL_MAX && fabs(z) <= NBG_DBL_MAX;
}

/* the root cube of collection s, octree.go:174-183 */
__device__ __forceinline__ void bh_root(const BhTree &t, int s, double &cx, double &cy, double &cz, double &half)
{
    const ull *b = t.sbox + 6 * (ll)s;
    const double minX = ord_dbl(b[0]), minY = ord_dbl(b[1]), minZ = ord_dbl(b[2]);
    const double maxX = ord_dbl(b[3]), maxY = ord_dbl(b[4]), maxZ = ord_dbl(b[5]);
    cx = (minX + maxX) / 2;
    cy = (minY + maxY) / 2;
    cz = (minZ + maxZ) / 2;
    half = nbg_go_max(maxX - minX, nbg_go_max(maxY - minY, maxZ - minZ)) / 2 * 1.05;
}

/* ---- 1. bounds, keys -------------------------------------------------------- */

/* empty boxes and counts for every collection */
__global__ void __launch_bounds__(1024) k_bh_reset(DevCtl *ctl, SimSegs seg, BhTree t)
{
    if (ctl->error) return;
    for (int s = threadIdx.x; s < seg.nsims; s += blockDim.x) {
        ull *b = t.sbox + 6 * (ll)s;
        for (int c = 0; c < 3; c++) {
            b[c] = ~0ull;
            b[3 + c] = 0ull;
        }
        t.scount[s] = 0;
    }
}

/* each collection's bounding box and tree-body count, and the largest
 * radius of any body */
__global__ void __launch_bounds__(BH_BLOCK) k_bh_bounds(BodyArrays A, DevCtl *ctl, SimSegs seg, BhTree t)
{
    if (ctl->error) return;
    const ll n = ctl->n;
    const int lane = threadIdx.x & 31;
    double rmax = 0;
    /* warp-uniform trip count: every lane takes part in the reductions */
    for (ll base = (ll)blockIdx.x * blockDim.x; base < n; base += (ll)gridDim.x * blockDim.x) {
        const ll k = base + threadIdx.x;
        ull lo[3] = {~0ull, ~0ull, ~0ull}, hi[3] = {0ull, 0ull, 0ull};
        unsigned cnt = 0;
        int sim = -1;
        if (k < n) {
            const double r = A.rad[k];
            if (r > rmax) rmax = r;
            sim = nbg_sim_of(seg.off, seg.nsims, k);
            if (tree_body(A, k)) {
                lo[0] = hi[0] = dbl_ord(A.x[k]);
                lo[1] = hi[1] = dbl_ord(A.y[k]);
                lo[2] = hi[2] = dbl_ord(A.z[k]);
                cnt = 1;
            }
        }
        /* bodies lie in collection order, so the collections of a warp are
         * runs of lanes: a segmented reduction down each run leaves its sum
         * in the run's first lane */
        for (int o = 1; o < 32; o <<= 1) {
            const int so = __shfl_down_sync(FULL_MASK, sim, o);
            ull l[3], h[3];
            for (int c = 0; c < 3; c++) {
                l[c] = __shfl_down_sync(FULL_MASK, lo[c], o);
                h[c] = __shfl_down_sync(FULL_MASK, hi[c], o);
            }
            const unsigned co = __shfl_down_sync(FULL_MASK, cnt, o);
            if (lane + o < 32 && so == sim) {
                for (int c = 0; c < 3; c++) {
                    lo[c] = l[c] < lo[c] ? l[c] : lo[c];
                    hi[c] = h[c] > hi[c] ? h[c] : hi[c];
                }
                cnt += co;
            }
        }
        const int sprev = __shfl_up_sync(FULL_MASK, sim, 1);
        if (sim >= 0 && cnt > 0 && (lane == 0 || sprev != sim)) {
            ull *b = t.sbox + 6 * (ll)sim;
            for (int c = 0; c < 3; c++) {
                atomicMin((unsigned long long *)&b[c], (unsigned long long)lo[c]);
                atomicMax((unsigned long long *)&b[3 + c], (unsigned long long)hi[c]);
            }
            atomicAdd((unsigned long long *)&t.scount[sim], (unsigned long long)cnt);
        }
    }
    for (int o = 16; o > 0; o >>= 1) rmax = fmax(rmax, __shfl_xor_sync(FULL_MASK, rmax, o));
    if (lane == 0) atomicMax((unsigned long long *)&ctl->bh_rmax, (unsigned long long)dbl_ord(rmax));
}

/* each collection's first sorted position and first walk group (exclusive
 * scans over the collections, one warp), and the tree-body total */
__global__ void __launch_bounds__(32) k_bh_segs(DevCtl *ctl, SimSegs seg, BhTree t)
{
    if (ctl->error) return;
    const int ns = seg.nsims, lane = threadIdx.x;
    const int per = (ns + 31) / 32;
    const int s0 = lane * per, s1 = s0 + per < ns ? s0 + per : ns;
    ll c = 0, g = 0;
    for (int s = s0; s < s1; s++) {
        c += t.scount[s];
        g += (t.scount[s] + 31) / 32;
    }
    ll xc = c, xg = g;
    for (int o = 1; o < 32; o <<= 1) {
        const ll yc = __shfl_up_sync(FULL_MASK, xc, o), yg = __shfl_up_sync(FULL_MASK, xg, o);
        if (lane >= o) {
            xc += yc;
            xg += yg;
        }
    }
    ll oc = xc - c, og = xg - g;
    for (int s = s0; s < s1; s++) {
        t.stree[s] = oc;
        t.sgrp[s] = og;
        oc += t.scount[s];
        og += (t.scount[s] + 31) / 32;
    }
    if (lane == 31) {
        t.stree[ns] = xc;
        t.sgrp[ns] = xg;
        ctl->bh_count = xc;
    }
}

/* the collection whose run of sorted tree positions holds p (0 <= p < M) */
__device__ __forceinline__ int bh_run_of(const BhTree &t, int nsims, ll p) { return nbg_sim_of(t.stree, nsims, p); }

/* octant path of every tree body in its collection's cube; other bodies
 * get the largest key */
__global__ void __launch_bounds__(BH_BLOCK) k_bh_keys(BodyArrays A, DevCtl *ctl, SimSegs seg, BhTree t, ull *keys,
                                                      unsigned *vals)
{
    if (ctl->error) return;
    const ll n = ctl->n;
    for (ll k = (ll)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (ll)gridDim.x * blockDim.x) {
        ull key = ~0ull;
        if (tree_body(A, k)) {
            const double x = A.x[k], y = A.y[k], z = A.z[k];
            double cx, cy, cz, half;
            bh_root(t, nbg_sim_of(seg.off, seg.nsims, k), cx, cy, cz, half);
            key = 0;
            for (int d = 0; d < BH_LEVELS; d++) {
                const unsigned oct = (x >= cx ? 1u : 0u) | (y >= cy ? 2u : 0u) | (z >= cz ? 4u : 0u);
                key = (key << 3) | oct;
                const double q = half / 2;
                cx = (oct & 1u) ? cx + q : cx - q;
                cy = (oct & 2u) ? cy + q : cy - q;
                cz = (oct & 4u) ? cz + q : cz - q;
                half = half / 2;
            }
        }
        keys[k] = key;
        vals[k] = (unsigned)k;
    }
}

/* ---- 2. 64-bit LSD radix sort (stable) ----------------------------------- */

/* The digit of a sort pass: 8 bits of the key (simpass < 0), or, in the
 * two passes that group the tree bodies by collection, 8 bits of the
 * collection index (nsims for a body outside the trees, so those go last) */
__device__ __forceinline__ unsigned bh_digit(const SimSegs &seg, ull key, unsigned val, int shift, int simpass)
{
    if (simpass < 0) return (unsigned)(key >> shift) & 0xffu;
    const unsigned d = key == ~0ull ? (unsigned)seg.nsims : (unsigned)nbg_sim_of(seg.off, seg.nsims, (ll)val);
    return (d >> (8 * simpass)) & 0xffu;
}

__global__ void __launch_bounds__(BH_RS_BLOCK) k_bh_rs_hist(DevCtl *ctl, SimSegs seg, const ull *keys,
                                                          const unsigned *vals, int shift, int simpass, ll *hist)
{
    __shared__ unsigned cnt[BH_RS_BINS];
    if (ctl->error) return;
    const ll n = ctl->n;
    const ll nb = (n + BH_RS_TILE - 1) / BH_RS_TILE;
    const ll b = blockIdx.x;
    if (b >= nb) return;
    for (int d = threadIdx.x; d < BH_RS_BINS; d += BH_RS_BLOCK) cnt[d] = 0;
    __syncthreads();
    for (int q = 0; q < BH_RS_ITEMS; q++) {
        const ll k = b * BH_RS_TILE + (ll)q * BH_RS_BLOCK + threadIdx.x;
        if (k < n) atomicAdd(&cnt[bh_digit(seg, keys[k], vals[k], shift, simpass)], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < BH_RS_BINS; d += BH_RS_BLOCK) hist[(ll)d * nb + b] = cnt[d];
}

/* exclusive scan of the digit-major histogram (one block, four entries per
 * thread per round) */
__global__ void __launch_bounds__(1024) k_bh_rs_scan(DevCtl *ctl, ll *hist)
{
    __shared__ ll warp_tot[32];
    if (ctl->error) return;
    const ll n = ctl->n;
    const ll total = ((n + BH_RS_TILE - 1) / BH_RS_TILE) * BH_RS_BINS;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    ll carry = 0;
    for (ll c0 = 0; c0 < total; c0 += 4096) {
        const ll c = c0 + (ll)threadIdx.x * 4;
        ll v[4], sum = 0;
        for (int q = 0; q < 4; q++) {
            v[q] = c + q < total ? hist[c + q] : 0;
            sum += v[q];
        }
        ll x = sum;
        for (int o = 1; o < 32; o <<= 1) {
            const ll y = __shfl_up_sync(FULL_MASK, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_tot[w] = x;
        __syncthreads();
        if (w == 0) {
            ll t = warp_tot[lane];
            for (int o = 1; o < 32; o <<= 1) {
                const ll y = __shfl_up_sync(FULL_MASK, t, o);
                if (lane >= o) t += y;
            }
            warp_tot[lane] = t;
        }
        __syncthreads();
        ll ex = carry + x - sum + (w > 0 ? warp_tot[w - 1] : 0);
        for (int q = 0; q < 4; q++) {
            if (c + q < total) hist[c + q] = ex;
            ex += v[q];
        }
        carry += warp_tot[31];
        __syncthreads();
    }
}

__global__ void __launch_bounds__(BH_RS_BLOCK) k_bh_rs_scatter(DevCtl *ctl, SimSegs seg, const ull *keys_in,
                                                             const unsigned *vals_in, ull *keys_out,
                                                             unsigned *vals_out, int shift, int simpass,
                                                             const ll *offs)
{
    __shared__ ll base[BH_RS_BINS];
    __shared__ unsigned wcnt[BH_RS_BLOCK / 32][BH_RS_BINS];
    if (ctl->error) return;
    const ll n = ctl->n;
    const ll nb = (n + BH_RS_TILE - 1) / BH_RS_TILE;
    const ll b = blockIdx.x;
    if (b >= nb) return;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int d = threadIdx.x; d < BH_RS_BINS; d += BH_RS_BLOCK) base[d] = offs[(ll)d * nb + b];
    const unsigned lt = (1u << lane) - 1u;
    for (int q = 0; q < BH_RS_ITEMS; q++) {
        for (int d = threadIdx.x; d < BH_RS_BINS * (BH_RS_BLOCK / 32); d += BH_RS_BLOCK) (&wcnt[0][0])[d] = 0;
        __syncthreads();
        const ll k = b * BH_RS_TILE + (ll)q * BH_RS_BLOCK + threadIdx.x;
        const bool ok = k < n;
        const ull key = ok ? keys_in[k] : 0ull;
        const unsigned val = ok ? vals_in[k] : 0u;
        const unsigned d = ok ? bh_digit(seg, key, val, shift, simpass) : BH_RS_BINS;
        const unsigned peers = __match_any_sync(FULL_MASK, d);
        const unsigned rank = __popc(peers & lt);
        if (ok && rank == 0) wcnt[w][d] = __popc(peers);
        __syncthreads();
        if (ok) {
            ll pos = base[d] + rank;
            for (int v = 0; v < w; v++) pos += wcnt[v][d];
            keys_out[pos] = key;
            vals_out[pos] = val;
        }
        __syncthreads();
        for (int dd = threadIdx.x; dd < BH_RS_BINS; dd += BH_RS_BLOCK) {
            ll s = 0;
            for (int v = 0; v < BH_RS_BLOCK / 32; v++) s += wcnt[v][dd];
            base[dd] += s;
        }
        __syncthreads();
    }
}

/* ---- 3. nodes -------------------------------------------------------------- */

/* levels two keys have in common (BH_LEVELS when equal) */
__device__ __forceinline__ int common_levels(ull a, ull b)
{
    const ull x = a ^ b;
    if (x == 0) return BH_LEVELS;
    return (__clzll((long long)x) - 1) / 3;
}

/* first and last level of the nodes that start at sorted position p of its
 * collection's run [lo, hi) (none when first > last) */
__device__ __forceinline__ void node_levels(const ull *keys, ll p, ll lo, ll hi, int &d0, int &d1)
{
    const int cp = p == lo ? -1 : common_levels(keys[p - 1], keys[p]);
    const int cn = p == hi - 1 ? -1 : common_levels(keys[p], keys[p + 1]);
    d0 = p == lo ? 0 : cp + 1;
    const int e = cn + 1 > d0 ? cn + 1 : d0;
    d1 = e < BH_LEVELS ? e : BH_LEVELS;
}

/* per-block sums of the node counts of sorted positions [0, M) */
__global__ void __launch_bounds__(BH_SCAN_BLOCK) k_bh_count(DevCtl *ctl, SimSegs seg, BhTree t, const ull *keys,
                                                            ll *base, ll *blk)
{
    __shared__ ll red[BH_SCAN_BLOCK / 32];
    if (ctl->error) return;
    const ll M = ctl->bh_count;
    const ll b0 = (ll)blockIdx.x * BH_SCAN_TILE;
    if (b0 > M) return;
    ll s = 0;
    for (int q = 0; q < BH_SCAN_ITEMS; q++) {
        const ll p = b0 + (ll)q * BH_SCAN_BLOCK + threadIdx.x;
        ll c = 0;
        if (p < M) {
            const int r = bh_run_of(t, seg.nsims, p);
            int d0, d1;
            node_levels(keys, p, t.stree[r], t.stree[r + 1], d0, d1);
            c = d1 >= d0 ? d1 - d0 + 1 : 0;
        }
        if (p <= M) base[p] = c; /* base[M] = 0: the scan leaves the total there */
        s += c;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL_MASK, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        ll t = 0;
        for (int w = 0; w < BH_SCAN_BLOCK / 32; w++) t += red[w];
        blk[blockIdx.x] = t;
    }
}

/* exclusive scan of the block sums (one block) and the node total */
__global__ void __launch_bounds__(1024) k_bh_count_top(DevCtl *ctl, ll *blk, ll node_cap)
{
    __shared__ ll warp_tot[32];
    if (ctl->error) return;
    const ll M = ctl->bh_count;
    const ll nblk = M / BH_SCAN_TILE + 1;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    ll carry = 0;
    for (ll c0 = 0; c0 < nblk; c0 += 1024) {
        const ll c = c0 + threadIdx.x;
        const ll v = c < nblk ? blk[c] : 0;
        ll x = v;
        for (int o = 1; o < 32; o <<= 1) {
            const ll y = __shfl_up_sync(FULL_MASK, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_tot[w] = x;
        __syncthreads();
        if (w == 0) {
            ll t = warp_tot[lane];
            for (int o = 1; o < 32; o <<= 1) {
                const ll y = __shfl_up_sync(FULL_MASK, t, o);
                if (lane >= o) t += y;
            }
            warp_tot[lane] = t;
        }
        __syncthreads();
        if (c < nblk) blk[c] = carry + x - v + (w > 0 ? warp_tot[w - 1] : 0);
        carry += warp_tot[31];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        ctl->bh_nodes = carry;
        if (carry > node_cap) {
            ctl->error = NBG_E_OVERFLOW;
            ctl->error_what = 5;
            ctl->error_need = carry;
        }
    }
}

/* exclusive scan of the node counts within each block, plus the block's
 * offset: base[p] = first node starting at p, base[M] = node total */
__global__ void __launch_bounds__(BH_SCAN_BLOCK) k_bh_count_scan(DevCtl *ctl, ll *base, const ll *blk)
{
    __shared__ ll warp_tot[32];
    if (ctl->error) return;
    const ll M = ctl->bh_count;
    const ll b0 = (ll)blockIdx.x * BH_SCAN_TILE;
    if (b0 > M) return;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    ll carry = blk[blockIdx.x];
    for (int q = 0; q < BH_SCAN_ITEMS; q++) {
        const ll p = b0 + (ll)q * BH_SCAN_BLOCK + threadIdx.x;
        const ll v = p <= M ? base[p] : 0;
        ll x = v;
        for (int o = 1; o < 32; o <<= 1) {
            const ll y = __shfl_up_sync(FULL_MASK, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_tot[w] = x;
        __syncthreads();
        if (w == 0) {
            ll t = warp_tot[lane];
            for (int o = 1; o < 32; o <<= 1) {
                const ll y = __shfl_up_sync(FULL_MASK, t, o);
                if (lane >= o) t += y;
            }
            warp_tot[lane] = t;
        }
        __syncthreads();
        if (p <= M) base[p] = carry + x - v + (w > 0 ? warp_tot[w - 1] : 0);
        carry += warp_tot[31];
        __syncthreads();
    }
}

/* each collection's root node: the first node of its run (nodes of an
 * empty collection: the empty range at the next one's root) */
__global__ void __launch_bounds__(1024) k_bh_roots(DevCtl *ctl, SimSegs seg, BhTree t, const ll *base)
{
    if (ctl->error) return;
    for (int s = threadIdx.x; s <= seg.nsims; s += blockDim.x) t.sroot[s] = base[t.stree[s]];
}

/* one thread per sorted position: every node that starts there */
__global__ void __launch_bounds__(BH_BLOCK) k_bh_nodes(DevCtl *ctl, SimSegs seg, const ull *keys, const ll *base,
                                                       BhTree t)
{
    if (ctl->error) return;
    const ll M = ctl->bh_count;
    const ll total = ctl->bh_nodes;
    for (ll p = (ll)blockIdx.x * blockDim.x + threadIdx.x; p < M; p += (ll)gridDim.x * blockDim.x) {
        const int r = bh_run_of(t, seg.nsims, p);
        const ll lo = t.stree[r], hi = t.stree[r + 1];
        int d0, d1;
        node_levels(keys, p, lo, hi, d0, d1);
        if (d1 < d0) continue;
        const ull key = keys[p];
        /* the cube of the level-d0 node: descend d0 levels along the key */
        double cx, cy, cz, half;
        bh_root(t, r, cx, cy, cz, half);
        for (int d = 0; d < d0; d++) {
            const unsigned oct = (unsigned)(key >> (3 * (BH_LEVELS - 1 - d))) & 7u;
            const double q = half / 2;
            cx = (oct & 1u) ? cx + q : cx - q;
            cy = (oct & 2u) ? cy + q : cy - q;
            cz = (oct & 4u) ? cz + q : cz - q;
            half = half / 2;
        }
        for (int d = d0; d <= d1; d++) {
            const ll id = base[p] + (d - d0);
            /* end of the body range: the first key of the run past this
             * node's prefix */
            ll end = hi;
            if (d > 0) {
                const int sh = 3 * (BH_LEVELS - d);
                const ull pre = key >> sh;
                ll a = p + 1, b = hi;
                while (a < b) {
                    const ll mid = (a + b) >> 1;
                    if ((keys[mid] >> sh) <= pre)
                        a = mid + 1;
                    else
                        b = mid;
                }
                end = a;
            }
            t.start[id] = (int)p;
            t.end[id] = (int)end;
            t.skip[id] = (int)(end >= M ? total : base[end]);
            t.level[id] = (unsigned char)d;
            t.flags[id] = (end - p == 1 || d == BH_LEVELS) ? BH_F_LEAF : 0u;
            t.cx[id] = cx;
            t.cy[id] = cy;
            t.cz[id] = cz;
            t.half[id] = half;
            t.fd[id] = make_float4((float)cx, (float)cy, (float)cz, (float)half);
            if (d < d1) {
                const unsigned oct = (unsigned)(key >> (3 * (BH_LEVELS - 1 - d))) & 7u;
                const double q = half / 2;
                cx = (oct & 1u) ? cx + q : cx - q;
                cy = (oct & 2u) ? cy + q : cy - q;
                cz = (oct & 4u) ? cz + q : cz - q;
                half = half / 2;
            }
        }
    }
}

/* ---- 4. mass and centre of mass, one level per launch, deepest first ------ */

__global__ void __launch_bounds__(BH_BLOCK) k_bh_mass(BodyArrays A, DevCtl *ctl, const unsigned *vals, BhTree t,
                                                      int level)
{
    if (ctl->error) return;
    const ll total = ctl->bh_nodes;
    for (ll id = (ll)blockIdx.x * blockDim.x + threadIdx.x; id < total; id += (ll)gridDim.x * blockDim.x) {
        if (t.level[id] != level) continue;
        double M = 0, mx = 0, my = 0, mz = 0;
        int first = 0x7fffffff;
        if (t.flags[id] & BH_F_LEAF) {
            for (int q = t.start[id]; q < t.end[id]; q++) {
                const unsigned k = vals[q];
                const double m = A.m[k];
                M = M + m;
                mx = mx + A.x[k] * m;
                my = my + A.y[k] * m;
                mz = mz + A.z[k] * m;
                if ((int)k < first) first = (int)k;
            }
        } else {
            const int stop = t.skip[id];
            for (int c = (int)id + 1; c < stop; c = t.skip[c]) {
                M = M + t.mass[c];
                mx = mx + t.mx[c];
                my = my + t.my[c];
                mz = mz + t.mz[c];
                if (t.first[c] < first) first = t.first[c];
            }
        }
        t.mass[id] = M;
        t.mx[id] = mx;
        t.my[id] = my;
        t.mz[id] = mz;
        t.first[id] = first;
        if (M != 0) {
            t.cmx[id] = mx / M;
            t.cmy[id] = my / M;
            t.cmz[id] = mz / M;
        }
        /* the reference's running centre is 0 / 0 when the node's first body
         * (in array order) is massless, and stays NaN */
        if (A.m[first] == 0) t.flags[id] |= BH_F_NAN_CM;
    }
}

/* ---- 5. forces ------------------------------------------------------------- */

/* accumForce's point-mass term, octree.go:286-292 */
__device__ __forceinline__ void bh_term(double gm_i, double M, double dx, double dy, double dz, double &fx,
                                        double &fy, double &fz)
{
    const double distSq = dx * dx + dy * dy + dz * dz + BH_SOFTENING * BH_SOFTENING;
    const double dist = sqrt(distSq);
    const double force = gm_i * M / distSq;
    fx += force * dx / dist;
    fy += force * dy / dist;
    fz += force * dz / dist;
}

/* The next group of 32 consecutive sorted bodies for this warp, or -1.  Walk
 * times vary with the bodies' surroundings, so warps take groups from one
 * queue until it is empty instead of a fixed share each: no SM idles while
 * another still holds a long run of groups.  A group is always the same 32
 * bodies, so the results do not depend on which warp takes it. */
__device__ __forceinline__ int bh_next_group(DevCtl *ctl, ll groups)
{
    unsigned g = 0;
    if ((threadIdx.x & 31) == 0) g = atomicAdd(&ctl->bh_next, 1u);
    g = __shfl_sync(FULL_MASK, g, 0);
    return (ll)g < groups ? (int)g : -1;
}

/* Group g holds sorted positions [p0, p1) of collection s: the groups of a
 * collection start at its first sorted position, 32 bodies each, so a
 * collection's groups are those it would have alone. */
__device__ __forceinline__ void bh_group(const BhTree &t, int nsims, int g, int &s, ll &p0, ll &p1)
{
    s = nbg_sim_of(t.sgrp, nsims, g);
    p0 = t.stree[s] + 32ll * (g - t.sgrp[s]);
    p1 = p0 + 32 < t.stree[s + 1] ? p0 + 32 : t.stree[s + 1];
}

/* one thread per tree body (sorted order, so a warp walks nearby paths) */
__global__ void __launch_bounds__(BH_BLOCK) k_bh_force(BodyArrays A, DevCtl *ctl, SimSegs seg, const unsigned *vals,
                                                       BhTree t)
{
    if (ctl->error) return;
    const ll groups = t.sgrp[seg.nsims];
    unsigned long long terms = 0;
    /* every lane runs the same number of rounds, for the warp reduction */
    for (int grp; (grp = bh_next_group(ctl, groups)) >= 0;) {
        int r;
        ll p0, p1;
        bh_group(t, seg.nsims, grp, r, p0, p1);
        const ll p = p0 + (threadIdx.x & 31);
        if (p >= p1) continue;
        const int total = (int)t.sroot[r + 1]; /* the end of the collection's nodes */
        const unsigned k = vals[p];
        if (A.flags[k] & NBG_F_IS_SUN) continue; /* k_bh_sun */
        const double x = A.x[k], y = A.y[k], z = A.z[k];
        const double gm = NBG_G * A.m[k];
        double fx = 0, fy = 0, fz = 0;
        int id = (int)t.sroot[r];
        while (id < total) {
            const double Mn = t.mass[id];
            if (Mn == 0) {
                id = t.skip[id];
                continue;
            }
            const unsigned fl = t.flags[id];
            const bool leaf = (fl & BH_F_LEAF) != 0;
            const double dx = t.cmx[id] - x;
            const double dy = t.cmy[id] - y;
            const double dz = t.cmz[id] - z;
            const double distSq = dx * dx + dy * dy + dz * dz + BH_SOFTENING * BH_SOFTENING;
            const double dist = sqrt(distSq);
            if (leaf || (!(fl & BH_F_NAN_CM) && (2 * t.half[id] / dist) < BH_THETA)) {
                const int s = t.start[id], e = t.end[id];
                if (leaf && e - s > 1) {
                    /* a leaf at the deepest level holding several bodies: each
                     * acts as a leaf of its own */
                    for (int q = s; q < e; q++) {
                        const unsigned j = vals[q];
                        const double mj = A.m[j];
                        if (j == k || mj == 0) continue;
                        bh_term(gm, mj, A.x[j] * mj / mj - x, A.y[j] * mj / mj - y, A.z[j] * mj / mj - z, fx, fy,
                                fz);
                        terms++;
                    }
                } else if (!(leaf && vals[s] == k)) {
                    const double force = gm * Mn / distSq;
                    fx += force * dx / dist;
                    fy += force * dy / dist;
                    fz += force * dz / dist;
                    terms++;
                }
                id = t.skip[id];
            } else {
                id = id + 1;
            }
        }
        A.fx[k] = fx;
        A.fy[k] = fy;
        A.fz[k] = fz;
    }
    /* point-mass terms summed, for the measured work */
    for (int o = 16; o > 0; o >>= 1) terms += __shfl_xor_sync(FULL_MASK, terms, o);
    if ((threadIdx.x & 31) == 0 && terms) atomicAdd((unsigned long long *)&ctl->acc_bh_terms, terms);
}

/* ---- 5b. the mixed-precision walk --------------------------------------------
 * The same tree and the same acceptance rule in FP32: centres of mass as
 * hi/lo float pairs (so dx = (cm_hi - x_hi) + (cm_lo - x_lo) keeps ~2^-24 of
 * |dx|), masses relative to the root's, the opening test as
 * r^2 > (2 half / theta)^2 on the softened r^2, and the reciprocal square
 * root of the SFU.  The 32 bodies of a warp (neighbours in key order) walk
 * one node sequence together: a lane that accepts a node waits until the
 * warp leaves that node's subtree (its skip pointer), and the warp descends
 * when any lane opens, so every node load is a broadcast and no lane
 * diverges.  A node with no mass below it is skipped by every lane.  Each
 * lane sums its terms in FP32 and, every 64 nodes, the warp folds them into
 * (hi, lo) FP32 pairs: the GB300 FP64 pipe is 1/64 of the FP32 rate, and a
 * few FP64 folds per node kept it saturated. */
__global__ void __launch_bounds__(BH_BLOCK) k_bh_prep_mixed(DevCtl *ctl, SimSegs seg, BhTree t)
{
    if (ctl->error) return;
    const ll total = ctl->bh_nodes;
    if (total <= 0) return;
    for (ll id = (ll)blockIdx.x * blockDim.x + threadIdx.x; id < total; id += (ll)gridDim.x * blockDim.x) {
        /* masses relative to the root of the node's own tree */
        const double mroot = t.mass[t.sroot[nbg_sim_of(t.sroot, seg.nsims, id)]];
        const double inv_root = mroot != 0 ? 1.0 / mroot : 0.0;
        const double M = t.mass[id];
        float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = make_float4(0.f, 0.f, 0.f, 0.f);
        if (M != 0) {
            const double cx = t.cmx[id], cy = t.cmy[id], cz = t.cmz[id];
            a.x = (float)cx;
            a.y = (float)cy;
            a.z = (float)cz;
            b.x = (float)(cx - (double)a.x);
            b.y = (float)(cy - (double)a.y);
            b.z = (float)(cz - (double)a.z);
            a.w = (float)(M * inv_root);
            const double o = 2 * t.half[id] / BH_THETA;
            b.w = (float)(o * o);
        }
        t.fa[id] = a;
        t.fb[id] = b;
        t.fc[id] = make_int4(t.skip[id], t.start[id], t.end[id], (int)t.flags[id]);
    }
}

/* (hi, lo) += v with the rounding error of hi + v kept in lo (TwoSum) */
__device__ __forceinline__ void fold2(float &hi, float &lo, float v)
{
    const float s = hi + v;
    const float bb = s - hi;
    const float e = (hi - (s - bb)) + (v - bb);
    hi = s;
    lo += e;
}

__device__ __forceinline__ float bh_rsqrt(float x)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

/* the terms of a leaf at the deepest level holding bodies [s, e) (rare; kept
 * out of the walk's registers) */
__device__ __noinline__ int bucket_terms(const BodyArrays &A, const unsigned *vals, int s, int e, unsigned k, float xh,
                                         float yh, float zh, float xl, float yl, float zl, float soft2, double mroot,
                                         float &ax, float &ay, float &az)
{
    int cnt = 0;
    for (int q = s; q < e; q++) {
        const unsigned j = vals[q];
        const double mj = A.m[j];
        if (j == k || mj == 0) continue;
        const float ex = (float)(A.x[j] - (double)xh - (double)xl);
        const float ey = (float)(A.y[j] - (double)yh - (double)yl);
        const float ez = (float)(A.z[j] - (double)zh - (double)zl);
        const float q2 = ex * ex + ey * ey + ez * ez + soft2;
        const float inv = bh_rsqrt(q2);
        const float w = (float)(mj / mroot) * inv * inv * inv;
        ax += w * ex;
        ay += w * ey;
        az += w * ez;
        cnt++;
    }
    return cnt;
}

template <int MINB>
__global__ void __launch_bounds__(BH_BLOCK, MINB) k_bh_force_mixed(BodyArrays A, DevCtl *ctl, SimSegs seg,
                                                                const unsigned *vals, BhTree t)
{
    if (ctl->error) return;
    if (ctl->bh_nodes <= 0) return;
    const ll groups = t.sgrp[seg.nsims];
    const float soft2 = (float)(BH_SOFTENING * BH_SOFTENING);
    unsigned long long terms = 0;
    for (int grp; (grp = bh_next_group(ctl, groups)) >= 0;) {
        int r;
        ll p0, p1;
        bh_group(t, seg.nsims, grp, r, p0, p1);
        const ll p = p0 + (threadIdx.x & 31);
        const int root = (int)t.sroot[r], total = (int)t.sroot[r + 1];
        const double mroot = t.mass[root];
        unsigned k = 0;
        bool have = p < p1;
        if (have) {
            k = vals[p];
            have = !(A.flags[k] & NBG_F_IS_SUN); /* k_bh_sun */
        }
        float xh = 0.f, yh = 0.f, zh = 0.f, xl = 0.f, yl = 0.f, zl = 0.f;
        if (have) {
            const double x = A.x[k], y = A.y[k], z = A.z[k];
            xh = (float)x;
            yh = (float)y;
            zh = (float)z;
            xl = (float)(x - (double)xh);
            yl = (float)(y - (double)yh);
            zl = (float)(z - (double)zh);
        }
        int wait = have ? 0 : 0x7fffffff;
        float ax = 0.f, ay = 0.f, az = 0.f;
        /* every 64 nodes the warp folds the FP32 partial sums into (hi, lo)
         * FP32 pairs (TwoSum): all lanes together, and no FP64 in the walk */
        float hx = 0.f, lx = 0.f, hy = 0.f, ly = 0.f, hz = 0.f, lz = 0.f;
        int nacc = 0, steps = 0;
        if (!__any_sync(FULL_MASK, have)) continue;
        /* The next node is the first child when any lane opens this one, and
         * otherwise this node's skip pointer: every lane that waits at this
         * node accepted an ancestor, whose subtree ends at or after this
         * node's.  So the next address is known right after the vote, and its
         * loads are in flight while the lanes add their terms. */
        int id = root;
        float4 a = t.fa[root], b = t.fb[root];
        int4 c = t.fc[root];
        while (id < total) {
            const int sk = c.x;
            const unsigned fl = (unsigned)c.w;
            const bool leaf = (fl & BH_F_LEAF) != 0;
            const bool live = a.w != 0.f; /* nothing with mass below: skipped by every lane */
            const bool active = live && id >= wait;
            const float dx = (a.x - xh) + (b.x - xl);
            const float dy = (a.y - yh) + (b.y - yl);
            const float dz = (a.z - zh) + (b.z - zl);
            const float r2 = dx * dx + dy * dy + dz * dz + soft2;
            const bool accept = leaf || (!(fl & BH_F_NAN_CM) && r2 > b.w);
            const int next = __any_sync(FULL_MASK, active && !accept) ? id + 1 : sk;
            const int s = c.y, e = c.z;
            const float mw = a.w;
            if (next < total) {
                a = t.fa[next];
                b = t.fb[next];
                c = t.fc[next];
            }
            if (active && accept) {
                if (leaf && e - s > 1) {
                    nacc += bucket_terms(A, vals, s, e, k, xh, yh, zh, xl, yl, zl, soft2, mroot, ax, ay, az);
                } else if (!(leaf && (ll)s == p)) { /* a one-body leaf holds sorted position s */
                    const float inv = bh_rsqrt(r2);
                    const float w = mw * inv * inv * inv;
                    ax += w * dx;
                    ay += w * dy;
                    az += w * dz;
                    nacc++;
                }
                wait = sk;
            }
            if (++steps == 64) {
                fold2(hx, lx, ax);
                fold2(hy, ly, ay);
                fold2(hz, lz, az);
                ax = ay = az = 0.f;
                steps = 0;
            }
            id = next;
        }
        if (have) {
            terms += nacc;
            const double gm = NBG_G * A.m[k] * mroot;
            A.fx[k] = gm * (((double)hx + (double)lx) + (double)ax);
            A.fy[k] = gm * (((double)hy + (double)ly) + (double)ay);
            A.fz[k] = gm * (((double)hz + (double)lz) + (double)az);
        }
    }
    for (int o = 16; o > 0; o >>= 1) terms += __shfl_xor_sync(FULL_MASK, terms, o);
    if ((threadIdx.x & 31) == 0 && terms) atomicAdd((unsigned long long *)&ctl->acc_bh_terms, terms);
}

/* a sun sums every tree body directly (directForce, octree.go:310-325): each
 * CTA scans a run of bodies for suns, and sums every sun it finds with all
 * its threads, in a fixed-order block reduction */
__global__ void __launch_bounds__(BH_BLOCK) k_bh_sun(BodyArrays A, DevCtl *ctl, SimSegs seg)
{
    __shared__ double red[3][BH_BLOCK];
    __shared__ unsigned s_mask[BH_BLOCK / 32];
    if (ctl->error) return;
    const ll n = ctl->n;
    for (ll base = (ll)blockIdx.x * BH_BLOCK; base < n; base += (ll)gridDim.x * BH_BLOCK) {
        const ll mine = base + threadIdx.x;
        const bool sun = mine < n &&
                         (A.flags[mine] & (NBG_LIVE_MASK | NBG_F_IS_SUN)) == (NBG_F_EXISTS | NBG_F_IS_SUN) &&
                         tree_body(A, mine);
        const unsigned m = __ballot_sync(FULL_MASK, sun);
        if ((threadIdx.x & 31) == 0) s_mask[threadIdx.x >> 5] = m;
        __syncthreads();
        for (int w = 0; w < BH_BLOCK / 32; w++) {
            unsigned bits = s_mask[w];
            while (bits) {
                const int lane = __ffs(bits) - 1;
                bits &= bits - 1;
                const ll k = base + w * 32 + lane;
                const double x = A.x[k], y = A.y[k], z = A.z[k];
                const double gm = NBG_G * A.m[k];
                double fx = 0, fy = 0, fz = 0;
                /* the bodies of the sun's own collection, each thread the
                 * same share of them as if the collection were alone */
                const int sim = nbg_sim_of(seg.off, seg.nsims, k);
                const ll j0 = seg.off[sim], j1 = seg.off[sim + 1];
                for (ll j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
                    if (j == k || (A.flags[j] & NBG_LIVE_MASK) != NBG_F_EXISTS) continue;
                    bh_term(gm, A.m[j], A.x[j] - x, A.y[j] - y, A.z[j] - z, fx, fy, fz);
                }
                red[0][threadIdx.x] = fx;
                red[1][threadIdx.x] = fy;
                red[2][threadIdx.x] = fz;
                __syncthreads();
                for (int st = BH_BLOCK / 2; st > 0; st >>= 1) {
                    if (threadIdx.x < st)
                        for (int q = 0; q < 3; q++) red[q][threadIdx.x] += red[q][threadIdx.x + st];
                    __syncthreads();
                }
                if (threadIdx.x == 0) {
                    A.fx[k] = red[0][0];
                    A.fy[k] = red[1][0];
                    A.fz[k] = red[2][0];
                }
                __syncthreads();
            }
        }
        __syncthreads(); /* s_mask is rewritten for the next run */
    }
}

/* ---- 6. collisions: Compute's second pass as a range query ----------------- */

/* Collided + the event rules for tree body i against body j (j != i) */
__device__ __forceinline__ void bh_test_pair(const BodyArrays &A, DevCtl *ctl, ull *ev_keys, ll ev_cap, ll i,
                                             double xi, double yi, double zi, double ri, unsigned bi, ll j)
{
    const double dx = A.x[j] - xi;
    const double dy = A.y[j] - yi;
    const double dz = A.z[j] - zi;
    const double dist = sqrt(dx * dx + dy * dy + dz * dz);
    const double rj = A.rad[j];
    if (dist <= ri + rj) {
        const int type = nbg_detect_event(bi, NBG_BEHAVIOR(A.flags[j]), ri, rj, dist);
        if (type >= 0) nbg_emit_event(ctl, ev_keys, ev_cap, i, j, type);
    }
}

__global__ void __launch_bounds__(BH_BLOCK) k_bh_collide(BodyArrays A, DevCtl *ctl, SimSegs seg,
                                                         const unsigned *vals, BhTree t, ull *ev_keys, ll ev_cap)
{
    if (ctl->error) return;
    const ll n = ctl->n;
    const ll M = ctl->bh_count;
    const double rmax = ord_dbl(ctl->bh_rmax);
    for (ll p = (ll)blockIdx.x * blockDim.x + threadIdx.x; p < M; p += (ll)gridDim.x * blockDim.x) {
        const int r = bh_run_of(t, seg.nsims, p);
        double cx0, cy0, cz0, half0;
        bh_root(t, r, cx0, cy0, cz0, half0);
        /* every coordinate, centre and half in the tree is at most this large */
        const float span = (float)((fabs(cx0) + fabs(cy0) + fabs(cz0) + 3 * half0) * (1.0 + 0x1p-20));
        const int total = (int)t.sroot[r + 1];
        const unsigned i = vals[p];
        const unsigned fi = A.flags[i];
        if (fi & NBG_F_COLLIDED) continue; /* Collided's guard (always clear here) */
        const double xi = A.x[i], yi = A.y[i], zi = A.z[i], ri = A.rad[i];
        const unsigned bi = NBG_BEHAVIOR(fi);
        /* The cube test runs in FP32 and only prunes: a node is skipped when
         * its cube lies farther than r_i + r_max plus a bound on every FP32
         * rounding of the coordinates, centres, halves and the test itself
         * (2^-18 of the tree's span); the pairs that remain get the exact
         * FP64 test. */
        const double Rd = ri + rmax;
        if (!(Rd >= 0)) continue; /* a NaN radius collides with nothing */
        const float R = (float)(Rd * (1.0 + 0x1p-20)) + span * 0x1p-18f;
        const float R2 = R * R * (1.0f + 0x1p-18f);
        const float xf = (float)xi, yf = (float)yi, zf = (float)zi;
        int id = (int)t.sroot[r];
        while (id < total) {
            const float4 q = t.fd[id];
            const float ax = fmaxf(fabsf(xf - q.x) - q.w, 0.f);
            const float ay = fmaxf(fabsf(yf - q.y) - q.w, 0.f);
            const float az = fmaxf(fabsf(zf - q.z) - q.w, 0.f);
            if (ax * ax + ay * ay + az * az > R2) {
                id = t.skip[id];
                continue;
            }
            if (t.flags[id] & BH_F_LEAF) {
                for (int qq = t.start[id]; qq < t.end[id]; qq++) {
                    const unsigned j = vals[qq];
                    if (j != i) bh_test_pair(A, ctl, ev_keys, ev_cap, i, xi, yi, zi, ri, bi, j);
                }
                id = t.skip[id];
            } else {
                id = id + 1;
            }
        }
        /* bodies of the collection outside its tree: they sit past every
         * tree body in ascending body order, so the collection's are one run */
        const ll lo_b = seg.off[r], hi_b = seg.off[r + 1];
        ll a = M, b = n;
        while (a < b) {
            const ll mid = (a + b) >> 1;
            if ((ll)vals[mid] < lo_b)
                a = mid + 1;
            else
                b = mid;
        }
        for (ll q = a; q < n && (ll)vals[q] < hi_b; q++)
            bh_test_pair(A, ctl, ev_keys, ev_cap, i, xi, yi, zi, ri, bi, vals[q]);
    }
}

/* ---- host side -------------------------------------------------------------- */

int nbg_bh_alloc(BhTree &t, ll cap, ll node_cap)
{
    nbg_bh_free(t);
    const ll nb = (cap + BH_RS_TILE - 1) / BH_RS_TILE;
    const ll nblk = cap / BH_SCAN_TILE + 2;
    bool ok = true;
#define ALLOC(p, cnt) ok = ok && cudaMalloc((void **)&(p), (size_t)(cnt) * sizeof(*(p))) == cudaSuccess
    ALLOC(t.key[0], cap);
    ALLOC(t.key[1], cap);
    ALLOC(t.val[0], cap);
    ALLOC(t.val[1], cap);
    ALLOC(t.hist, nb * BH_RS_BINS);
    ALLOC(t.base, cap + 1);
    ALLOC(t.blk, nblk);
    ALLOC(t.mass, node_cap);
    ALLOC(t.mx, node_cap);
    ALLOC(t.my, node_cap);
    ALLOC(t.mz, node_cap);
    ALLOC(t.cmx, node_cap);
    ALLOC(t.cmy, node_cap);
    ALLOC(t.cmz, node_cap);
    ALLOC(t.cx, node_cap);
    ALLOC(t.cy, node_cap);
    ALLOC(t.cz, node_cap);
    ALLOC(t.half, node_cap);
    ALLOC(t.skip, node_cap);
    ALLOC(t.start, node_cap);
    ALLOC(t.end, node_cap);
    ALLOC(t.first, node_cap);
    ALLOC(t.level, node_cap);
    ALLOC(t.flags, node_cap);
    ALLOC(t.fa, node_cap);
    ALLOC(t.fb, node_cap);
    ALLOC(t.fc, node_cap);
    ALLOC(t.fd, node_cap);
    ALLOC(t.sbox, 6 * (ll)NBG_MAX_SIMS);
    ALLOC(t.scount, NBG_MAX_SIMS + 1);
    ALLOC(t.stree, NBG_MAX_SIMS + 1);
    ALLOC(t.sroot, NBG_MAX_SIMS + 1);
    ALLOC(t.sgrp, NBG_MAX_SIMS + 1);
#undef ALLOC
    if (!ok) {
        nbg_bh_free(t);
        return NBG_E_CUDA;
    }
    t.node_cap = node_cap;
    return NBG_OK;
}

void nbg_bh_free(BhTree &t)
{
    void *ps[] = {t.key[0], t.key[1], t.val[0], t.val[1], t.hist, t.base, t.blk, t.mass, t.mx, t.my,
                  t.mz, t.cmx, t.cmy, t.cmz, t.cx, t.cy, t.cz, t.half, t.skip, t.start,
                  t.end, t.first, t.level, t.flags, t.fa, t.fb, t.fc, t.fd,
                  t.sbox, t.scount, t.stree, t.sroot, t.sgrp};
    for (void *p : ps) cudaFree(p);
    memset(&t, 0, sizeof t);
}

/* The force and collision pass of one cycle (the replacement of the pair
 * kernel): bounds, keys, sort, nodes, masses, forces (FP64, or the mixed
 * walk), suns, collisions. */
void nbg_launch_bh(const CycleBufs &cb, DevCtl *ctl, cudaStream_t st, bool mixed)
{
    const BhTree &t = cb.t;
    const SimSegs &seg = cb.seg;
    const ll cap = cb.cap;
    const ll gmost = (ll)(cb.sms > 0 ? cb.sms : 1) * 8;
    int g = (int)((cap + BH_BLOCK - 1) / BH_BLOCK < gmost ? (cap + BH_BLOCK - 1) / BH_BLOCK : gmost);
    if (g < 1) g = 1;
    k_bh_reset<<<1, 1024, 0, st>>>(ctl, seg, t);
    k_bh_bounds<<<g, BH_BLOCK, 0, st>>>(cb.a, ctl, seg, t);
    k_bh_segs<<<1, 32, 0, st>>>(ctl, seg, t);
    k_bh_keys<<<g, BH_BLOCK, 0, st>>>(cb.a, ctl, seg, t, t.key[0], t.val[0]);
    const int nb = (int)((cap + BH_RS_TILE - 1) / BH_RS_TILE);
    /* eight passes of the key, then (several collections) two of the
     * collection index: an even count, so the sorted keys and values end in
     * buffer 0 */
    const int passes = seg.nsims > 1 ? 10 : 8;
    int in = 0;
    for (int pass = 0; pass < passes; pass++) {
        const int shift = pass < 8 ? 8 * pass : 0, simpass = pass < 8 ? -1 : pass - 8;
        k_bh_rs_hist<<<nb, BH_RS_BLOCK, 0, st>>>(ctl, seg, t.key[in], t.val[in], shift, simpass, t.hist);
        k_bh_rs_scan<<<1, 1024, 0, st>>>(ctl, t.hist);
        k_bh_rs_scatter<<<nb, BH_RS_BLOCK, 0, st>>>(ctl, seg, t.key[in], t.val[in], t.key[in ^ 1], t.val[in ^ 1],
                                                   shift, simpass, t.hist);
        in ^= 1;
    }
    const int sb = (int)(cap / BH_SCAN_TILE + 1);
    k_bh_count<<<sb, BH_SCAN_BLOCK, 0, st>>>(ctl, seg, t, t.key[0], t.base, t.blk);
    k_bh_count_top<<<1, 1024, 0, st>>>(ctl, t.blk, t.node_cap);
    k_bh_count_scan<<<sb, BH_SCAN_BLOCK, 0, st>>>(ctl, t.base, t.blk);
    k_bh_roots<<<1, 1024, 0, st>>>(ctl, seg, t, t.base);
    k_bh_nodes<<<g, BH_BLOCK, 0, st>>>(ctl, seg, t.key[0], t.base, t);
    int ng = (int)((t.node_cap + BH_BLOCK - 1) / BH_BLOCK < gmost ? (t.node_cap + BH_BLOCK - 1) / BH_BLOCK : gmost);
    if (ng < 1) ng = 1;
    for (int level = BH_LEVELS; level >= 0; level--)
        k_bh_mass<<<ng, BH_BLOCK, 0, st>>>(cb.a, ctl, t.val[0], t, level);
    if (mixed) {
        k_bh_prep_mixed<<<ng, BH_BLOCK, 0, st>>>(ctl, seg, t);
        /* CTAs per SM the walk's registers are capped for: the walk is bound
         * by the latency of its node loads, so occupancy is what counts */
        /* one wave of resident CTAs; their warps share the group queue */
        const int minb = cb.bh_shape == 1 ? 4 : cb.bh_shape == 2 ? 5 : 3;
        const int gw = g < cb.sms * minb ? g : cb.sms * minb;
        switch (cb.bh_shape) {
        case 1: k_bh_force_mixed<4><<<gw, BH_BLOCK, 0, st>>>(cb.a, ctl, seg, t.val[0], t); break;
        case 2: k_bh_force_mixed<5><<<gw, BH_BLOCK, 0, st>>>(cb.a, ctl, seg, t.val[0], t); break;
        default: k_bh_force_mixed<3><<<gw, BH_BLOCK, 0, st>>>(cb.a, ctl, seg, t.val[0], t); break;
        }
    } else {
        k_bh_force<<<g, BH_BLOCK, 0, st>>>(cb.a, ctl, seg, t.val[0], t);
    }
    k_bh_sun<<<64, BH_BLOCK, 0, st>>>(cb.a, ctl, seg);
    k_bh_collide<<<g, BH_BLOCK, 0, st>>>(cb.a, ctl, seg, t.val[0], t, cb.ev_keys, cb.ev_cap);
}

int nbg_bh_launches(const CycleBufs &cb, bool mixed)
{
    const int passes = cb.seg.nsims > 1 ? 10 : 8;
    /* reset, bounds, segs, keys; the sort; count, top, scan, roots, nodes;
     * masses; (prep,) walk; suns; collisions */
    return 4 + 3 * passes + 5 + (BH_LEVELS + 1) + (mixed ? 2 : 1) + 2;
}
