/*
 * nbg_api.cu - the C ABI of include/nbgpu.h: context, device buffers, the
 * cycle launch sequence (direct or as a replayed CUDA graph), cycle-boundary
 * edits and the overflow / retry protocol.
 *
 * A cycle is the kernel sequence
 *   begin | fragment count + scan | [mixed: reduce, pack, tile origins]
 *   | pair kernel | [mixed: partial-sum reduction] | event sort | fragment
 *   emission | resolution | integration | keep scan | compaction + adds
 *   | copy back | end
 * all on one stream, reading and updating a control block in device memory,
 * so one captured cycle can be replayed nsteps times.  A kernel that finds a
 * buffer too small sets a sticky error before anything of the cycle is
 * mutated (the force arrays of live bodies excepted, which every cycle
 * recomputes); the remaining kernels return at once, the host grows the
 * buffer and re-runs the cycle.
 */
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "nbg_internal.cuh"

/* An NVTX range over one C-ABI call (domain "nbgpu"), so a timeline tool
 * shows the host calls around the kernels; without a tool attached each
 * push and pop is a check of a null function pointer. */
namespace {
nvtxDomainHandle_t nvtx_domain()
{
    static nvtxDomainHandle_t d = nvtxDomainCreateA("nbgpu");
    return d;
}
struct NvtxRange {
    explicit NvtxRange(const char *name)
    {
        nvtxEventAttributes_t a = {};
        a.version = NVTX_VERSION;
        a.size = NVTX_EVENT_ATTRIB_STRUCT_SIZE;
        a.messageType = NVTX_MESSAGE_TYPE_ASCII;
        a.message.ascii = name;
        nvtxDomainRangePushEx(nvtx_domain(), &a);
    }
    ~NvtxRange() { nvtxDomainRangePop(nvtx_domain()); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};
} // namespace

struct nbg_ctx {
    int device = 0;
    int precision = NBG_PRECISION_FP64;
    cudaStream_t st = nullptr;     /* stream the work runs on */
    cudaStream_t own_st = nullptr; /* the context's own stream */
    DevCtl *ctl = nullptr;   /* device */
    DevCtl *ctl_h = nullptr; /* pinned host copy */
    CycleBufs cb{};
    std::string err;
    ll n_host = 0;          /* bodies in the array, as of the last sync */
    ll pending_adds = 0;    /* host adds staged for the next cycle */
    /* collection of each staged add, in the order of cb.adds: grouped by
     * collection, arrival order within one (the order k_append_adds reads) */
    std::vector<int> add_sim;
    bool timing = false;
    nbg_timing tacc{};
    std::vector<cudaEvent_t> evs;
    int use_graph = 1;
    int graph_cycles = 1; /* cycles captured in one graph */
    cudaGraphExec_t graph = nullptr;
    bool graph_valid = false;
    int graph_precision = -1;
    void *scratch = nullptr;
    size_t scratch_bytes = 0;
    ll launches_per_cycle = 0;
    ll bh_cap = 0; /* capacity the Barnes-Hut buffers were sized for */
    ll p64_split_max = NBG_P64_SPLIT_MAX_CAP; /* plain form: split pair pass up to this capacity */
    void *ring_host = nullptr; /* the caller's render ring, registered here */
    void *seg_mem = nullptr; /* SimSegs arrays */
    int seg_cap = 0;         /* sims the allocation holds */
    ll *seg_h = nullptr;     /* pinned staging of the segment offsets */
    unsigned *flags_h = nullptr; /* pinned staging for the packed flag words */
    ll flags_cap = 0;
    /* stopping a long nbg_step at a cycle boundary: nbg_cancel (any thread)
     * and the wall-clock limit of one call (NBG_OPT_STEP_DEADLINE_MS) */
    std::atomic<int> cancel{0};
    ll deadline_ms = 0;
    int ev_sort_mode = 0; /* NBG_OPT_EVENT_SORT */
    int ev_radix_auto = 0; /* automatic choice for the next call */
    bool test_fail_growth = false; /* NBG_OPT_TEST_FAIL_GROWTH: the next growth fails */
    cudaEvent_t win[2] = {nullptr, nullptr}; /* the last two launches in flight */
};

/* (Re)allocates the per-sim arrays for nsims sims and uploads the offsets of
 * the given counts (host array, nsims entries), stream-ordered through a
 * pinned staging array (whose previous copy the caller has synchronised).
 * *reshaped tells whether the arrays moved or the sim count changed: the
 * kernels of a captured graph carry both. */
static int set_segments(nbg_ctx *ctx, int nsims, const ll *counts, bool *reshaped)
{
    *reshaped = nsims != ctx->cb.seg.nsims;
    if (!ctx->seg_h) {
        cudaError_t e = cudaMallocHost((void **)&ctx->seg_h, (size_t)(NBG_MAX_SIMS + 1) * sizeof(ll));
        if (e != cudaSuccess) {
            ctx->seg_h = nullptr;
            ctx->err = std::string("segment staging: ") + cudaGetErrorString(e);
            return NBG_E_CUDA;
        }
    }
    if (nsims > ctx->seg_cap) {
        /* without the arrays the context holds no collection (nsims 0):
         * the cycle refuses to run until a load succeeds */
        cudaFree(ctx->seg_mem);
        ctx->seg_mem = nullptr;
        ctx->seg_cap = 0;
        memset(&ctx->cb.seg, 0, sizeof ctx->cb.seg);
        *reshaped = true;
        cudaError_t e = cudaMalloc(&ctx->seg_mem, NBG_SEG_BYTES(nsims));
        if (e != cudaSuccess) {
            ctx->seg_mem = nullptr;
            cudaGetLastError();
            ctx->err = std::string("segment allocation: ") + cudaGetErrorString(e);
            return NBG_E_CUDA;
        }
        ctx->seg_cap = nsims;
    }
    ctx->cb.seg = nbg_seg_carve(ctx->seg_mem, nsims);
    ll *h = ctx->seg_h;
    h[0] = 0;
    for (int s = 0; s < nsims; s++) h[s + 1] = h[s] + counts[s];
    cudaError_t e = cudaMemsetAsync(ctx->seg_mem, 0, NBG_SEG_BYTES(nsims), ctx->st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ctx->cb.seg.off, h, (size_t)(nsims + 1) * sizeof(ll), cudaMemcpyHostToDevice, ctx->st);
    if (e != cudaSuccess) {
        ctx->err = std::string("segment upload: ") + cudaGetErrorString(e);
        return NBG_E_CUDA;
    }
    return NBG_OK;
}

/* one per host thread, as errno: threads that create contexts at once do
 * not share it */
static thread_local std::string g_last_error;

/* error message of calls without a context (read by nbg_last_error(NULL)) */
const char *nbg_set_global_error(const char *msg)
{
    g_last_error = msg ? msg : "";
    return g_last_error.c_str();
}

#define CK(call)                                                                                     \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess) {                                                                     \
            set_err(ctx, std::string(#call) + ": " + cudaGetErrorString(e_));                        \
            return NBG_E_CUDA;                                                                       \
        }                                                                                            \
    } while (0)

static void set_err(nbg_ctx *ctx, const std::string &m)
{
    if (ctx)
        ctx->err = m;
    else
        g_last_error = m;
}

static int fail(nbg_ctx *ctx, int code, const std::string &m)
{
    set_err(ctx, m);
    return code;
}

/* ---- small utility kernels --------------------------------------------- */

/* the body count of a freshly loaded collection (stream-ordered, no sync) */
__global__ void k_set_loaded(DevCtl *ctl, ll n)
{
    ctl->n = n;
    ctl->n_host_adds = 0;
    ctl->sort_valid = 0;
}

__global__ void k_fill_f64(double *p, ll n, double v)
{
    for (ll k = (ll)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (ll)gridDim.x * blockDim.x) p[k] = v;
}

__global__ void k_fill_i64(ll *p, ll n, ll v)
{
    for (ll k = (ll)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (ll)gridDim.x * blockDim.x) p[k] = v;
}

static int grid_for(ll n)
{
    ll g = (n + 255) / 256;
    if (g > 4096) g = 4096;
    return (int)(g < 1 ? 1 : g);
}

/* ---- BodyArrays allocation ---------------------------------------------- */

/* the 20 FP64 field pointers of a BodyArrays, in declaration order */
static void f64_fields(BodyArrays &A, double **out[NBG_NF64])
{
    double **t[NBG_NF64] = {&A.x,  &A.y,  &A.z,  &A.vx,     &A.vy,        &A.vz,      &A.m,
                            &A.rad, &A.fx, &A.fy, &A.fz,     &A.ff,        &A.fs,      &A.rest,
                            &A.fr_rad, &A.fr_newrad, &A.fr_mass, &A.fr_cx, &A.fr_cy, &A.fr_cz};
    for (int q = 0; q < NBG_NF64; q++) out[q] = t[q];
}

static void free_arrays(BodyArrays &A)
{
    double **f[NBG_NF64];
    f64_fields(A, f);
    for (int q = 0; q < NBG_NF64; q++) cudaFree(*f[q]);
    cudaFree(A.fr_cnt);
    cudaFree(A.id);
    cudaFree(A.flags);
    memset(&A, 0, sizeof A);
}

/* every array for cap bodies; on failure none stays allocated and A is
 * zeroed */
static cudaError_t alloc_arrays(BodyArrays &A, ll cap)
{
    memset(&A, 0, sizeof A);
    size_t c = (size_t)(cap > 0 ? cap : 1);
    double **f[NBG_NF64];
    f64_fields(A, f);
    cudaError_t e = cudaSuccess;
    for (int q = 0; q < NBG_NF64 && e == cudaSuccess; q++) e = cudaMalloc((void **)f[q], c * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc((void **)&A.fr_cnt, c * sizeof(ll));
    if (e == cudaSuccess) e = cudaMalloc((void **)&A.id, c * sizeof(ll));
    if (e == cudaSuccess) e = cudaMalloc((void **)&A.flags, c * sizeof(unsigned));
    if (e != cudaSuccess) {
        cudaGetLastError();
        free_arrays(A);
    }
    return e;
}

static cudaError_t copy_arrays(BodyArrays &D, const BodyArrays &S, ll n, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    double **fd[NBG_NF64], **fs[NBG_NF64];
    f64_fields(D, fd);
    f64_fields(const_cast<BodyArrays &>(S), fs);
    for (int q = 0; q < NBG_NF64; q++) {
        cudaError_t e = cudaMemcpyAsync(*fd[q], *fs[q], (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return e;
    }
    cudaError_t e = cudaMemcpyAsync(D.fr_cnt, S.fr_cnt, (size_t)n * sizeof(ll), cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return e;
    e = cudaMemcpyAsync(D.id, S.id, (size_t)n * sizeof(ll), cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return e;
    return cudaMemcpyAsync(D.flags, S.flags, (size_t)n * sizeof(unsigned), cudaMemcpyDeviceToDevice, st);
}

static ll next_pow2(ll v)
{
    ll p = 1;
    while (p < v) p <<= 1;
    return p;
}

static void invalidate_graph(nbg_ctx *ctx)
{
    if (ctx->graph) cudaGraphExecDestroy(ctx->graph);
    ctx->graph = nullptr;
    ctx->graph_valid = false;
}

static void free_cap_buffers(CycleBufs &cb);
static int ensure_bh(nbg_ctx *ctx, ll nodes);

/* (re)allocates the body-capacity dependent buffers, keeping the first
 * `keep` bodies of the collection */
/* partial-sum doubles the mixed pair kernel of the current shape needs */
static ll part_need(const nbg_ctx *ctx, ll cap)
{
    const int itile = ctx->cb.itile > 0 ? ctx->cb.itile : NBG_MIX_ITILE;
    return NBG_PART_DOUBLES(cap, (ll)ctx->cb.slots * NBG_MIX_CHUNKS_PER_CTA, itile);
}

/* The mixed path's Morton order no longer matches the bodies: the arrays
 * were replaced, or bodies were edited or moved from the host. */
static int drop_order(nbg_ctx *ctx)
{
    static const int zero = 0;
    if (!ctx->ctl) return NBG_OK;
    CK(cudaMemcpyAsync(&ctx->ctl->sort_valid, &zero, sizeof zero, cudaMemcpyHostToDevice, ctx->st));
    return NBG_OK;
}

/* After a failed growth: the bodies, the staged adds and every buffer of
 * the capacity are released, and the context holds one empty collection
 * (it stays usable: the next load or cycle allocates again). */
static void lose_bodies(nbg_ctx *ctx)
{
    cudaGetLastError();
    cudaStreamSynchronize(ctx->st);
    free_arrays(ctx->cb.a);
    free_arrays(ctx->cb.b);
    free_cap_buffers(ctx->cb);
    ctx->cb.cap = 0;
    ctx->n_host = 0;
    ctx->pending_adds = 0;
    ctx->add_sim.clear();
    invalidate_graph(ctx);
    const ll zero = 0;
    bool reshaped = false;
    if (set_segments(ctx, 1, &zero, &reshaped) == NBG_OK) {
        k_set_loaded<<<1, 1, 0, ctx->st>>>(ctx->ctl, 0);
        cudaStreamSynchronize(ctx->st);
    }
    cudaGetLastError();
}

static int ensure_cap(nbg_ctx *ctx, ll need, ll keep)
{
    if (need <= ctx->cb.cap) return NBG_OK;
    if (need > NBG_MAX_BODIES) return fail(ctx, NBG_E_ARG, "body count exceeds 2^30");
    ll cap = ctx->cb.cap > 0 ? ctx->cb.cap : 1024;
    while (cap < need) cap *= 2;
    if (cap > NBG_MAX_BODIES) cap = NBG_MAX_BODIES;
    BodyArrays na;
    CK(alloc_arrays(na, cap)); /* nothing has changed if this fails */
    if (ctx->cb.cap > 0) {
        cudaError_t e = copy_arrays(na, ctx->cb.a, keep, ctx->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->st);
        if (e != cudaSuccess) {
            free_arrays(na);
            CK(e);
        }
        free_arrays(ctx->cb.a);
        free_arrays(ctx->cb.b);
        free_cap_buffers(ctx->cb);
    }
    /* the old buffers are gone: until every new one exists the capacity is
     * 0, and a failure leaves a context with no bodies (lose_bodies) */
    ctx->cb.a = na;
    ctx->cb.cap = 0;
    /* the test hook stands in for a device out of memory at this point */
    cudaError_t e = ctx->test_fail_growth ? cudaErrorMemoryAllocation : alloc_arrays(ctx->cb.b, cap);
    ctx->test_fail_growth = false;
#define CAP_ALLOC(ptr, bytes) \
    if (e == cudaSuccess) e = cudaMalloc((void **)&(ptr), (size_t)(bytes))
    CAP_ALLOC(ctx->cb.rend, cap * sizeof(nbg_renderable));
    const ll nblk = (cap + NBG_SCAN_TILE - 1) / NBG_SCAN_TILE;
    CAP_ALLOC(ctx->cb.blk_sum, nblk * sizeof(ll));
    CAP_ALLOC(ctx->cb.blk_off, nblk * sizeof(ll));
    CAP_ALLOC(ctx->cb.jhi, cap * sizeof(float4));
    CAP_ALLOC(ctx->cb.jlo, cap * sizeof(float4));
    /* every sim may end in a partial tile: at most cap / itile + nsims tiles */
    const ll tiles = (cap + NBG_MIX_MIN_ITILE - 1) / NBG_MIX_MIN_ITILE + NBG_MAX_SIMS + 1;
    CAP_ALLOC(ctx->cb.tile_c, tiles * sizeof(float4));
    CAP_ALLOC(ctx->cb.tile_t, tiles * sizeof(float));
    CAP_ALLOC(ctx->cb.iprep, cap * sizeof(float4));
    const ll pdoubles = part_need(ctx, cap);
    CAP_ALLOC(ctx->cb.part, pdoubles * sizeof(double));
    CAP_ALLOC(ctx->cb.perm, cap * sizeof(unsigned));
    CAP_ALLOC(ctx->cb.sval, cap * sizeof(unsigned));
    CAP_ALLOC(ctx->cb.skey[0], cap * sizeof(unsigned));
    CAP_ALLOC(ctx->cb.skey[1], cap * sizeof(unsigned));
    CAP_ALLOC(ctx->cb.shist, nbg_sort_scratch_hist(cap) * sizeof(ll));
#undef CAP_ALLOC
    if (e != cudaSuccess) {
        const std::string m = "buffers for " + std::to_string(cap) + " bodies: " + cudaGetErrorString(e) +
                              " (the context now holds no bodies)";
        lose_bodies(ctx);
        return fail(ctx, NBG_E_CUDA, m);
    }
    ctx->cb.nblk_cap = nblk;
    ctx->cb.part_doubles = pdoubles;
    ctx->cb.cap = cap;
    invalidate_graph(ctx);
    int rc = drop_order(ctx);
    if (rc != NBG_OK) return rc;
    if (ctx->cb.bh) return ensure_bh(ctx, 0);
    return NBG_OK;
}

/* the mixed kernel's partial sums: at least `need` doubles */
static int ensure_part(nbg_ctx *ctx, ll need)
{
    if (need <= ctx->cb.part_doubles) return NBG_OK;
    cudaFree(ctx->cb.part);
    ctx->cb.part = nullptr;
    ctx->cb.part_doubles = 0;
    CK(cudaMalloc((void **)&ctx->cb.part, (size_t)need * sizeof(double)));
    ctx->cb.part_doubles = need;
    invalidate_graph(ctx);
    return NBG_OK;
}

/* Barnes-Hut buffers for the current capacity and at least `nodes` nodes */
/* The plain form's split pair pass (k_p64_terms + k_p64_sum) serves one
 * collection of capacity up to p64_split_max: one thread per body would leave
 * the FP64 pipes idle below some 64 thousand bodies.  Its term buffer (3 x
 * 2048 x capacity doubles) is allocated by the first FP64 pass that wants it
 * and freed when the form, the collection count or the capacity no longer
 * do.  If it cannot be allocated, the one-thread-per-body kernel runs: the
 * two give identical results. */
static int ensure_p64(nbg_ctx *ctx)
{
    CycleBufs &cb = ctx->cb;
    const bool want = ctx->precision == NBG_PRECISION_FP64 && cb.seg.nsims == 1 && !cb.bh && cb.cap > 0 &&
                      cb.cap <= ctx->p64_split_max;
    const ll jc = cb.cap < NBG_P64_SPLIT_JC ? cb.cap : NBG_P64_SPLIT_JC;
    if (want == (cb.p64_terms != nullptr) && (!want || cb.p64_jc == jc)) return NBG_OK;
    CK(cudaStreamSynchronize(ctx->st));
    cudaFree(cb.p64_terms);
    cudaFree(cb.p64_acc);
    cb.p64_terms = cb.p64_acc = nullptr;
    cb.p64_jc = 0;
    invalidate_graph(ctx);
    if (!want) return NBG_OK;
    if (cudaMalloc((void **)&cb.p64_terms, (size_t)3 * jc * cb.cap * sizeof(double)) != cudaSuccess ||
        cudaMalloc((void **)&cb.p64_acc, (size_t)3 * cb.cap * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(cb.p64_terms);
        cb.p64_terms = nullptr;
        cb.p64_acc = nullptr;
        return NBG_OK;
    }
    cb.p64_jc = jc;
    return NBG_OK;
}

static int ensure_bh(nbg_ctx *ctx, ll nodes)
{
    BhTree &t = ctx->cb.t;
    const ll want = nodes > 2 * ctx->cb.cap + 64 ? nodes + nodes / 4 : 2 * ctx->cb.cap + 64;
    if (t.key[0] && t.node_cap >= nodes && ctx->bh_cap == ctx->cb.cap) return NBG_OK;
    if (nbg_bh_alloc(t, ctx->cb.cap, want) != NBG_OK) return fail(ctx, NBG_E_CUDA, "Barnes-Hut buffers");
    ctx->bh_cap = ctx->cb.cap;
    invalidate_graph(ctx);
    return NBG_OK;
}

static void free_cap_buffers(CycleBufs &cb)
{
    cudaFree(cb.rend);
    cudaFree(cb.blk_sum);
    cudaFree(cb.blk_off);
    cudaFree(cb.jhi);
    cudaFree(cb.jlo);
    cudaFree(cb.tile_c);
    cudaFree(cb.tile_t);
    cudaFree(cb.iprep);
    cudaFree(cb.p64_terms);
    cudaFree(cb.p64_acc);
    cb.p64_terms = cb.p64_acc = nullptr;
    cb.p64_jc = 0;
    cudaFree(cb.part);
    cudaFree(cb.perm);
    cudaFree(cb.sval);
    cudaFree(cb.skey[0]);
    cudaFree(cb.skey[1]);
    cudaFree(cb.shist);
    cb.rend = nullptr;
    cb.blk_sum = cb.blk_off = nullptr;
    cb.nblk_cap = 0;
    cb.jhi = cb.jlo = cb.tile_c = cb.iprep = nullptr;
    cb.tile_t = nullptr;
    cb.part = nullptr;
    cb.part_doubles = 0;
    cb.perm = cb.sval = cb.skey[0] = cb.skey[1] = nullptr;
    cb.shist = nullptr;
}

/* the symmetric mixed kernel's j-partial slots: at least `need` units (with
 * a quarter to spare, as collections grow by fragments and adds) */
static int ensure_jpart(nbg_ctx *ctx, ll need)
{
    if (need <= ctx->cb.jpart_units) return NBG_OK;
    const ll units = need + need / 4 + 16;
    const size_t bytes = (size_t)units * 3 * NBG_MIX_ITILE * sizeof(float);
    cudaFree(ctx->cb.jpart);
    ctx->cb.jpart = nullptr;
    ctx->cb.jpart_units = 0;
    /* the slots grow with the square of the body count (13 GB at 2^20
     * bodies): past half of the free device memory the shape is refused */
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && bytes > free_b / 2)
        return fail(ctx, NBG_E_CUDA, "the symmetric kernel's j partials would take over half of the free device memory");
    CK(cudaMalloc((void **)&ctx->cb.jpart, bytes));
    ctx->cb.jpart_units = units;
    invalidate_graph(ctx);
    return NBG_OK;
}

static int ensure_frag_cap(nbg_ctx *ctx, ll need)
{
    if (need <= ctx->cb.frag_cap) return NBG_OK;
    ll c = ctx->cb.frag_cap > 0 ? ctx->cb.frag_cap : 4096;
    while (c < need) c *= 2;
    /* no capacity until the new arrays exist: a cycle that would emit
     * fragments then stops with the overflow status */
    free_arrays(ctx->cb.frags);
    ctx->cb.frag_cap = 0;
    invalidate_graph(ctx);
    CK(alloc_arrays(ctx->cb.frags, c));
    ctx->cb.frag_cap = c;
    return NBG_OK;
}

static int ensure_adds_cap(nbg_ctx *ctx, ll need)
{
    if (need <= ctx->cb.adds_cap) return NBG_OK;
    ll c = ctx->cb.adds_cap > 0 ? ctx->cb.adds_cap : 1024;
    while (c < need) c *= 2;
    BodyArrays na;
    CK(alloc_arrays(na, c));
    if (ctx->cb.adds_cap > 0) {
        cudaError_t e = copy_arrays(na, ctx->cb.adds, ctx->pending_adds, ctx->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->st);
        if (e != cudaSuccess) {
            free_arrays(na);
            CK(e);
        }
        free_arrays(ctx->cb.adds);
    }
    ctx->cb.adds = na;
    ctx->cb.adds_cap = c;
    invalidate_graph(ctx);
    return NBG_OK;
}

static void free_events(CycleBufs &cb)
{
    cudaFree(cb.ev_keys);
    cudaFree(cb.ev_out);
    cudaFree(cb.ev_sort);
    cudaFree(cb.ev_hist);
    cudaFree(cb.inc[0]);
    cudaFree(cb.inc[1]);
    cudaFree(cb.inc_hist);
    cudaFree(cb.ev_link);
    cudaFree(cb.ev_pend);
    cudaFree(cb.ev_front);
    cudaFree(cb.ev_lo);
    cb.ev_keys = cb.ev_sort = cb.inc[0] = cb.inc[1] = nullptr;
    cb.ev_out = nullptr;
    cb.ev_hist = cb.inc_hist = cb.ev_link = cb.ev_front = cb.ev_lo = nullptr;
    cb.ev_pend = nullptr;
    cb.ev_cap = 0;
}

/* the event list of capacity c (a power of two), its sorted output and the
 * multi-block sort's ping-pong buffer and histogram */
static int alloc_events(nbg_ctx *ctx, ll c)
{
    free_events(ctx->cb);
    CK(cudaMalloc((void **)&ctx->cb.ev_keys, (size_t)c * sizeof(ull)));
    CK(cudaMalloc((void **)&ctx->cb.ev_out, (size_t)c * sizeof(nbg_event)));
    CK(cudaMalloc((void **)&ctx->cb.ev_sort, (size_t)c * sizeof(ull)));
    CK(cudaMalloc((void **)&ctx->cb.ev_hist, (size_t)nbg_sort_scratch_hist(c) * sizeof(ll)));
    /* the resolution's links (busy cycles) */
    CK(cudaMalloc((void **)&ctx->cb.inc[0], (size_t)(2 * c) * sizeof(ull)));
    CK(cudaMalloc((void **)&ctx->cb.inc[1], (size_t)(2 * c) * sizeof(ull)));
    CK(cudaMalloc((void **)&ctx->cb.inc_hist, (size_t)nbg_sort_scratch_hist(2 * c) * sizeof(ll)));
    CK(cudaMalloc((void **)&ctx->cb.ev_link, (size_t)(2 * c) * sizeof(ll)));
    CK(cudaMalloc((void **)&ctx->cb.ev_pend, (size_t)c * sizeof(int)));
    CK(cudaMalloc((void **)&ctx->cb.ev_front, (size_t)(2 * c) * sizeof(ll)));
    CK(cudaMalloc((void **)&ctx->cb.ev_lo, (size_t)(NBG_MAX_SIMS + 1) * sizeof(ll)));
    ctx->cb.ev_cap = c;
    invalidate_graph(ctx);
    return NBG_OK;
}

static int ensure_ev_cap(nbg_ctx *ctx, ll need)
{
    if (need <= ctx->cb.ev_cap) return NBG_OK;
    return alloc_events(ctx, next_pow2(need > 65536 ? need : 65536));
}

static int ensure_scratch(nbg_ctx *ctx, size_t bytes)
{
    if (bytes <= ctx->scratch_bytes) return NBG_OK;
    size_t b = 1 << 16;
    while (b < bytes) {
        if (b > ((size_t)1 << 46)) return fail(ctx, NBG_E_ARG, "scratch request too large");
        b <<= 1;
    }
    cudaFree(ctx->scratch);
    ctx->scratch = nullptr;
    ctx->scratch_bytes = 0;
    CK(cudaMalloc(&ctx->scratch, b));
    ctx->scratch_bytes = b;
    return NBG_OK;
}

static int sync_ctl(nbg_ctx *ctx)
{
    CK(cudaMemcpyAsync(ctx->ctl_h, ctx->ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    ctx->n_host = ctx->ctl_h->n;
    return NBG_OK;
}

template <typename T>
static int put_field(nbg_ctx *ctx, T *dst, const T *src, ll n)
{
    if (n <= 0 || !src) return NBG_OK;
    CK(cudaMemcpyAsync(dst, src, (size_t)n * sizeof(T), cudaMemcpyHostToDevice, ctx->st));
    return NBG_OK;
}

template <typename T>
static int get_field(nbg_ctx *ctx, T *dst, const T *src, ll n)
{
    if (n <= 0 || !dst) return NBG_OK;
    CK(cudaMemcpyAsync(dst, src, (size_t)n * sizeof(T), cudaMemcpyDeviceToHost, ctx->st));
    return NBG_OK;
}

/* Copies between device arrays and host arrays in one kernel when the host
 * side is pinned (page-locked memory is mapped into the device's address
 * space): the SMs read or write it over the host link in one launch, where
 * one DMA copy per field would pay a fixed cost each.  Pageable host memory
 * takes cudaMemcpyAsync. */
#define NBG_COPY_BATCH 32
/* entry kinds: a plain copy, or a flag word split into one of its host-side
 * fields (the nbg_soa flags byte, or the collision behaviour) */
enum { COPY_BYTES = 0, COPY_FLAGS_LOW = 1, COPY_FLAGS_BEHAVIOR = 2 };

struct CopyBatch {
    void *dst[NBG_COPY_BATCH];
    const void *src[NBG_COPY_BATCH];
    ll bytes[NBG_COPY_BATCH];
    int op[NBG_COPY_BATCH];
    int n;
};

__global__ void k_copy_batch(CopyBatch b)
{
    const int e = blockIdx.y;
    if (e >= b.n) return;
    const ll bytes = b.bytes[e];
    const ll stride = (ll)gridDim.x * blockDim.x;
    const ll t0 = (ll)blockIdx.x * blockDim.x + threadIdx.x;
    const uintptr_t d = (uintptr_t)b.dst[e], s = (uintptr_t)b.src[e];
    if (b.op[e] != COPY_BYTES) {
        const ll u = bytes >> 2;
        const unsigned *src = (const unsigned *)s;
        if (b.op[e] == COPY_FLAGS_LOW)
            for (ll k = t0; k < u; k += stride) ((unsigned *)d)[k] = src[k] & 0xffu;
        else
            for (ll k = t0; k < u; k += stride) ((int *)d)[k] = (int)NBG_BEHAVIOR(src[k]);
    } else if (((d | s) & 15) == 0) {
        const ll u = bytes >> 4;
        for (ll k = t0; k < u; k += stride) ((uint4 *)d)[k] = ((const uint4 *)s)[k];
        for (ll k = (u << 4) + t0; k < bytes; k += stride) ((char *)d)[k] = ((const char *)s)[k];
    } else if (((d | s) & 7) == 0) {
        const ll u = bytes >> 3;
        for (ll k = t0; k < u; k += stride) ((ull *)d)[k] = ((const ull *)s)[k];
        for (ll k = (u << 3) + t0; k < bytes; k += stride) ((char *)d)[k] = ((const char *)s)[k];
    } else {
        for (ll k = t0; k < bytes; k += stride) ((char *)d)[k] = ((const char *)s)[k];
    }
}

/* the device address of pinned host memory, or NULL (pageable) */
static const void *mapped_host(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

static int batch_flush(nbg_ctx *ctx, CopyBatch &b)
{
    if (b.n == 0) return NBG_OK;
    ll most = 0;
    for (int k = 0; k < b.n; k++) most = b.bytes[k] > most ? b.bytes[k] : most;
    ll blocks = (most / 16 + 255) / 256;
    if (blocks > 64) blocks = 64;
    if (blocks < 1) blocks = 1;
    k_copy_batch<<<dim3((unsigned)blocks, (unsigned)b.n), 256, 0, ctx->st>>>(b);
    CK(cudaGetLastError());
    b.n = 0;
    return NBG_OK;
}

/* host -> device (dir 0) or device -> host (dir 1) copy of n elements */
template <typename T>
static int batch_copy(nbg_ctx *ctx, CopyBatch &b, T *dst, const T *src, ll n, int dir)
{
    if (n <= 0 || !dst || !src) return NBG_OK;
    const void *host = dir == 0 ? (const void *)src : (const void *)dst;
    const void *mapped = mapped_host(host);
    if (!mapped) {
        CK(cudaMemcpyAsync(dst, src, (size_t)n * sizeof(T), dir == 0 ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost,
                           ctx->st));
        return NBG_OK;
    }
    if (b.n == NBG_COPY_BATCH) {
        int rc = batch_flush(ctx, b);
        if (rc != NBG_OK) return rc;
    }
    b.dst[b.n] = dir == 0 ? (void *)dst : const_cast<void *>(mapped);
    b.src[b.n] = dir == 0 ? mapped : (const void *)src;
    b.bytes[b.n] = n * (ll)sizeof(T);
    b.op[b.n] = COPY_BYTES;
    b.n++;
    return NBG_OK;
}

/* device flag words -> one of their fields in pinned host memory (mapped:
 * the device address of dst); op is COPY_FLAGS_LOW or COPY_FLAGS_BEHAVIOR */
static int batch_flags_out(nbg_ctx *ctx, CopyBatch &b, const void *mapped, const unsigned *src, ll n, int op)
{
    if (n <= 0) return NBG_OK;
    if (b.n == NBG_COPY_BATCH) {
        int rc = batch_flush(ctx, b);
        if (rc != NBG_OK) return rc;
    }
    b.dst[b.n] = const_cast<void *>(mapped);
    b.src[b.n] = src;
    b.bytes[b.n] = n * (ll)sizeof(unsigned);
    b.op[b.n] = op;
    b.n++;
    return NBG_OK;
}

/* pinned host staging of at least n flag words (the previous copy out of it
 * must be complete: every user syncs the stream before reuse) */
static int ensure_flags_h(nbg_ctx *ctx, ll n)
{
    if (n <= ctx->flags_cap) return NBG_OK;
    CK(cudaStreamSynchronize(ctx->st));
    if (ctx->flags_h) cudaFreeHost(ctx->flags_h);
    ctx->flags_h = nullptr;
    ctx->flags_cap = 0;
    CK(cudaMallocHost((void **)&ctx->flags_h, (size_t)n * sizeof(unsigned)));
    ctx->flags_cap = n;
    return NBG_OK;
}

/* Uploads n bodies from a host SoA into D at offset `off`; NULL optional
 * fields get NewBody defaults. */
static int upload_soa(nbg_ctx *ctx, BodyArrays &D, ll off, const nbg_soa *h, ll n)
{
    if (n <= 0) return NBG_OK;
    if (!h->x || !h->y || !h->z || !h->vx || !h->vy || !h->vz || !h->radius || !h->mass)
        return fail(ctx, NBG_E_ARG, "x, y, z, vx, vy, vz, radius and mass are required");
    int rc0 = ensure_flags_h(ctx, n);
    if (rc0 != NBG_OK) return rc0;
    CK(cudaStreamSynchronize(ctx->st)); /* the staging's last copy is done */
    unsigned *flags = ctx->flags_h;
    /* the flag words are composed into the host staging in branch-free
     * loops the compiler vectorises, with the behaviours' range taken in the
     * same pass; an out-of-range behaviour fails the call before anything
     * is copied */
    const int32_t *coll = h->collision;
    const uint32_t *hf = h->flags;
    const unsigned dflt_b = (unsigned)NBG_ELASTIC << NBG_BEHAVIOR_SHIFT;
    if (coll) {
        int32_t lo = coll[0], hi = coll[0];
        if (hf)
            for (ll k = 0; k < n; k++) {
                const int32_t c = coll[k];
                lo = c < lo ? c : lo;
                hi = c > hi ? c : hi;
                flags[k] = (hf[k] & 0xffu) | ((unsigned)c << NBG_BEHAVIOR_SHIFT);
            }
        else
            for (ll k = 0; k < n; k++) {
                const int32_t c = coll[k];
                lo = c < lo ? c : lo;
                hi = c > hi ? c : hi;
                flags[k] = NBG_F_EXISTS | ((unsigned)c << NBG_BEHAVIOR_SHIFT);
            }
        if (lo < NBG_NONE || hi > NBG_FRAGMENT) return fail(ctx, NBG_E_ARG, "collision behaviour out of range");
    } else if (hf) {
        for (ll k = 0; k < n; k++) flags[k] = (hf[k] & 0xffu) | dflt_b;
    } else {
        for (ll k = 0; k < n; k++) flags[k] = NBG_F_EXISTS | dflt_b;
    }
    int rc;
    CopyBatch cb;
    cb.n = 0;
#define PUTD(fld, src)                                                                                 \
    if ((src) != nullptr) {                                                                            \
        if ((rc = batch_copy(ctx, cb, D.fld + off, (const double *)(src), n, 0)) != NBG_OK) return rc; \
    }
#define FILLD(fld, v) k_fill_f64<<<grid_for(n), 256, 0, ctx->st>>>(D.fld + off, n, v)
    PUTD(x, h->x);
    PUTD(y, h->y);
    PUTD(z, h->z);
    PUTD(vx, h->vx);
    PUTD(vy, h->vy);
    PUTD(vz, h->vz);
    PUTD(rad, h->radius);
    PUTD(m, h->mass);
    if (h->frag_factor) { PUTD(ff, h->frag_factor); } else FILLD(ff, 0.0);
    if (h->frag_step) { PUTD(fs, h->frag_step); } else FILLD(fs, 0.0);
    if (h->r) { PUTD(rest, h->r); } else FILLD(rest, 1.0);
    if (h->fx) { PUTD(fx, h->fx); } else FILLD(fx, 0.0);
    if (h->fy) { PUTD(fy, h->fy); } else FILLD(fy, 0.0);
    if (h->fz) { PUTD(fz, h->fz); } else FILLD(fz, 0.0);
    if (h->frag_radius) { PUTD(fr_rad, h->frag_radius); } else FILLD(fr_rad, 0.0);
    if (h->frag_new_radius) { PUTD(fr_newrad, h->frag_new_radius); } else FILLD(fr_newrad, 0.0);
    if (h->frag_mass) { PUTD(fr_mass, h->frag_mass); } else FILLD(fr_mass, 0.0);
    if (h->frag_cx) { PUTD(fr_cx, h->frag_cx); } else FILLD(fr_cx, 0.0);
    if (h->frag_cy) { PUTD(fr_cy, h->frag_cy); } else FILLD(fr_cy, 0.0);
    if (h->frag_cz) { PUTD(fr_cz, h->frag_cz); } else FILLD(fr_cz, 0.0);
#undef PUTD
#undef FILLD
    if (h->frag_fragments) {
        if ((rc = batch_copy(ctx, cb, D.fr_cnt + off, (const ll *)h->frag_fragments, n, 0)) != NBG_OK) return rc;
    } else {
        k_fill_i64<<<grid_for(n), 256, 0, ctx->st>>>(D.fr_cnt + off, n, 0);
    }
    if (h->id) {
        if ((rc = batch_copy(ctx, cb, D.id + off, (const ll *)h->id, n, 0)) != NBG_OK) return rc;
    }
    if ((rc = batch_copy(ctx, cb, D.flags + off, (const unsigned *)flags, n, 0)) != NBG_OK) return rc;
    if ((rc = batch_flush(ctx, cb)) != NBG_OK) return rc;
    CK(cudaGetLastError());
    /* the caller's arrays are read before this returns (they may be reused
     * at once, cgo memory included) */
    CK(cudaStreamSynchronize(ctx->st));
    return NBG_OK;
}

/* ---- public API ---------------------------------------------------------- */

extern "C" {

const char *nbg_last_error(const nbg_ctx *ctx) { return ctx ? ctx->err.c_str() : g_last_error.c_str(); }

int nbg_create(int device, int precision, int64_t capacity, nbg_ctx **out)
{
    if (!out) return fail(nullptr, NBG_E_ARG, "out is NULL");
    *out = nullptr;
    if (precision != NBG_PRECISION_FP64 && precision != NBG_PRECISION_MIXED)
        return fail(nullptr, NBG_E_ARG, "unknown precision");
    if (capacity < 0 || capacity > NBG_MAX_BODIES) return fail(nullptr, NBG_E_ARG, "capacity out of range");
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return fail(nullptr, NBG_E_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
    if (device < 0 || device >= ndev) return fail(nullptr, NBG_E_ARG, "device index out of range");
    nbg_ctx *ctx = new nbg_ctx();
    ctx->device = device;
    ctx->precision = precision;
    int rc = NBG_OK;
    do {
        if (cudaSetDevice(device) != cudaSuccess) {
            rc = fail(ctx, NBG_E_CUDA, "cudaSetDevice failed");
            break;
        }
        if (cudaStreamCreateWithFlags(&ctx->own_st, cudaStreamNonBlocking) != cudaSuccess) {
            rc = fail(ctx, NBG_E_CUDA, "cudaStreamCreate failed");
            break;
        }
        ctx->st = ctx->own_st;
        if (cudaMalloc((void **)&ctx->ctl, sizeof(DevCtl)) != cudaSuccess ||
            cudaMallocHost((void **)&ctx->ctl_h, sizeof(DevCtl)) != cudaSuccess) {
            rc = fail(ctx, NBG_E_CUDA, "control block allocation failed");
            break;
        }
        memset(ctx->ctl_h, 0, sizeof(DevCtl));
        ctx->ctl_h->seed = 0x6e626f6479676f31ull;
        ctx->ctl_h->near_kappa = NBG_NEAR_KAPPA_DEFAULT;
        if (cudaMemcpy(ctx->ctl, ctx->ctl_h, sizeof(DevCtl), cudaMemcpyHostToDevice) != cudaSuccess) {
            rc = fail(ctx, NBG_E_CUDA, "control block upload failed");
            break;
        }
        ctx->cb.work_cap = 0;
        ctx->cb.mix_variant = 0;
        ctx->cb.itile = nbg_mix_variant_info(0).block * nbg_mix_variant_info(0).k;
        ctx->cb.slots = nbg_mixed_slots(device, 0);
        ctx->cb.sms = 0;
        cudaDeviceGetAttribute(&ctx->cb.sms, cudaDevAttrMultiProcessorCount, device);
        if (ctx->cb.sms < 1) ctx->cb.sms = 1;
        if ((rc = ensure_cap(ctx, capacity > 0 ? capacity : 1024, 0)) != NBG_OK) break;
        if ((rc = ensure_frag_cap(ctx, 4096)) != NBG_OK) break;
        if ((rc = ensure_adds_cap(ctx, 1024)) != NBG_OK) break;
        if ((rc = ensure_ev_cap(ctx, 65536)) != NBG_OK) break;
        const ll zero = 0;
        bool reshaped;
        if ((rc = set_segments(ctx, 1, &zero, &reshaped)) != NBG_OK) break;
    } while (0);
    if (rc != NBG_OK) {
        g_last_error = ctx->err;
        nbg_destroy(ctx);
        return rc;
    }
    *out = ctx;
    return NBG_OK;
}

void nbg_destroy(nbg_ctx *ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->st) cudaStreamSynchronize(ctx->st);
    invalidate_graph(ctx);
    free_arrays(ctx->cb.a);
    free_arrays(ctx->cb.b);
    free_arrays(ctx->cb.adds);
    free_arrays(ctx->cb.frags);
    free_events(ctx->cb);
    free_cap_buffers(ctx->cb);
    cudaFree(ctx->cb.jpart);
    nbg_bh_free(ctx->cb.t);
    if (ctx->ring_host) cudaHostUnregister(ctx->ring_host);
    if (ctx->flags_h) cudaFreeHost(ctx->flags_h);
    if (ctx->seg_h) cudaFreeHost(ctx->seg_h);
    cudaFree(ctx->seg_mem);
    cudaFree(ctx->scratch);
    cudaFree(ctx->ctl);
    if (ctx->ctl_h) cudaFreeHost(ctx->ctl_h);
    for (cudaEvent_t e : ctx->evs) cudaEventDestroy(e);
    for (cudaEvent_t e : ctx->win)
        if (e) cudaEventDestroy(e);
    if (ctx->own_st) cudaStreamDestroy(ctx->own_st);
    delete ctx;
}

int nbg_set_precision(nbg_ctx *ctx, int precision)
{
    if (!ctx) return NBG_E_ARG;
    if (precision != NBG_PRECISION_FP64 && precision != NBG_PRECISION_MIXED)
        return fail(ctx, NBG_E_ARG, "unknown precision");
    ctx->precision = precision;
    return NBG_OK;
}

int nbg_get_precision(nbg_ctx *ctx, int *precision)
{
    if (!ctx || !precision) return fail(ctx, NBG_E_ARG, "bad arguments");
    *precision = ctx->precision;
    return NBG_OK;
}

int nbg_set_stream(nbg_ctx *ctx, void *stream)
{
    if (!ctx) return NBG_E_ARG;
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->st));
    ctx->st = stream ? (cudaStream_t)stream : ctx->own_st;
    invalidate_graph(ctx);
    return NBG_OK;
}

static int ctl_put(nbg_ctx *ctx, size_t off, const void *v, size_t bytes)
{
    CK(cudaSetDevice(ctx->device));
    CK(cudaMemcpyAsync((char *)ctx->ctl + off, v, bytes, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return NBG_OK;
}

int nbg_set_seed(nbg_ctx *ctx, uint64_t seed)
{
    if (!ctx) return NBG_E_ARG;
    ull s = seed;
    return ctl_put(ctx, offsetof(DevCtl, seed), &s, sizeof s);
}

int nbg_set_next_id(nbg_ctx *ctx, int64_t next_id)
{
    if (!ctx) return NBG_E_ARG;
    ll v = next_id;
    return ctl_put(ctx, offsetof(DevCtl, next_id), &v, sizeof v);
}

int nbg_get_next_id(nbg_ctx *ctx, int64_t *next_id)
{
    if (!ctx || !next_id) return NBG_E_ARG;
    CK(cudaSetDevice(ctx->device));
    int rc = sync_ctl(ctx);
    if (rc != NBG_OK) return rc;
    *next_id = ctx->ctl_h->next_id;
    return NBG_OK;
}

int nbg_set_cycle(nbg_ctx *ctx, uint64_t cycle)
{
    if (!ctx) return NBG_E_ARG;
    ull c = cycle;
    return ctl_put(ctx, offsetof(DevCtl, cycle), &c, sizeof c);
}

int nbg_set_collections(nbg_ctx *ctx, int64_t nsims, const int64_t *counts, const nbg_soa *host)
{
    NvtxRange nvtx("nbg_set_collections");
    if (!ctx || nsims < 1 || nsims > NBG_MAX_SIMS || !counts) return fail(ctx, NBG_E_ARG, "bad arguments");
    ll n = 0;
    for (ll s = 0; s < nsims; s++) {
        if (counts[s] < 0) return fail(ctx, NBG_E_ARG, "negative body count");
        /* bounded one by one, so the sum cannot wrap */
        if (counts[s] > NBG_MAX_BODIES) return fail(ctx, NBG_E_ARG, "body count exceeds 2^30");
        n += counts[s];
    }
    if (n > NBG_MAX_BODIES) return fail(ctx, NBG_E_ARG, "body count exceeds 2^30");
    if (n > 0 && !host) return fail(ctx, NBG_E_ARG, "host is NULL");
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->st));
    ctx->pending_adds = 0; /* a new collection drops staged adds */
    ctx->add_sim.clear();
    int rc = ensure_cap(ctx, n, 0);
    if (rc != NBG_OK) return rc;
    if ((rc = upload_soa(ctx, ctx->cb.a, 0, host, n)) != NBG_OK) return rc;
    if (!host || !host->id) {
        /* ids default to the array index, as the reference's tests do */
        std::vector<ll> ids((size_t)(n > 0 ? n : 1));
        for (ll k = 0; k < n; k++) ids[(size_t)k] = k;
        if ((rc = put_field(ctx, ctx->cb.a.id, ids.data(), n)) != NBG_OK) return rc;
        CK(cudaStreamSynchronize(ctx->st));
    }
    bool reshaped = false;
    if ((rc = set_segments(ctx, (int)nsims, (const ll *)counts, &reshaped)) != NBG_OK) return rc;
    if (reshaped) invalidate_graph(ctx);
    k_set_loaded<<<1, 1, 0, ctx->st>>>(ctx->ctl, n);
    CK(cudaGetLastError());
    ctx->n_host = n;
    return NBG_OK;
}

int nbg_set_bodies(nbg_ctx *ctx, const nbg_soa *host, int64_t n)
{
    NvtxRange nvtx("nbg_set_bodies");
    if (!ctx || n < 0 || (n > 0 && !host)) return fail(ctx, NBG_E_ARG, "bad arguments");
    const int64_t counts[1] = {n};
    return nbg_set_collections(ctx, 1, counts, host);
}

int nbg_sim_counts(nbg_ctx *ctx, int64_t *counts, int64_t cap, int64_t *nsims)
{
    if (!ctx || cap < 0) return fail(ctx, NBG_E_ARG, "bad arguments");
    CK(cudaSetDevice(ctx->device));
    const int ns = ctx->cb.seg.nsims;
    if (nsims) *nsims = ns;
    if (counts && cap > 0) {
        std::vector<ll> off((size_t)ns + 1);
        CK(cudaMemcpyAsync(off.data(), ctx->cb.seg.off, off.size() * sizeof(ll), cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
        for (ll s = 0; s < ns && s < cap; s++) counts[s] = off[(size_t)s + 1] - off[(size_t)s];
    }
    return NBG_OK;
}

int nbg_count(nbg_ctx *ctx, int64_t *n)
{
    if (!ctx || !n) return NBG_E_ARG;
    CK(cudaSetDevice(ctx->device));
    int rc = sync_ctl(ctx);
    if (rc != NBG_OK) return rc;
    *n = ctx->ctl_h->n;
    return NBG_OK;
}

int nbg_get_state(nbg_ctx *ctx, nbg_soa *h, int64_t cap, int64_t *n_out)
{
    NvtxRange nvtx("nbg_get_state");
    if (!ctx || !h || cap < 0) return fail(ctx, NBG_E_ARG, "bad arguments");
    CK(cudaSetDevice(ctx->device));
    int rc = sync_ctl(ctx);
    if (rc != NBG_OK) return rc;
    const ll n0 = ctx->ctl_h->n;
    const ll n = n0 < cap ? n0 : cap;
    if (n_out) *n_out = n0;
    BodyArrays &A = ctx->cb.a;
    CopyBatch cb;
    cb.n = 0;
#define GETD(hf, df) \
    if ((rc = batch_copy(ctx, cb, h->hf, (const double *)A.df, n, 1)) != NBG_OK) return rc;
    GETD(x, x);
    GETD(y, y);
    GETD(z, z);
    GETD(vx, vx);
    GETD(vy, vy);
    GETD(vz, vz);
    GETD(radius, rad);
    GETD(mass, m);
    GETD(frag_factor, ff);
    GETD(frag_step, fs);
    GETD(r, rest);
    GETD(fx, fx);
    GETD(fy, fy);
    GETD(fz, fz);
    GETD(frag_radius, fr_rad);
    GETD(frag_new_radius, fr_newrad);
    GETD(frag_mass, fr_mass);
    GETD(frag_cx, fr_cx);
    GETD(frag_cy, fr_cy);
    GETD(frag_cz, fr_cz);
#undef GETD
    if ((rc = batch_copy(ctx, cb, (ll *)h->id, (const ll *)A.id, n, 1)) != NBG_OK) return rc;
    if ((rc = batch_copy(ctx, cb, (ll *)h->frag_fragments, (const ll *)A.fr_cnt, n, 1)) != NBG_OK) return rc;
    /* pinned outputs take their flag fields straight from the copy kernel;
     * otherwise the words go through pinned staging and are split here */
    const void *mf = h->flags && n > 0 ? mapped_host(h->flags) : nullptr;
    const void *mc = h->collision && n > 0 ? mapped_host(h->collision) : nullptr;
    const bool staged = (h->flags && !mf) || (h->collision && !mc);
    if (staged) {
        if ((rc = ensure_flags_h(ctx, n)) != NBG_OK) return rc;
        if ((rc = batch_copy(ctx, cb, ctx->flags_h, (const unsigned *)A.flags, n, 1)) != NBG_OK) return rc;
    } else {
        if (mf && (rc = batch_flags_out(ctx, cb, mf, A.flags, n, COPY_FLAGS_LOW)) != NBG_OK) return rc;
        if (mc && (rc = batch_flags_out(ctx, cb, mc, A.flags, n, COPY_FLAGS_BEHAVIOR)) != NBG_OK) return rc;
    }
    if ((rc = batch_flush(ctx, cb)) != NBG_OK) return rc;
    CK(cudaStreamSynchronize(ctx->st));
    const unsigned *fl = ctx->flags_h;
    for (ll k = 0; k < n && staged; k++) {
        if (h->flags) h->flags[k] = fl[k] & 0xffu;
        if (h->collision) h->collision[k] = (int32_t)NBG_BEHAVIOR(fl[k]);
    }
    return NBG_OK;
}

/* a view of the arrays starting at body `off` */
static BodyArrays arrays_at(const BodyArrays &A, ll off)
{
    BodyArrays v = A;
    double **f[NBG_NF64];
    f64_fields(v, f);
    for (int q = 0; q < NBG_NF64; q++) *f[q] += off;
    v.fr_cnt += off;
    v.id += off;
    v.flags += off;
    return v;
}

/* Uploads the staged-add count of every collection (seg.hadd) and their
 * total (the layout kernels recompute it from seg.hadd at the next cycle). */
static int put_staged_counts(nbg_ctx *ctx)
{
    const int ns = ctx->cb.seg.nsims;
    ll *h = ctx->seg_h; /* pinned; its previous copy was synchronised */
    for (int s = 0; s < ns; s++) h[s] = 0;
    for (int s : ctx->add_sim) h[s]++;
    CK(cudaMemcpyAsync(ctx->cb.seg.hadd, h, (size_t)ns * sizeof(ll), cudaMemcpyHostToDevice, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    ll pa = ctx->pending_adds;
    return ctl_put(ctx, offsetof(DevCtl, n_host_adds), &pa, sizeof pa);
}

int nbg_add_bodies_to(nbg_ctx *ctx, int64_t sim, const nbg_soa *host, int64_t n, int64_t *ids_out)
{
    if (!ctx || n < 0 || (n > 0 && !host)) return fail(ctx, NBG_E_ARG, "bad arguments");
    if (sim < 0 || sim >= ctx->cb.seg.nsims) return fail(ctx, NBG_E_ARG, "collection index out of range");
    if (n == 0) return NBG_OK;
    if (n > NBG_MAX_BODIES || ctx->n_host + ctx->pending_adds + n > NBG_MAX_BODIES)
        return fail(ctx, NBG_E_ARG, "body count exceeds 2^30");
    CK(cudaSetDevice(ctx->device));
    int rc = sync_ctl(ctx);
    if (rc != NBG_OK) return rc;
    const ll pend = ctx->pending_adds;
    if ((rc = ensure_adds_cap(ctx, pend + n)) != NBG_OK) return rc;
    if ((rc = ensure_cap(ctx, ctx->n_host + pend + n, ctx->n_host)) != NBG_OK) return rc;
    std::vector<ll> ids((size_t)n);
    ll next = ctx->ctl_h->next_id;
    for (ll k = 0; k < n; k++) {
        ll want = host->id ? host->id[k] : -1;
        ids[(size_t)k] = want >= 0 ? want : next++;
    }
    nbg_soa tmp = *host;
    tmp.id = (int64_t *)ids.data();
    if ((rc = upload_soa(ctx, ctx->cb.adds, pend, &tmp, n)) != NBG_OK) return rc;
    /* keep the staged adds grouped by collection: the new ones belong after
     * the last staged add of collections <= sim */
    ll p = 0;
    while (p < pend && ctx->add_sim[(size_t)p] <= (int)sim) p++;
    if (p < pend) {
        /* rotate [p, pend + n) so the new bodies come first: through the
         * compaction target, which is free between cycles */
        const ll m = pend + n - p;
        if ((rc = ensure_scratch(ctx, (size_t)m * sizeof(ll))) != NBG_OK) return rc;
        std::vector<ll> idx((size_t)m);
        for (ll t = 0; t < m; t++) idx[(size_t)t] = t < n ? pend + t : p + (t - n);
        CK(cudaMemcpyAsync(ctx->scratch, idx.data(), (size_t)m * sizeof(ll), cudaMemcpyHostToDevice, ctx->st));
        nbg_launch_gather(ctx->cb, ctx->cb.adds, ctx->cb.b, (const ll *)ctx->scratch, m, ctx->st);
        CK(cudaGetLastError());
        BodyArrays dst = arrays_at(ctx->cb.adds, p);
        CK(copy_arrays(dst, ctx->cb.b, m, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
    }
    ctx->add_sim.insert(ctx->add_sim.begin() + p, (size_t)n, (int)sim);
    ctx->pending_adds = pend + n;
    if ((rc = put_staged_counts(ctx)) != NBG_OK) return rc;
    if ((rc = ctl_put(ctx, offsetof(DevCtl, next_id), &next, sizeof next)) != NBG_OK) return rc;
    if (ids_out)
        for (ll k = 0; k < n; k++) ids_out[k] = ids[(size_t)k];
    return NBG_OK;
}

int nbg_add_bodies(nbg_ctx *ctx, const nbg_soa *host, int64_t n, int64_t *ids_out)
{
    if (!ctx || n < 0 || (n > 0 && !host)) return fail(ctx, NBG_E_ARG, "bad arguments");
    if (n == 0) return NBG_OK;
    if (ctx->cb.seg.nsims != 1)
        return fail(ctx, NBG_E_STATE, "several collections: name one with nbg_add_bodies_to");
    return nbg_add_bodies_to(ctx, 0, host, n, ids_out);
}

int nbg_apply_edits(nbg_ctx *ctx, const nbg_edit *edits, int64_t k, int32_t *results)
{
    return nbg_apply_edits_in(ctx, -1, edits, k, results);
}

int nbg_apply_edits_in(nbg_ctx *ctx, int64_t sim, const nbg_edit *edits, int64_t k, int32_t *results)
{
    if (!ctx || k < 0 || (k > 0 && !edits) || k > NBG_MAX_BODIES) return fail(ctx, NBG_E_ARG, "bad arguments");
    if (ctx->cb.seg.nsims < 1) return fail(ctx, NBG_E_STATE, "no collection is loaded (a segment allocation failed)");
    if (sim < -1 || sim >= ctx->cb.seg.nsims) return fail(ctx, NBG_E_ARG, "collection index out of range");
    if (k == 0) return NBG_OK;
    for (ll q = 0; q < k; q++)
        if ((edits[q].mask & NBG_M_COLLISION) && (edits[q].collision < NBG_NONE || edits[q].collision > NBG_FRAGMENT))
            return fail(ctx, NBG_E_ARG, "collision behaviour out of range");
    CK(cudaSetDevice(ctx->device));
    size_t eb = (size_t)k * sizeof(nbg_edit), rb = (size_t)k * sizeof(int);
    int rc = ensure_scratch(ctx, eb + rb + 256);
    if (rc != NBG_OK) return rc;
    nbg_edit *ed = (nbg_edit *)ctx->scratch;
    int *res = (int *)((char *)ctx->scratch + ((eb + 255) / 256) * 256);
    CK(cudaMemcpyAsync(ed, edits, eb, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemsetAsync(res, 0, rb, ctx->st));
    nbg_launch_edits(ctx->cb, ctx->ctl, (int)sim, ed, k, res, ctx->st);
    if ((rc = drop_order(ctx)) != NBG_OK) return rc;
    CK(cudaGetLastError());
    std::vector<int> hr((size_t)k);
    CK(cudaMemcpyAsync(hr.data(), res, rb, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    if (results)
        for (ll q = 0; q < k; q++) results[q] = hr[(size_t)q];
    return NBG_OK;
}

int nbg_remove_bodies(nbg_ctx *ctx, int64_t count, int64_t *removed)
{
    if (!ctx) return NBG_E_ARG;
    if (ctx->cb.seg.nsims != 1)
        return fail(ctx, NBG_E_STATE, "several collections: name one with nbg_remove_bodies_from");
    return nbg_remove_bodies_from(ctx, 0, count, removed);
}

int nbg_remove_bodies_from(nbg_ctx *ctx, int64_t sim, int64_t count, int64_t *removed)
{
    if (!ctx) return NBG_E_ARG;
    if (count == 0 || count < -1) return fail(ctx, NBG_E_ARG, "count must be -1 or positive");
    if (sim < 0 || sim >= ctx->cb.seg.nsims) return fail(ctx, NBG_E_ARG, "collection index out of range");
    CK(cudaSetDevice(ctx->device));
    int rc = ensure_scratch(ctx, sizeof(ll));
    if (rc != NBG_OK) return rc;
    nbg_launch_remove(ctx->cb, ctx->ctl, (int)sim, count, (ll *)ctx->scratch, ctx->st);
    if ((rc = drop_order(ctx)) != NBG_OK) return rc;
    CK(cudaGetLastError());
    ll r = 0;
    CK(cudaMemcpyAsync(&r, ctx->scratch, sizeof r, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    if (removed) *removed = r;
    return NBG_OK;
}

int nbg_get_body(nbg_ctx *ctx, int64_t id, nbg_soa *h, int32_t *found)
{
    return nbg_get_body_in(ctx, -1, id, h, found);
}

int nbg_get_body_in(nbg_ctx *ctx, int64_t sim, int64_t id, nbg_soa *h, int32_t *found)
{
    if (!ctx || !h || !found) return fail(ctx, NBG_E_ARG, "bad arguments");
    if (ctx->cb.seg.nsims < 1) return fail(ctx, NBG_E_STATE, "no collection is loaded (a segment allocation failed)");
    if (sim < -1 || sim >= ctx->cb.seg.nsims) return fail(ctx, NBG_E_ARG, "collection index out of range");
    CK(cudaSetDevice(ctx->device));
    int rc = ensure_scratch(ctx, sizeof(ll));
    if (rc != NBG_OK) return rc;
    ll big = (ll)1 << 62;
    CK(cudaMemcpyAsync(ctx->scratch, &big, sizeof big, cudaMemcpyHostToDevice, ctx->st));
    nbg_launch_find(ctx->cb, ctx->ctl, (int)sim, id, (ll *)ctx->scratch, ctx->st);
    CK(cudaGetLastError());
    ll idx = 0;
    CK(cudaMemcpyAsync(&idx, ctx->scratch, sizeof idx, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    if (idx >= big) {
        *found = 0;
        return NBG_OK;
    }
    *found = 1;
    BodyArrays &A = ctx->cb.a;
#define GET1(hf, df) \
    if ((rc = get_field(ctx, h->hf, (const double *)(A.df + idx), 1)) != NBG_OK) return rc;
    GET1(x, x);
    GET1(y, y);
    GET1(z, z);
    GET1(vx, vx);
    GET1(vy, vy);
    GET1(vz, vz);
    GET1(radius, rad);
    GET1(mass, m);
    GET1(frag_factor, ff);
    GET1(frag_step, fs);
    GET1(r, rest);
    GET1(fx, fx);
    GET1(fy, fy);
    GET1(fz, fz);
    GET1(frag_radius, fr_rad);
    GET1(frag_new_radius, fr_newrad);
    GET1(frag_mass, fr_mass);
    GET1(frag_cx, fr_cx);
    GET1(frag_cy, fr_cy);
    GET1(frag_cz, fr_cz);
#undef GET1
    if ((rc = get_field(ctx, (ll *)h->id, A.id + idx, 1)) != NBG_OK) return rc;
    if ((rc = get_field(ctx, (ll *)h->frag_fragments, A.fr_cnt + idx, 1)) != NBG_OK) return rc;
    unsigned f = 0;
    if ((rc = get_field(ctx, &f, A.flags + idx, 1)) != NBG_OK) return rc;
    CK(cudaStreamSynchronize(ctx->st));
    if (h->flags) h->flags[0] = f & 0xffu;
    if (h->collision) h->collision[0] = (int32_t)NBG_BEHAVIOR(f);
    return NBG_OK;
}

/* ---- snapshots -------------------------------------------------------------
 * Everything a later cycle reads, so a run resumed from a snapshot repeats
 * the uninterrupted run bit for bit:
 *   header (NBG_SNAP_HEADER_BYTES): counters, options and the layout below;
 *   the body count of each collection, then its staged host adds;
 *   the body arrays: the 20 FP64 fields of BodyArrays in declaration order,
 *     fragment counts and ids (int64), flag words (uint32: NBG_F_* bits and
 *     the behaviour), each field n values, padded to 8 bytes;
 *   the staged host adds in the same layout (grouped by collection, arrival
 *     order within one);
 *   mixed form: the Morton order of the bodies (uint32 per body) when one is
 *     current, so the FP32 pair sums group the same bodies.
 * Values are stored in the machine's byte order (little-endian on x86-64 and
 * aarch64); the header records the field count and per-body bytes. */
static int select_variant(nbg_ctx *ctx, int v);

#define NBG_SNAP_HEADER_BYTES 256
#define NBG_SNAP_VERSION 1
static const char NBG_SNAP_MAGIC[8] = {'N', 'B', 'G', 'S', 'N', 'A', 'P', '1'};

struct SnapHeader {
    char magic[8];
    uint32_t version, header_bytes;
    int32_t precision, nsims;
    int64_t n, pending_adds, next_id;
    uint64_t cycle, seed, sort_cycle;
    int32_t sort_valid, sort_interval;
    float near_kappa;
    int32_t mix_variant, barnes_hut, has_order;
    int32_t f64_fields, body_bytes;
    int64_t total_bytes;
};
static_assert(sizeof(SnapHeader) <= NBG_SNAP_HEADER_BYTES, "snapshot header too large");

static ll align8(ll v) { return (v + 7) & ~(ll)7; }

/* bytes of one block of body arrays holding n bodies */
static ll snap_arrays_bytes(ll n) { return (NBG_NF64 + 2) * align8(n * 8) + align8(n * 4); }

struct SnapLayout {
    ll counts, hadd, bodies, adds, order, total;
};

static SnapLayout snap_layout(ll nsims, ll n, ll pending, bool order)
{
    SnapLayout L;
    L.counts = NBG_SNAP_HEADER_BYTES;
    L.hadd = L.counts + nsims * 8;
    L.bodies = L.hadd + nsims * 8;
    L.adds = L.bodies + snap_arrays_bytes(n);
    L.order = L.adds + snap_arrays_bytes(pending);
    L.total = L.order + (order ? align8(n * 4) : 0);
    return L;
}

/* Copies n bodies between device arrays A and the block at host address
 * blk (to_host: device to host), stream-ordered; the caller synchronises. */
static int snap_copy_arrays(nbg_ctx *ctx, BodyArrays &A, char *blk, ll n, bool to_host)
{
    if (n <= 0) return NBG_OK;
    double **f[NBG_NF64];
    f64_fields(A, f);
    const cudaMemcpyKind kind = to_host ? cudaMemcpyDeviceToHost : cudaMemcpyHostToDevice;
    ll o = 0;
    for (int q = 0; q < NBG_NF64 + 3; q++) {
        void *dev = q < NBG_NF64 ? (void *)*f[q] : q == NBG_NF64 ? (void *)A.fr_cnt : q == NBG_NF64 + 1
                                                                    ? (void *)A.id : (void *)A.flags;
        const ll bytes = n * (q < NBG_NF64 + 2 ? 8 : 4);
        if (to_host)
            CK(cudaMemcpyAsync(blk + o, dev, (size_t)bytes, kind, ctx->st));
        else
            CK(cudaMemcpyAsync(dev, blk + o, (size_t)bytes, kind, ctx->st));
        o += align8(bytes);
    }
    return NBG_OK;
}

int nbg_save_state(nbg_ctx *ctx, void *buf, int64_t cap, int64_t *size)
{
    NvtxRange nvtx("nbg_save_state");
    if (!ctx || !size || cap < 0) return fail(ctx, NBG_E_ARG, "bad arguments");
    CK(cudaSetDevice(ctx->device));
    int rc = sync_ctl(ctx);
    if (rc != NBG_OK) return rc;
    const DevCtl *h = ctx->ctl_h;
    const ll n = h->n, pend = ctx->pending_adds;
    const int ns = ctx->cb.seg.nsims;
    const bool order = ctx->precision == NBG_PRECISION_MIXED && !ctx->cb.bh && h->sort_valid;
    const SnapLayout L = snap_layout(ns, n, pend, order);
    *size = L.total;
    if (!buf) return NBG_OK;
    if (cap < L.total) {
        char m[128];
        snprintf(m, sizeof m, "snapshot buffer too small: %lld bytes needed", (long long)L.total);
        return fail(ctx, NBG_E_OVERFLOW, m);
    }
    char *out = (char *)buf;
    memset(out, 0, NBG_SNAP_HEADER_BYTES);
    SnapHeader H;
    memset(&H, 0, sizeof H);
    memcpy(H.magic, NBG_SNAP_MAGIC, 8);
    H.version = NBG_SNAP_VERSION;
    H.header_bytes = NBG_SNAP_HEADER_BYTES;
    H.precision = ctx->precision;
    H.nsims = ns;
    H.n = n;
    H.pending_adds = pend;
    H.next_id = h->next_id;
    H.cycle = h->cycle;
    H.seed = h->seed;
    H.sort_cycle = h->sort_cycle;
    H.sort_valid = order ? 1 : 0;
    H.sort_interval = h->sort_interval;
    H.near_kappa = h->near_kappa;
    H.mix_variant = ctx->cb.mix_variant;
    H.barnes_hut = ctx->cb.bh;
    H.has_order = order ? 1 : 0;
    H.f64_fields = NBG_NF64;
    H.body_bytes = NBG_NF64 * 8 + 8 + 8 + 4;
    H.total_bytes = L.total;
    memcpy(out, &H, sizeof H);
    std::vector<ll> off((size_t)ns + 1);
    CK(cudaMemcpyAsync(off.data(), ctx->cb.seg.off, off.size() * sizeof(ll), cudaMemcpyDeviceToHost, ctx->st));
    if ((rc = snap_copy_arrays(ctx, ctx->cb.a, out + L.bodies, n, true)) != NBG_OK) return rc;
    if ((rc = snap_copy_arrays(ctx, ctx->cb.adds, out + L.adds, pend, true)) != NBG_OK) return rc;
    if (order) CK(cudaMemcpyAsync(out + L.order, ctx->cb.perm, (size_t)n * 4, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    ll *counts = (ll *)(out + L.counts), *hadd = (ll *)(out + L.hadd);
    for (int s = 0; s < ns; s++) {
        counts[s] = off[(size_t)s + 1] - off[(size_t)s];
        hadd[s] = 0;
    }
    for (int s : ctx->add_sim) hadd[s]++;
    return NBG_OK;
}

int nbg_load_state(nbg_ctx *ctx, const void *buf, int64_t size)
{
    NvtxRange nvtx("nbg_load_state");
    if (!ctx || !buf || size < NBG_SNAP_HEADER_BYTES) return fail(ctx, NBG_E_ARG, "not a snapshot: too short");
    const char *in = (const char *)buf;
    SnapHeader H;
    memcpy(&H, in, sizeof H);
    if (memcmp(H.magic, NBG_SNAP_MAGIC, 8) != 0) return fail(ctx, NBG_E_ARG, "not a snapshot: bad magic");
    if (H.version != NBG_SNAP_VERSION || H.header_bytes != NBG_SNAP_HEADER_BYTES || H.f64_fields != NBG_NF64 ||
        H.body_bytes != NBG_NF64 * 8 + 8 + 8 + 4)
        return fail(ctx, NBG_E_ARG, "snapshot of another format version");
    if (H.nsims < 1 || H.nsims > NBG_MAX_SIMS || H.n < 0 || H.n > NBG_MAX_BODIES || H.pending_adds < 0 ||
        H.pending_adds > NBG_MAX_BODIES ||
        (H.precision != NBG_PRECISION_FP64 && H.precision != NBG_PRECISION_MIXED) || H.mix_variant < 0 ||
        H.mix_variant >= NBG_MIX_VARIANTS || H.sort_interval < 0 || H.sort_interval > 1000)
        return fail(ctx, NBG_E_ARG, "snapshot header out of range");
    const SnapLayout L = snap_layout(H.nsims, H.n, H.pending_adds, H.has_order != 0);
    if (L.total != H.total_bytes || L.total > size) return fail(ctx, NBG_E_ARG, "snapshot truncated");
    const ll *counts = (const ll *)(in + L.counts), *hadd = (const ll *)(in + L.hadd);
    ll nsum = 0, asum = 0;
    for (int s = 0; s < H.nsims; s++) {
        if (counts[s] < 0 || hadd[s] < 0 || counts[s] > NBG_MAX_BODIES || hadd[s] > NBG_MAX_BODIES)
            return fail(ctx, NBG_E_ARG, "snapshot counts out of range");
        nsum += counts[s];
        asum += hadd[s];
    }
    if (nsum != H.n || asum != H.pending_adds) return fail(ctx, NBG_E_ARG, "snapshot counts do not add up");
    if (H.has_order) {
        /* the kernels index the bodies through the order: it must map each
         * collection's positions onto that collection's bodies, once each */
        const unsigned *ord = (const unsigned *)(in + L.order);
        std::vector<unsigned char> seen((size_t)H.n, 0);
        ll o = 0;
        for (int s = 0; s < H.nsims; s++) {
            for (ll p = o; p < o + counts[s]; p++) {
                const ll k = (ll)ord[p];
                if (k < o || k >= o + counts[s] || seen[(size_t)k])
                    return fail(ctx, NBG_E_ARG, "snapshot order is not a permutation of each collection");
                seen[(size_t)k] = 1;
            }
            o += counts[s];
        }
    }
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->st));
    int rc;
    /* the form and kernel shape the run used */
    ctx->precision = H.precision;
    if ((rc = nbg_set_option(ctx, NBG_OPT_BARNES_HUT, H.barnes_hut)) != NBG_OK) return rc;
    if (H.mix_variant != ctx->cb.mix_variant && (rc = select_variant(ctx, H.mix_variant)) != NBG_OK) return rc;
    ctx->pending_adds = 0;
    ctx->add_sim.clear();
    if ((rc = ensure_cap(ctx, H.n + H.pending_adds + 1, 0)) != NBG_OK) return rc;
    char *src = const_cast<char *>(in);
    if ((rc = snap_copy_arrays(ctx, ctx->cb.a, src + L.bodies, H.n, false)) != NBG_OK) return rc;
    bool reshaped = false;
    if ((rc = set_segments(ctx, H.nsims, counts, &reshaped)) != NBG_OK) return rc;
    if (reshaped) invalidate_graph(ctx);
    k_set_loaded<<<1, 1, 0, ctx->st>>>(ctx->ctl, H.n);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(ctx->st)); /* the segment staging is free again */
    ctx->n_host = H.n;
    if (H.pending_adds > 0) {
        if ((rc = ensure_adds_cap(ctx, H.pending_adds)) != NBG_OK) return rc;
        if ((rc = snap_copy_arrays(ctx, ctx->cb.adds, src + L.adds, H.pending_adds, false)) != NBG_OK) return rc;
        for (int s = 0; s < H.nsims; s++) ctx->add_sim.insert(ctx->add_sim.end(), (size_t)hadd[s], s);
        ctx->pending_adds = H.pending_adds;
    }
    if ((rc = put_staged_counts(ctx)) != NBG_OK) return rc;
    if (H.has_order) CK(cudaMemcpyAsync(ctx->cb.perm, in + L.order, (size_t)H.n * 4, cudaMemcpyHostToDevice, ctx->st));
    /* counters and options, after k_set_loaded cleared the order */
    DevCtl *h = ctx->ctl_h;
    if ((rc = sync_ctl(ctx)) != NBG_OK) return rc;
    h->next_id = H.next_id;
    h->cycle = H.cycle;
    h->seed = H.seed;
    h->sort_valid = H.has_order ? 1 : 0;
    h->sort_cycle = H.sort_cycle;
    h->sort_interval = H.sort_interval;
    h->near_kappa = H.near_kappa;
    h->rend_n = 0;
    h->last_ev_n = 0;
    CK(cudaMemcpyAsync(ctx->ctl, h, sizeof(DevCtl), cudaMemcpyHostToDevice, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return NBG_OK;
}

/* ---- the cycle ------------------------------------------------------------ */

static cudaEvent_t get_event(nbg_ctx *ctx, size_t k)
{
    while (ctx->evs.size() <= k) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        ctx->evs.push_back(e);
    }
    return ctx->evs[k];
}

/* Launches one cycle.  With ev_base >= 0, events ev_base..ev_base+2 bracket
 * (cycle start, pair kernel start, pair kernel end, cycle end). */
static void launch_cycle(nbg_ctx *ctx, int precision, long ev_base)
{
    const CycleBufs &cb = ctx->cb;
    cudaStream_t st = ctx->st;
    if (ev_base >= 0) cudaEventRecord(get_event(ctx, (size_t)ev_base), st);
    nbg_launch_begin(cb, ctx->ctl, st);
    nbg_launch_frag_count(cb, ctx->ctl, st);
    if (cb.bh) {
        if (ev_base >= 0) cudaEventRecord(get_event(ctx, (size_t)ev_base + 1), st);
        nbg_launch_bh(cb, ctx->ctl, st, precision == NBG_PRECISION_MIXED);
        if (ev_base >= 0) cudaEventRecord(get_event(ctx, (size_t)ev_base + 2), st);
    } else if (precision == NBG_PRECISION_MIXED) {
        nbg_launch_mixed_prep(cb, ctx->ctl, st);
        if (ev_base >= 0) cudaEventRecord(get_event(ctx, (size_t)ev_base + 1), st);
        nbg_launch_mixed_pair(cb, ctx->ctl, st);
        if (ev_base >= 0) cudaEventRecord(get_event(ctx, (size_t)ev_base + 2), st);
        nbg_launch_mixed_out(cb, ctx->ctl, st);
    } else {
        if (ev_base >= 0) cudaEventRecord(get_event(ctx, (size_t)ev_base + 1), st);
        nbg_launch_pair_fp64(cb, ctx->ctl, st);
        if (ev_base >= 0) cudaEventRecord(get_event(ctx, (size_t)ev_base + 2), st);
    }
    /* the mixed direct path keeps its Morton order through compaction */
    nbg_launch_after_pair(cb, ctx->ctl, st, !cb.bh && precision == NBG_PRECISION_MIXED);
    if (ev_base >= 0) cudaEventRecord(get_event(ctx, (size_t)ev_base + 3), st);
    /* begin, fragment count + scan, 10 after the pair kernel, and the pair
     * kernel; mixed adds reduce, the sort decision and 21 sort launches
     * (which return at once in cycles that keep the order), pack, tile
     * origins, i-body set-up, the output and 4 that carry the order through
     * compaction; Barnes-Hut replaces the pair kernel (nbg_bh_launches) */
    ctx->launches_per_cycle = (cb.ev_radix ? nbg_event_radix_launches(cb) : 0) +
                              (cb.bh ? 13 + nbg_bh_launches(cb, precision == NBG_PRECISION_MIXED)
                                     : precision == NBG_PRECISION_MIXED ? 45 : 13 + nbg_pair_fp64_launches(cb)) +
                              (cb.ring_head ? 1 : 0);
}

/* One CUDA graph of ctx->graph_cycles consecutive cycles. */
static int build_graph(nbg_ctx *ctx)
{
    if (ctx->graph_valid && ctx->graph_precision == ctx->precision) return NBG_OK;
    invalidate_graph(ctx);
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(ctx->st, cudaStreamCaptureModeThreadLocal));
    for (int c = 0; c < ctx->graph_cycles; c++) launch_cycle(ctx, ctx->precision, -1);
    CK(cudaStreamEndCapture(ctx->st, &g));
    cudaError_t e = cudaGraphInstantiate(&ctx->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(ctx, NBG_E_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    ctx->graph_valid = true;
    ctx->graph_precision = ctx->precision;
    return NBG_OK;
}

/* Launches of one nbg_step call, at most two in flight: before each launch
 * after the second, the host waits for the launch two back to finish and
 * then honours a cancel request or the call's deadline, so a long call
 * stops within about two launches of cycles, at a cycle boundary. */
struct LaunchWindow {
    nbg_ctx *ctx;
    std::chrono::steady_clock::time_point deadline;
    bool has_deadline;
    int issued = 0;
    int stop = NBG_OK; /* NBG_E_CANCELLED or NBG_E_TIMEOUT once asked to stop */

    /* true if the next launch may go */
    bool admit(int *err)
    {
        *err = NBG_OK;
        if (stop != NBG_OK) return false;
        if (issued >= 2) {
            cudaError_t e = cudaEventSynchronize(ctx->win[issued % 2]);
            if (e != cudaSuccess) {
                *err = fail(ctx, NBG_E_CUDA, std::string("cudaEventSynchronize: ") + cudaGetErrorString(e));
                return false;
            }
        }
        if (ctx->cancel.exchange(0) != 0)
            stop = NBG_E_CANCELLED;
        else if (has_deadline && std::chrono::steady_clock::now() >= deadline)
            stop = NBG_E_TIMEOUT;
        return stop == NBG_OK;
    }
    /* after a launch */
    int issued_one()
    {
        cudaError_t e = cudaEventRecord(ctx->win[issued % 2], ctx->st);
        issued++;
        if (e != cudaSuccess) return fail(ctx, NBG_E_CUDA, std::string("cudaEventRecord: ") + cudaGetErrorString(e));
        return NBG_OK;
    }
};

int nbg_step(nbg_ctx *ctx, double dt, double R, int nsteps, nbg_step_info *info)
{
    NvtxRange nvtx("nbg_step");
    if (!ctx || nsteps < 0) return fail(ctx, NBG_E_ARG, "bad arguments");
    if (ctx->cb.seg.nsims < 1) return fail(ctx, NBG_E_STATE, "no collection is loaded (a segment allocation failed)");
    CK(cudaSetDevice(ctx->device));
    /* dt, R and the per-call accumulators */
    {
        DevCtl *h = ctx->ctl_h;
        int rc = sync_ctl(ctx);
        if (rc != NBG_OK) return rc;
        h->dt = dt;
        h->R = R;
        h->error = 0;
        h->error_what = 0;
        h->error_need = 0;
        h->acc_steps = h->acc_interactions = h->acc_events = h->acc_frags = h->acc_removed = h->acc_nan = 0;
        h->acc_bh_terms = 0;
        h->acc_ev_max = 0;
        CK(cudaMemcpyAsync(ctx->ctl, h, sizeof(DevCtl), cudaMemcpyHostToDevice, ctx->st));
    }
    ctx->tacc = nbg_timing{};
    {
        /* whether the cycles launch the multi-block event sort: forced by the
         * option, else as the last call's busiest cycle asked */
        const int want = ctx->ev_sort_mode == 1 ? 1 : ctx->ev_sort_mode == 2 ? 0 : ctx->ev_radix_auto;
        if (want != ctx->cb.ev_radix) {
            ctx->cb.ev_radix = want;
            invalidate_graph(ctx);
        }
    }
    for (cudaEvent_t &e : ctx->win)
        if (!e) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    LaunchWindow win{ctx, std::chrono::steady_clock::now() + std::chrono::milliseconds(ctx->deadline_ms),
                     ctx->deadline_ms > 0};
    int done = 0;
    int retries = 0;
    while (done < nsteps) {
        int rc = ensure_cap(ctx, ctx->n_host + ctx->pending_adds + 1, ctx->n_host);
        if (rc != NBG_OK) return rc;
        /* the event buffers exist (an earlier failed reallocation leaves
         * none, and the cycle's kernels write the per-sim event ranges) */
        if ((rc = ensure_ev_cap(ctx, 1)) != NBG_OK) return rc;
        if (ctx->cb.bh && (rc = ensure_bh(ctx, 0)) != NBG_OK) return rc; /* likewise the octree's */
        if ((rc = ensure_p64(ctx)) != NBG_OK) return rc;
        const int todo = nsteps - done;
        if (ctx->timing || !ctx->use_graph || todo < ctx->graph_cycles || todo == 1) {
            for (int s = 0; s < todo; s++) {
                if (!win.admit(&rc)) break;
                launch_cycle(ctx, ctx->precision, ctx->timing ? 4L * s : -1L);
                if ((rc = win.issued_one()) != NBG_OK) break;
            }
        } else {
            /* whole graphs of graph_cycles cycles, the remainder directly */
            if ((rc = build_graph(ctx)) != NBG_OK) return rc;
            const int graphs = todo / ctx->graph_cycles;
            for (int s = 0; s < graphs && rc == NBG_OK; s++) {
                if (!win.admit(&rc)) break;
                CK(cudaGraphLaunch(ctx->graph, ctx->st));
                rc = win.issued_one();
            }
            for (int s = graphs * ctx->graph_cycles; s < todo && rc == NBG_OK && win.stop == NBG_OK; s++) {
                if (!win.admit(&rc)) break;
                launch_cycle(ctx, ctx->precision, -1L);
                rc = win.issued_one();
            }
        }
        if (rc != NBG_OK) return rc;
        CK(cudaGetLastError());
        if ((rc = sync_ctl(ctx)) != NBG_OK) return rc;
        DevCtl *h = ctx->ctl_h;
        const int now = (int)h->acc_steps;
        if (ctx->timing) {
            for (int s = 0; s < now - done; s++) {
                float a = 0, b = 0, c = 0;
                cudaEventElapsedTime(&a, get_event(ctx, 4 * s), get_event(ctx, 4 * s + 1));
                cudaEventElapsedTime(&b, get_event(ctx, 4 * s + 1), get_event(ctx, 4 * s + 2));
                cudaEventElapsedTime(&c, get_event(ctx, 4 * s + 2), get_event(ctx, 4 * s + 3));
                ctx->tacc.pair_ms += b;
                ctx->tacc.other_ms += a + c;
                ctx->tacc.pair_launches += 1;
            }
        }
        ctx->tacc.kernel_launches += (ll)(now - done) * ctx->launches_per_cycle;
        if (now > done) {
            /* consumed by the first cycle */
            ctx->pending_adds = 0;
            ctx->add_sim.clear();
        }
        done = now;
        if (h->error == 0 && win.stop != NBG_OK) break; /* stopped at a cycle boundary */
        if (h->error == 0) continue;
        if (h->error != NBG_E_OVERFLOW || ++retries > 8) {
            char m[160];
            snprintf(m, sizeof m, "cycle %d failed: status %d (what %d, need %lld)", done, h->error, h->error_what,
                     (long long)h->error_need);
            /* the failed cycle may have claimed a sort it never finished */
            drop_order(ctx);
            return fail(ctx, h->error, m);
        }
        /* grow the short buffer and re-run the interrupted cycle */
        if (h->error_what == 1)
            rc = ensure_cap(ctx, h->error_need, ctx->n_host);
        else if (h->error_what == 2)
            rc = ensure_ev_cap(ctx, h->error_need);
        else if (h->error_what == 4)
            rc = ensure_part(ctx, h->error_need);
        else if (h->error_what == 5)
            rc = ensure_bh(ctx, h->error_need);
        else if (h->error_what == 6)
            rc = ensure_jpart(ctx, h->error_need);
        else
            rc = ensure_frag_cap(ctx, h->error_need);
        if (rc != NBG_OK) return rc;
        h->error = 0;
        int z = 0;
        CK(cudaMemcpyAsync(&ctx->ctl->error, &z, sizeof z, cudaMemcpyHostToDevice, ctx->st));
        /* the failed cycle may have claimed a sort it never finished - unless
         * k_begin stopped it (partial-sum or j-partial slots) before any
         * other kernel ran: then the order stands, as it would have without
         * the retry (a resumed snapshot's cycles repeat the run's) */
        if (h->error_what != 4 && h->error_what != 6 && (rc = drop_order(ctx)) != NBG_OK) return rc;
    }
    {
        /* a cycle with more events than one block sorts in shared memory
         * makes the next calls launch the multi-block sort; they drop it once
         * a call stays well below that */
        const ll evmax = ctx->ctl_h->acc_ev_max;
        if (evmax > NBG_EV_BLOCK_SORT)
            ctx->ev_radix_auto = 1;
        else if (evmax <= NBG_EV_BLOCK_SORT / 4 && done > 0)
            ctx->ev_radix_auto = 0;
    }
    if (info) {
        DevCtl *h = ctx->ctl_h;
        info->steps_done = h->acc_steps;
        info->n_bodies = h->n;
        info->interactions = h->acc_interactions;
        info->events = h->acc_events;
        info->fragments_emitted = h->acc_frags;
        info->removed = h->acc_removed;
        info->nan_removed = h->acc_nan;
        info->next_id = h->next_id;
        info->bh_terms = h->acc_bh_terms;
    }
    if (win.stop != NBG_OK && done < nsteps) {
        char m[160];
        snprintf(m, sizeof m, "%s after %d of %d cycles; the state is that after those cycles",
                 win.stop == NBG_E_CANCELLED ? "cancelled" : "deadline reached", done, nsteps);
        return fail(ctx, win.stop, m);
    }
    return NBG_OK;
}

int nbg_cancel(nbg_ctx *ctx)
{
    if (!ctx) return NBG_E_ARG;
    ctx->cancel.store(1);
    return NBG_OK;
}

int nbg_force_pass(nbg_ctx *ctx)
{
    NvtxRange nvtx("nbg_force_pass");
    if (!ctx) return NBG_E_ARG;
    if (ctx->cb.seg.nsims < 1) return fail(ctx, NBG_E_STATE, "no collection is loaded (a segment allocation failed)");
    CK(cudaSetDevice(ctx->device));
    {
        int rc = ensure_p64(ctx);
        if (rc != NBG_OK) return rc;
        /* the octree's buffers exist (a failed allocation leaves none) */
        if (ctx->cb.bh && (rc = ensure_bh(ctx, 0)) != NBG_OK) return rc;
    }
    for (int attempt = 0;; attempt++) {
        int z = 0;
        CK(cudaMemcpyAsync(&ctx->ctl->error, &z, sizeof z, cudaMemcpyHostToDevice, ctx->st));
        /* a retry follows a buffer k_begin found short (partial-sum or
         * j-partial slots) or the octree's (Barnes-Hut, which keeps no Morton
         * order): no kernel after k_begin ran, so the order stands */
        nbg_launch_begin(ctx->cb, ctx->ctl, ctx->st);
        if (ctx->cb.bh) {
            nbg_launch_bh(ctx->cb, ctx->ctl, ctx->st, ctx->precision == NBG_PRECISION_MIXED);
        } else if (ctx->precision == NBG_PRECISION_MIXED) {
            nbg_launch_mixed_prep(ctx->cb, ctx->ctl, ctx->st);
            nbg_launch_mixed_pair(ctx->cb, ctx->ctl, ctx->st);
            nbg_launch_mixed_out(ctx->cb, ctx->ctl, ctx->st);
        } else {
            nbg_launch_pair_fp64(ctx->cb, ctx->ctl, ctx->st);
        }
        CK(cudaGetLastError());
        int rc = sync_ctl(ctx);
        if (rc != NBG_OK) return rc;
        const DevCtl *h = ctx->ctl_h;
        if (h->error == NBG_E_OVERFLOW && attempt < 4 &&
            (h->error_what == 4 || h->error_what == 5 || h->error_what == 6)) {
            /* a buffer of the force pass was short: grow it, run again */
            rc = h->error_what == 4 ? ensure_part(ctx, h->error_need)
                 : h->error_what == 5 ? ensure_bh(ctx, h->error_need)
                                      : ensure_jpart(ctx, h->error_need);
            if (rc != NBG_OK) return rc;
            continue;
        }
        if (h->error) return fail(ctx, h->error, "force pass failed");
        return NBG_OK;
    }
}

static int select_variant(nbg_ctx *ctx, int v)
{
    if (v < 0 || v >= NBG_MIX_VARIANTS) return fail(ctx, NBG_E_ARG, "unknown kernel shape");
    const MixVariantInfo vi = nbg_mix_variant_info(v);
    ctx->cb.mix_variant = v;
    ctx->cb.itile = vi.block * vi.k;
    ctx->cb.slots = nbg_mixed_slots(ctx->device, v);
    invalidate_graph(ctx);
    return ensure_part(ctx, part_need(ctx, ctx->cb.cap));
}

/* Device time of the mixed pair kernel in one force pass of the current
 * collection (CUDA events around the kernel on the context's stream). */
static int time_mixed_pair(nbg_ctx *ctx, float *ms)
{
    cudaEvent_t e0 = get_event(ctx, 0), e1 = get_event(ctx, 1);
    int z = 0;
    CK(cudaMemcpyAsync(&ctx->ctl->error, &z, sizeof z, cudaMemcpyHostToDevice, ctx->st));
    nbg_launch_begin(ctx->cb, ctx->ctl, ctx->st);
    nbg_launch_mixed_prep(ctx->cb, ctx->ctl, ctx->st);
    CK(cudaEventRecord(e0, ctx->st));
    nbg_launch_mixed_pair(ctx->cb, ctx->ctl, ctx->st);
    CK(cudaEventRecord(e1, ctx->st));
    nbg_launch_mixed_out(ctx->cb, ctx->ctl, ctx->st);
    CK(cudaGetLastError());
    CK(cudaEventSynchronize(e1));
    CK(cudaEventElapsedTime(ms, e0, e1));
    int rc = sync_ctl(ctx);
    if (rc != NBG_OK) return rc;
    if (ctx->ctl_h->error) return fail(ctx, ctx->ctl_h->error, "autotune: the timed force pass failed");
    return NBG_OK;
}

static std::string tune_key(nbg_ctx *ctx, ll n)
{
    cudaDeviceProp p;
    cudaGetDeviceProperties(&p, ctx->device);
    int bucket = 0;
    while (((ll)1 << (bucket + 1)) <= n) bucket++;
    int sb = 0;
    while ((1 << (sb + 1)) <= ctx->cb.seg.nsims) sb++;
    std::string name(p.name);
    for (char &c : name)
        if (c == ' ') c = '_';
    char buf[256];
    snprintf(buf, sizeof buf, "%s|sm%d|n2^%d|sims2^%d", name.c_str(), p.multiProcessorCount, bucket, sb);
    return buf;
}

int nbg_autotune(nbg_ctx *ctx, const char *cache_path, int *variant, double *best_ms)
{
    NvtxRange nvtx("nbg_autotune");
    if (!ctx) return NBG_E_ARG;
    if (ctx->cb.seg.nsims < 1) return fail(ctx, NBG_E_STATE, "no collection is loaded (a segment allocation failed)");
    CK(cudaSetDevice(ctx->device));
    int rc = sync_ctl(ctx);
    if (rc != NBG_OK) return rc;
    const ll n = ctx->ctl_h->n;
    if (n <= 0) return fail(ctx, NBG_E_STATE, "autotune needs a loaded collection");
    const std::string key = tune_key(ctx, n);
    int best = -1;
    double best_t = 0;
    if (cache_path) {
        if (FILE *f = fopen(cache_path, "r")) {
            char k[256];
            int v;
            double t;
            while (fscanf(f, "%255s %d %lf", k, &v, &t) == 3)
                if (key == k && v >= 0 && v < NBG_MIX_VARIANTS) {
                    best = v;
                    best_t = t;
                }
            fclose(f);
        }
    }
    if (best < 0) {
        const int prev = ctx->cb.mix_variant;
        for (int v = 0; v < NBG_MIX_VARIANTS; v++) {
            if ((rc = select_variant(ctx, v)) != NBG_OK) return rc;
            /* one untimed force pass grows the buffers this shape needs; a
             * symmetric shape whose j partials do not fit is passed over */
            if ((rc = nbg_force_pass(ctx)) != NBG_OK) {
                if (nbg_mix_is_sym(v) && rc == NBG_E_CUDA) {
                    cudaGetLastError();
                    continue;
                }
                select_variant(ctx, prev);
                return rc;
            }
            float ms = 0, t = 1e30f;
            for (int rep = 0; rep < 4; rep++) {
                if ((rc = time_mixed_pair(ctx, &ms)) != NBG_OK) {
                    select_variant(ctx, prev);
                    return rc;
                }
                if (rep > 0 && ms < t) t = ms; /* the first run warms up */
            }
            if (best < 0 || t < best_t) {
                best = v;
                best_t = t;
            }
        }
        if (cache_path) {
            if (FILE *f = fopen(cache_path, "a")) {
                fprintf(f, "%s %d %.6f\n", key.c_str(), best, best_t);
                fclose(f);
            }
        }
    }
    if ((rc = select_variant(ctx, best)) != NBG_OK) return rc;
    if (!nbg_mix_is_sym(best) && ctx->cb.jpart) {
        /* a one-sided shape won: the symmetric kernel's slots go */
        CK(cudaStreamSynchronize(ctx->st));
        cudaFree(ctx->cb.jpart);
        ctx->cb.jpart = nullptr;
        ctx->cb.jpart_units = 0;
        invalidate_graph(ctx);
    }
    if (variant) *variant = best;
    if (best_ms) *best_ms = best_t;
    return NBG_OK;
}

int nbg_get_renderables(nbg_ctx *ctx, nbg_renderable *host, int64_t cap, int64_t *n)
{
    if (!ctx || cap < 0) return fail(ctx, NBG_E_ARG, "bad arguments");
    CK(cudaSetDevice(ctx->device));
    int rc = sync_ctl(ctx);
    if (rc != NBG_OK) return rc;
    ll m = ctx->ctl_h->rend_n;
    if (n) *n = m;
    if (host && m > 0) {
        if ((rc = get_field(ctx, host, ctx->cb.rend, m < cap ? m : cap)) != NBG_OK) return rc;
        CK(cudaStreamSynchronize(ctx->st));
    }
    return NBG_OK;
}

int nbg_set_render_ring(nbg_ctx *ctx, void *ring, int64_t slot_cap, int slots)
{
    if (!ctx) return NBG_E_ARG;
    if (ring && (slot_cap < 1 || slots < 1)) return fail(ctx, NBG_E_ARG, "ring needs slot_cap >= 1 and slots >= 1");
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->st)); /* no cycle in flight writes the old ring */
    if (ctx->ring_host) {
        cudaHostUnregister(ctx->ring_host);
        ctx->ring_host = nullptr;
    }
    ctx->cb.ring_head = nullptr;
    ctx->cb.ring_rend = nullptr;
    ctx->cb.ring_cap = 0;
    ctx->cb.ring_slots = 0;
    invalidate_graph(ctx);
    if (!ring) return NBG_OK;
    nbg_ring_slot *h = (nbg_ring_slot *)ring;
    for (int s = 0; s < slots; s++) h[s] = nbg_ring_slot{-1, 0, 0, 0};
    const size_t bytes = (size_t)NBG_RING_BYTES(slots, slot_cap);
    cudaError_t e = cudaHostRegister(ring, bytes, cudaHostRegisterMapped);
    if (e != cudaSuccess) return fail(ctx, NBG_E_CUDA, std::string("cudaHostRegister: ") + cudaGetErrorString(e));
    void *dev = nullptr;
    e = cudaHostGetDevicePointer(&dev, ring, 0);
    if (e != cudaSuccess) {
        cudaHostUnregister(ring);
        return fail(ctx, NBG_E_CUDA, std::string("cudaHostGetDevicePointer: ") + cudaGetErrorString(e));
    }
    ctx->ring_host = ring;
    ctx->cb.ring_head = (nbg_ring_slot *)dev;
    ctx->cb.ring_rend = (nbg_renderable *)((char *)dev + (size_t)slots * sizeof(nbg_ring_slot));
    ctx->cb.ring_cap = slot_cap;
    ctx->cb.ring_slots = slots;
    return NBG_OK;
}

int nbg_get_events(nbg_ctx *ctx, nbg_event *host, int64_t cap, int64_t *n)
{
    if (!ctx || cap < 0) return fail(ctx, NBG_E_ARG, "bad arguments");
    CK(cudaSetDevice(ctx->device));
    int rc = sync_ctl(ctx);
    if (rc != NBG_OK) return rc;
    ll m = ctx->ctl_h->last_ev_n;
    if (n) *n = m;
    if (host && m > 0) {
        if ((rc = get_field(ctx, host, ctx->cb.ev_out, m < cap ? m : cap)) != NBG_OK) return rc;
        CK(cudaStreamSynchronize(ctx->st));
    }
    return NBG_OK;
}

int nbg_get_forces(nbg_ctx *ctx, double *fx, double *fy, double *fz, int64_t cap, int64_t *n)
{
    if (!ctx || cap < 0) return fail(ctx, NBG_E_ARG, "bad arguments");
    CK(cudaSetDevice(ctx->device));
    int rc = sync_ctl(ctx);
    if (rc != NBG_OK) return rc;
    ll m = ctx->ctl_h->n;
    if (n) *n = m;
    ll c = m < cap ? m : cap;
    if ((rc = get_field(ctx, fx, (const double *)ctx->cb.a.fx, c)) != NBG_OK) return rc;
    if ((rc = get_field(ctx, fy, (const double *)ctx->cb.a.fy, c)) != NBG_OK) return rc;
    if ((rc = get_field(ctx, fz, (const double *)ctx->cb.a.fz, c)) != NBG_OK) return rc;
    CK(cudaStreamSynchronize(ctx->st));
    return NBG_OK;
}

int nbg_energy(nbg_ctx *ctx, double *kinetic, double *potential, double momentum[3])
{
    if (!ctx) return NBG_E_ARG;
    if (ctx->cb.seg.nsims < 1) return fail(ctx, NBG_E_STATE, "no collection is loaded (a segment allocation failed)");
    CK(cudaSetDevice(ctx->device));
    int rc = sync_ctl(ctx);
    if (rc != NBG_OK) return rc;
    ll nb = (ctx->cb.cap + 127) / 128;
    if ((rc = ensure_scratch(ctx, (size_t)nb * 5 * sizeof(double))) != NBG_OK) return rc;
    CK(cudaMemsetAsync(ctx->scratch, 0, (size_t)nb * 5 * sizeof(double), ctx->st));
    nbg_launch_energy(ctx->cb, ctx->ctl, (double *)ctx->scratch, ctx->st);
    CK(cudaGetLastError());
    std::vector<double> p((size_t)nb * 5);
    CK(cudaMemcpyAsync(p.data(), ctx->scratch, p.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    double s[5] = {0, 0, 0, 0, 0};
    for (ll b = 0; b < nb; b++)
        for (int q = 0; q < 5; q++) s[q] += p[(size_t)(b * 5 + q)];
    if (kinetic) *kinetic = s[0];
    if (potential) *potential = s[1];
    if (momentum) {
        momentum[0] = s[2];
        momentum[1] = s[3];
        momentum[2] = s[4];
    }
    return NBG_OK;
}

int nbg_enable_timing(nbg_ctx *ctx, int on)
{
    if (!ctx) return NBG_E_ARG;
    ctx->timing = on != 0;
    return NBG_OK;
}

int nbg_get_timing(nbg_ctx *ctx, nbg_timing *t)
{
    if (!ctx || !t) return NBG_E_ARG;
    *t = ctx->tacc;
    return NBG_OK;
}

int nbg_set_option(nbg_ctx *ctx, int key, int64_t value)
{
    if (!ctx) return NBG_E_ARG;
    switch (key) {
    case NBG_OPT_SPLIT:
        if (value < 0 || value > (1 << 24)) return fail(ctx, NBG_E_ARG, "chunk cap must be 0..2^24");
        if (value != ctx->cb.work_cap) {
            ctx->cb.work_cap = (int)value;
            invalidate_graph(ctx);
        }
        return NBG_OK;
    case NBG_OPT_GRAPH:
        ctx->use_graph = value != 0;
        return NBG_OK;
    case NBG_OPT_MIX_SHAPE:
        if (value < 0 || value >= NBG_MIX_VARIANTS) return fail(ctx, NBG_E_ARG, "unknown kernel shape");
        return select_variant(ctx, (int)value);
    case NBG_OPT_BH_SHAPE:
        if (value < 0 || value > 2) return fail(ctx, NBG_E_ARG, "Barnes-Hut walk shape must be 0..2");
        ctx->cb.bh_shape = (int)value;
        invalidate_graph(ctx);
        return NBG_OK;
    case NBG_OPT_BARNES_HUT: {
        CK(cudaSetDevice(ctx->device));
        const int on = value != 0;
        if (on == ctx->cb.bh) return NBG_OK;
        ctx->cb.bh = on;
        invalidate_graph(ctx);
        if (on) return ensure_bh(ctx, 0);
        nbg_bh_free(ctx->cb.t);
        ctx->bh_cap = 0;
        return NBG_OK;
    }
    case NBG_OPT_GRAPH_CYCLES:
        if (value < 1 || value > 1000) return fail(ctx, NBG_E_ARG, "cycles per graph must be 1..1000");
        if (value != ctx->graph_cycles) {
            ctx->graph_cycles = (int)value;
            invalidate_graph(ctx);
        }
        return NBG_OK;
    case NBG_OPT_EVENT_SORT:
        if (value < 0 || value > 2) return fail(ctx, NBG_E_ARG, "event sort mode must be 0..2");
        ctx->ev_sort_mode = (int)value;
        return NBG_OK;
    case NBG_OPT_TEST_WAIT_STALL: {
        if (value < 0 || value > 1) return fail(ctx, NBG_E_ARG, "wait-stall hook must be 0 or 1");
        const unsigned extra = value ? 16u : 0u;
        ctx->ctl_h->test_tx_extra = extra;
        return ctl_put(ctx, offsetof(DevCtl, test_tx_extra), &extra, sizeof extra);
    }
    case NBG_OPT_TEST_FAIL_GROWTH:
        if (value < 0 || value > 1) return fail(ctx, NBG_E_ARG, "growth-failure hook must be 0 or 1");
        ctx->test_fail_growth = value != 0;
        return NBG_OK;
    case NBG_OPT_STEP_DEADLINE_MS:
        if (value < 0 || value > ((ll)1 << 40)) return fail(ctx, NBG_E_ARG, "deadline must be 0..2^40 ms");
        ctx->deadline_ms = value;
        return NBG_OK;
    case NBG_OPT_P64_SPLIT_MAX:
        if (value < 0 || value > NBG_MAX_BODIES) return fail(ctx, NBG_E_ARG, "split limit must be 0..2^30");
        ctx->p64_split_max = value;
        return NBG_OK;
    case NBG_OPT_SORT_INTERVAL: {
        if (value < 1 || value > 1000) return fail(ctx, NBG_E_ARG, "sort interval must be 1..1000 cycles");
        const int k = (int)value;
        return ctl_put(ctx, offsetof(DevCtl, sort_interval), &k, sizeof k);
    }
    case NBG_OPT_NEAR_PPM: {
        if (value < 0 || value > 10000000) return fail(ctx, NBG_E_ARG, "near radius factor out of range");
        float kappa = (float)((double)value * 1e-6);
        return ctl_put(ctx, offsetof(DevCtl, near_kappa), &kappa, sizeof kappa);
    }
    case NBG_OPT_EV_CAP: {
        if (value < 1 || value > ((ll)1 << 34)) return fail(ctx, NBG_E_ARG, "event capacity out of range");
        CK(cudaSetDevice(ctx->device));
        CK(cudaStreamSynchronize(ctx->st));
        return alloc_events(ctx, next_pow2(value));
    }
    case NBG_OPT_FRAG_CAP: {
        if (value < 1 || value > NBG_MAX_BODIES) return fail(ctx, NBG_E_ARG, "fragment capacity out of range");
        CK(cudaSetDevice(ctx->device));
        CK(cudaStreamSynchronize(ctx->st));
        free_arrays(ctx->cb.frags);
        ctx->cb.frag_cap = 0;
        invalidate_graph(ctx);
        CK(alloc_arrays(ctx->cb.frags, value));
        ctx->cb.frag_cap = value;
        return NBG_OK;
    }
    default:
        return fail(ctx, NBG_E_ARG, "unknown option");
    }
}

int nbg_probe_peaks(int device, double *fp32_flops, double *fp64_flops, double *sm_clock_mhz)
{
    return nbg_run_probes(device, fp32_flops, fp64_flops, sm_clock_mhz);
}

} /* extern "C" */
