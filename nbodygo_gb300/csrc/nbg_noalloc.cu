/*
 * nbg_noalloc.cu - the mixed-precision force pass for callers that cannot
 * allocate device memory.
 *
 * Some callers of this library may not call cudaMalloc at all: a host
 * framework whose memory pool already owns the device (and forbids
 * allocations behind its back), a real-time loop that must never block in
 * the CUDA allocator, or code that runs where an allocation would
 * disturb a memory budget fixed in advance.  nbg_forces_mixed_noalloc serves
 * them.  The caller passes device pointers for the inputs and outputs; every
 * intermediate buffer the force pass needs (sorted packed positions, Morton
 * sort keys, tile origins, partial sums, the control block) lives in one
 * file-scope __device__ array of NBG_NOALLOC_BYTES bytes.  Every GPU that
 * loads the library holds that array until the process exits, which is why
 * it is sized for at most NBG_NOALLOC_MAX_BODIES bodies.
 *
 * The kernels are the ones the context path runs (k_mixed.cu, k_sort.cu);
 * only the buffers differ.
 */
#include <cuda.h> /* CUcontext / CUresult types only; the entry points are resolved at run time */
#include <mutex>
#include <string>

#include "nbg_internal.cuh"

/* partial sums: 786,432 doubles, 512 slots of a 512-body i-tile; a 65,536-body
 * collection has 128 i-tiles, which leaves room for 385 CTAs */
#define NOALLOC_PART_DOUBLES (4 * 3 * NBG_NOALLOC_MAX_BODIES)

static constexpr size_t align256(size_t v) { return (v + 255) / 256 * 256; }

static constexpr size_t OFF_CTL = 0;
static constexpr size_t OFF_JHI = align256(sizeof(DevCtl));
static constexpr size_t OFF_JLO = OFF_JHI + align256((size_t)NBG_NOALLOC_MAX_BODIES * 16);
static constexpr size_t OFF_TILE = OFF_JLO + align256((size_t)NBG_NOALLOC_MAX_BODIES * 16);
static constexpr size_t OFF_IPREP =
    OFF_TILE + align256((size_t)((NBG_NOALLOC_MAX_BODIES + NBG_MIX_ITILE - 1) / NBG_MIX_ITILE) * 16);
static constexpr size_t OFF_PART = OFF_IPREP + align256((size_t)NBG_NOALLOC_MAX_BODIES * 16);
static constexpr size_t OFF_PERM = OFF_PART + align256((size_t)NOALLOC_PART_DOUBLES * 8);
static constexpr size_t OFF_SVAL = OFF_PERM + align256((size_t)NBG_NOALLOC_MAX_BODIES * 4);
static constexpr size_t OFF_KEY0 = OFF_SVAL + align256((size_t)NBG_NOALLOC_MAX_BODIES * 4);
static constexpr size_t OFF_KEY1 = OFF_KEY0 + align256((size_t)NBG_NOALLOC_MAX_BODIES * 4);
static constexpr size_t OFF_HIST = OFF_KEY1 + align256((size_t)NBG_NOALLOC_MAX_BODIES * 4);
/* radix-sort histogram: 256 digits per 4096-body block, then one sum per
 * 8192-entry chunk of it */
static constexpr size_t HIST_ENTRIES = (size_t)((NBG_NOALLOC_MAX_BODIES + 4095) / 4096) * 256;
static constexpr size_t HIST_BYTES = (HIST_ENTRIES + (HIST_ENTRIES + 8191) / 8192) * 8;
/* the per-sim layout arrays of one collection */
static constexpr size_t OFF_SEG = OFF_HIST + align256(HIST_BYTES);
static constexpr size_t TOTAL_BYTES = OFF_SEG + align256(NBG_SEG_BYTES(1));
static_assert(TOTAL_BYTES == NBG_NOALLOC_BYTES, "NBG_NOALLOC_BYTES in nbgpu.h is out of date");

/* The scratch of every call on this device.  In host code this name is only
 * a stand-in: the device address comes from cudaGetSymbolAddress. */
static __device__ __align__(256) unsigned char g_noalloc_scratch[TOTAL_BYTES];

#define NOALLOC_MAX_DEVICES 64
/* The scratch array's device address on each device, with the id of the
 * context it was looked up in.  A device reset (cudaDeviceReset by the host
 * framework) destroys the context and the module with it; the next context
 * gets a new id, so the address is looked up again instead of reused. */
struct ScratchSlot {
    unsigned long long ctx_id;
    unsigned char *addr;
};
static ScratchSlot g_scratch[NOALLOC_MAX_DEVICES];
static std::mutex g_setup_mutex;

/* Driver entry points for the id of the current context, resolved through
 * the runtime (the library does not link the driver library itself). */
typedef CUresult (*PfnCtxGetCurrent)(CUcontext *);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long *);

/* Id of the context current on this thread; 0 if there is none or the
 * driver cannot tell (then the address is looked up on every call).  Called
 * with g_setup_mutex held. */
static unsigned long long current_ctx_id()
{
    static bool resolved = false;
    static PfnCtxGetCurrent get_current = nullptr;
    static PfnCtxGetId get_id = nullptr;
    if (!resolved) {
        resolved = true;
        cudaDriverEntryPointQueryResult q1, q2;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", (void **)&get_current, 12000, cudaEnableDefault,
                                             &q1) != cudaSuccess || q1 != cudaDriverEntryPointSuccess)
            get_current = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", (void **)&get_id, 12000, cudaEnableDefault, &q2) !=
                cudaSuccess || q2 != cudaDriverEntryPointSuccess)
            get_id = nullptr;
    }
    if (!get_current || !get_id) return 0;
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
    if (get_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

/* The control block's reductions and counters, and the per-sim arrays, must
 * start at zero; the collection is one sim of n bodies. */
__global__ void k_noalloc_init(DevCtl *ctl, SimSegs seg, ll n, float kappa)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    unsigned char *p = (unsigned char *)ctl;
    for (size_t k = 0; k < sizeof(DevCtl); k++) p[k] = 0;
    unsigned char *q = (unsigned char *)seg.off;
    for (size_t k = 0; k < NBG_SEG_BYTES(1); k++) q[k] = 0;
    ctl->n = n;
    ctl->near_kappa = kappa;
    seg.off[1] = n;
}

static int noalloc_fail(int code, const char *msg);

extern "C" int nbg_forces_mixed_noalloc(const double *x, const double *y, const double *z, const double *mass,
                                        const double *radius, const uint32_t *flags, int64_t n, double *fx,
                                        double *fy, double *fz, void *stream)
{
    if (n < 0 || n > NBG_NOALLOC_MAX_BODIES)
        return noalloc_fail(NBG_E_ARG, "nbg_forces_mixed_noalloc: n must be 0..NBG_NOALLOC_MAX_BODIES (65536)");
    if (n > 0 && (!x || !y || !z || !mass || !radius || !flags || !fx || !fy || !fz))
        return noalloc_fail(NBG_E_ARG, "nbg_forces_mixed_noalloc: a pointer is NULL");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEVICES)
        return noalloc_fail(NBG_E_CUDA, "nbg_forces_mixed_noalloc: no current CUDA device");
    unsigned char *base;
    {
        /* once per device context, with that device current: the device
         * address of the scratch array */
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        unsigned long long id = current_ctx_id();
        if (id == 0) {
            /* no context current on this thread yet: make the device's
             * primary context current, as the runtime's first call would */
            if (cudaSetDevice(dev) != cudaSuccess)
                return noalloc_fail(NBG_E_CUDA, "nbg_forces_mixed_noalloc: cudaSetDevice failed");
            id = current_ctx_id();
        }
        if (id == 0 || g_scratch[dev].ctx_id != id || !g_scratch[dev].addr) {
            void *ptr = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
            if (e != cudaSuccess || !ptr)
                return noalloc_fail(NBG_E_CUDA, "nbg_forces_mixed_noalloc: cudaGetSymbolAddress failed");
            g_scratch[dev].ctx_id = id;
            g_scratch[dev].addr = (unsigned char *)ptr;
        }
        base = g_scratch[dev].addr;
    }
    if (n == 0) return NBG_OK;
    cudaStream_t st = (cudaStream_t)stream;

    CycleBufs cb;
    memset(&cb, 0, sizeof cb);
    cb.a.x = const_cast<double *>(x);
    cb.a.y = const_cast<double *>(y);
    cb.a.z = const_cast<double *>(z);
    cb.a.m = const_cast<double *>(mass);
    cb.a.rad = const_cast<double *>(radius);
    cb.a.flags = const_cast<unsigned *>(flags);
    cb.a.fx = fx;
    cb.a.fy = fy;
    cb.a.fz = fz;
    cb.cap = NBG_NOALLOC_MAX_BODIES;
    cb.jhi = (float4 *)(base + OFF_JHI);
    cb.jlo = (float4 *)(base + OFF_JLO);
    cb.tile_c = (float4 *)(base + OFF_TILE);
    cb.iprep = (float4 *)(base + OFF_IPREP);
    cb.part = (double *)(base + OFF_PART);
    cb.perm = (unsigned *)(base + OFF_PERM);
    cb.sval = (unsigned *)(base + OFF_SVAL);
    cb.skey[0] = (unsigned *)(base + OFF_KEY0);
    cb.skey[1] = (unsigned *)(base + OFF_KEY1);
    cb.shist = (ll *)(base + OFF_HIST);
    cb.ev_keys = nullptr; /* events are discarded */
    cb.ev_cap = 0;
    cb.part_doubles = NOALLOC_PART_DOUBLES;
    cb.work_cap = 0;
    cb.mix_variant = 0; /* the default shape: 512-body i-tiles */
    cb.itile = NBG_MIX_ITILE;
    cb.slots = nbg_mixed_slots(dev, 0);
    if (cudaDeviceGetAttribute(&cb.sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || cb.sms < 1)
        return noalloc_fail(NBG_E_CUDA, "nbg_forces_mixed_noalloc: no multiprocessor count for the device");
    cb.seg = nbg_seg_carve(base + OFF_SEG, 1);
    DevCtl *ctl = (DevCtl *)(base + OFF_CTL);

    k_noalloc_init<<<1, 1, 0, st>>>(ctl, cb.seg, (ll)n, NBG_NEAR_KAPPA_DEFAULT);
    nbg_launch_begin(cb, ctl, st); /* work layout of the one collection */
    nbg_launch_mixed_prep(cb, ctl, st);
    nbg_launch_mixed_pair(cb, ctl, st);
    nbg_launch_mixed_out(cb, ctl, st);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return noalloc_fail(NBG_E_CUDA, cudaGetErrorString(e));
    return NBG_OK;
}

/* the message is read through nbg_last_error(NULL) */
const char *nbg_set_global_error(const char *msg);

static int noalloc_fail(int code, const char *msg)
{
    nbg_set_global_error(msg);
    return code;
}
