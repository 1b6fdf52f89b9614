/*
 * nbgpu.h - C ABI of the GB300 compute cycle for nbodygo (libnbgpu.so).
 *
 * One context owns the device copy of a body collection and runs the
 * reference's compute cycle on it:
 *
 *   force + collision detection   cmd/body/body.go:148-225 (Compute,
 *                                  calcForceFrom, Collided)
 *   collision resolution          cmd/body/body_collection.go:212-233
 *                                  (ProcessMods), event.go:53-62,
 *                                  body.go:228-264, collisioncalc.go:26-186,
 *                                  fragcalc.go:24-117
 *   integration                   cmd/body/body.go:114-139 (Update)
 *   compaction + adds             cmd/body/body_collection.go:253-296 (Cycle)
 *
 * nbg_step replaces the block of ComputationRunner.runOneComputation from
 * "submit slices" to "bc.Cycle(r.R)" (cmd/runner/computation-runner.go:284-322).
 *
 * Conventions
 *  - Every call returns NBG_OK (0) or an NBG_E_* status; nbg_last_error gives
 *    a message.  Nothing aborts the process or traps on the device.
 *  - Inputs are copied before a call returns; no caller pointer is kept
 *    (this satisfies the cgo pointer-passing rules).
 *  - One thread drives a context at a time (the runner goroutine); calls on
 *    one context are not synchronised against each other.  Different
 *    contexts are independent: several host threads may each drive their
 *    own at the same time, on one GPU or several.
 *  - Body order is the reference's array order: results depend on it exactly
 *    as in the reference (force summation order, event order, compaction).
 *  - Strings (Name, Class), colour and light intensity stay with the caller,
 *    keyed by body id.
 */
#ifndef NBGPU_H
#define NBGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define NBG_OK 0
#define NBG_E_CUDA 1     /* a CUDA runtime call failed (a failed growth of the body capacity leaves
                            the context with no bodies: load a collection again) */
#define NBG_E_ARG 2      /* bad argument (null pointer, size, enum value) */
#define NBG_E_OVERFLOW 3 /* a device buffer was too small; state is unchanged */
#define NBG_E_TIMEOUT 4  /* nbg_step reached its deadline (NBG_OPT_STEP_DEADLINE_MS), or a device wait gave up */
#define NBG_E_NAN 5      /* non-finite value where a finite one is required */
#define NBG_E_STATE 6    /* call not valid in the context's current state */
#define NBG_E_CANCELLED 7 /* nbg_step stopped by nbg_cancel */

/* collision behaviours, values of globals.CollisionBehavior
 * (cmd/globals/globals.go:9-16) */
#define NBG_NONE 0
#define NBG_SUBSUME 1
#define NBG_ELASTIC 2
#define NBG_FRAGMENT 3

/* body flag bits (Body.Exists, IsSun, Pinned, WithTelemetry and the private
 * fragmenting / collided flags, cmd/body/body.go:34-52) */
#define NBG_F_EXISTS 0x01u
#define NBG_F_IS_SUN 0x02u
#define NBG_F_PINNED 0x04u
#define NBG_F_TELEMETRY 0x08u
#define NBG_F_FRAGMENTING 0x10u
#define NBG_F_COLLIDED 0x20u

/* precision forms */
#define NBG_PRECISION_FP64 0  /* plain: the reference's FP64 arithmetic, op for op */
#define NBG_PRECISION_MIXED 1 /* FP32 pair terms, FP64 everything else */

/* event types reported by nbg_get_events (event.go:18-24) */
#define NBG_EV_COLLISION 0 /* b1.ResolveCollision(b2) */
#define NBG_EV_SUBSUME 1   /* b1 subsumes b2 */

typedef struct nbg_ctx nbg_ctx;

/*
 * Structure-of-arrays view of a body collection in host memory.  Element k of
 * every array describes body k.  On input, the optional arrays may be NULL:
 * r defaults to 1 (NewBody, body.go:78), forces and fragment state to 0.
 * On output, NULL arrays are skipped.
 */
typedef struct nbg_soa {
    /* public Body fields (body.go:34-48) */
    int64_t *id;
    double *x, *y, *z, *vx, *vy, *vz, *radius, *mass;
    double *frag_factor, *frag_step;
    int32_t *collision; /* NBG_NONE .. NBG_FRAGMENT */
    uint32_t *flags;    /* NBG_F_* */
    /* private Body fields (body.go:49-52), optional */
    double *r;          /* restitution copy used by doElastic */
    double *fx, *fy, *fz;
    double *frag_radius, *frag_new_radius, *frag_mass;
    int64_t *frag_fragments;
    double *frag_cx, *frag_cy, *frag_cz;
} nbg_soa;

/* Per-call summary filled by nbg_step. */
typedef struct nbg_step_info {
    int64_t steps_done;        /* steps completed by this call */
    int64_t n_bodies;          /* bodies after the last Cycle */
    int64_t interactions;      /* sum over steps of N*(N-1), N at step start */
    int64_t events;            /* collision + subsume events resolved */
    int64_t fragments_emitted; /* bodies added by fragmentation */
    int64_t removed;           /* bodies removed by Cycle */
    int64_t nan_removed;       /* bodies removed because x, y or z became NaN */
    int64_t next_id;           /* next id NextId() would return */
    int64_t bh_terms;          /* Barnes-Hut: point-mass terms the force pass summed */
} nbg_step_info;

/* Renderable (cmd/body/renderable.go:9-17) minus host-side colour/intensity. */
typedef struct nbg_renderable {
    int64_t id;
    float x, y, z;
    uint32_t flags; /* NBG_F_EXISTS, NBG_F_IS_SUN */
    double radius;
} nbg_renderable;

/* One resolved event of the last step, in the order it was handled. */
typedef struct nbg_event {
    int64_t id1, id2; /* b1, b2 of event.go:38-41 */
    int32_t type;     /* NBG_EV_* */
    int32_t pad;
} nbg_event;

/* ModBody edit of one body (body.go:274-313 ApplyMods, after parsing).  Each
 * bit of `mask` selects one field. */
#define NBG_M_X 0x0001u
#define NBG_M_Y 0x0002u
#define NBG_M_Z 0x0004u
#define NBG_M_VX 0x0008u
#define NBG_M_VY 0x0010u
#define NBG_M_VZ 0x0020u
#define NBG_M_MASS 0x0040u
#define NBG_M_RADIUS 0x0080u
#define NBG_M_FRAG_FACTOR 0x0100u
#define NBG_M_FRAG_STEP 0x0200u
#define NBG_M_COLLISION 0x0400u
#define NBG_M_TELEMETRY 0x0800u
#define NBG_M_EXISTS 0x1000u
typedef struct nbg_edit {
    int64_t id;  /* body to modify */
    uint32_t mask;
    int32_t collision;
    double x, y, z, vx, vy, vz, mass, radius, frag_factor, frag_step;
    int32_t telemetry, exists;
} nbg_edit;

/* ---- context ---------------------------------------------------------- */

/* Creates a context on CUDA device `device` able to hold `capacity` bodies
 * (it grows on demand).  precision: NBG_PRECISION_FP64 or _MIXED.
 * Replaces NewComputationRunner's worker pool (computation-runner.go:81-98). */
int nbg_create(int device, int precision, int64_t capacity, nbg_ctx **out);
void nbg_destroy(nbg_ctx *ctx);
/* the context's last error message; with NULL, the calling thread's last
 * error of a call that had no context (nbg_create, the allocation-free pass) */
const char *nbg_last_error(const nbg_ctx *ctx);
int nbg_set_precision(nbg_ctx *ctx, int precision);
/* The context's current form (NBG_PRECISION_*): the one it was created or
 * set to, or the one a loaded snapshot carried. */
int nbg_get_precision(nbg_ctx *ctx, int *precision);
/* Runs the context's work on the caller's CUDA stream (a cudaStream_t passed
 * as void *; NULL restores the context's own stream). */
int nbg_set_stream(nbg_ctx *ctx, void *stream);

/* Seed of the fragment-position generator and the id counter (NextId,
 * body.go:316-329).  Fragments take ids from this counter. */
int nbg_set_seed(nbg_ctx *ctx, uint64_t seed);
int nbg_set_next_id(nbg_ctx *ctx, int64_t next_id);
int nbg_get_next_id(nbg_ctx *ctx, int64_t *next_id);
/* Cycle index used to key the fragment generator (starts at 0). */
int nbg_set_cycle(nbg_ctx *ctx, uint64_t cycle);

/* ---- body set ---------------------------------------------------------- */

/* Replaces the whole collection (NewSimBodyCollection, body_collection.go:45-68). */
int nbg_set_bodies(nbg_ctx *ctx, const nbg_soa *host, int64_t n);
/* Replaces the contents with `nsims` independent collections (1..2048) stored
 * one after another: counts[s] bodies each, concatenated in `host`.  Bodies
 * of different collections never interact; every collection follows the
 * cycle exactly as if it were alone (its own event order, compaction, adds),
 * and one nbg_step advances all of them with the same dt and R.  This is
 * the batched form: many small simulations share each kernel launch.  No
 * counterpart in the reference, which runs one collection per process.
 * nbg_add_bodies and nbg_remove_bodies need a single collection; their
 * per-collection forms (nbg_add_bodies_to, nbg_remove_bodies_from) take one. */
int nbg_set_collections(nbg_ctx *ctx, int64_t nsims, const int64_t *counts, const nbg_soa *host);
/* Body count of each collection (up to cap entries); *nsims = collections. */
int nbg_sim_counts(nbg_ctx *ctx, int64_t *counts, int64_t cap, int64_t *nsims);
/* Number of bodies in the array (BodyCollection.Count, body_collection.go:203-207). */
int nbg_count(nbg_ctx *ctx, int64_t *n);
/* Copies up to `cap` bodies out; *n receives the count. */
int nbg_get_state(nbg_ctx *ctx, nbg_soa *host, int64_t cap, int64_t *n);

/* Enqueue(NewAdd(b)) for n bodies (body_collection.go:82-88, event.go:104-111):
 * they are appended by the next step's Cycle, newest first, with r = R.
 * If host->id is NULL or an entry is negative, an id is taken from the
 * counter; assigned ids are written to ids_out (may be NULL). */
int nbg_add_bodies(nbg_ctx *ctx, const nbg_soa *host, int64_t n, int64_t *ids_out);

/* ModBody by id (body_collection.go:154-191 HandleModBody): applies each edit
 * to every body with that id; results[k] = number of bodies matched. */
int nbg_apply_edits(nbg_ctx *ctx, const nbg_edit *edits, int64_t k, int32_t *results);

/* RemoveBodies (computation-runner.go:171-216 processDeletes): count == -1
 * removes every body, otherwise `count` unpinned bodies spread evenly through
 * the array.  *removed receives the number removed (may be NULL). */
int nbg_remove_bodies(nbg_ctx *ctx, int64_t count, int64_t *removed);

/* GetBody by id (body_collection.go:111-135): copies the first body with that
 * id into element 0 of `host`; *found = 0 if there is none. */
int nbg_get_body(nbg_ctx *ctx, int64_t id, nbg_soa *host, int32_t *found);

/* The same four controls addressed to collection `sim` (0-based, in the
 * order nbg_set_collections loaded them) of a context holding several: the
 * gRPC AddBody / ModBody / RemoveBodies / GetBody of one simulation
 * (cmd/sim/grpcsimcb.go:15-70), each collection behaving as its own
 * reference process.  sim = -1 means every collection for nbg_apply_edits_in
 * and nbg_get_body_in.  Adds are appended by that collection's next Cycle,
 * newest first; their ids come from the context's one counter unless given.
 * processDeletes spreads `count` removals over that collection alone
 * (computation-runner.go:176-216). */
int nbg_add_bodies_to(nbg_ctx *ctx, int64_t sim, const nbg_soa *host, int64_t n, int64_t *ids_out);
int nbg_apply_edits_in(nbg_ctx *ctx, int64_t sim, const nbg_edit *edits, int64_t k, int32_t *results);
int nbg_remove_bodies_from(nbg_ctx *ctx, int64_t sim, int64_t count, int64_t *removed);
int nbg_get_body_in(nbg_ctx *ctx, int64_t sim, int64_t id, nbg_soa *host, int32_t *found);

/* ---- snapshots ---------------------------------------------------------- */

/*
 * A binary snapshot of everything the next cycle reads, so a run can stop
 * and resume later, in this or another context, and repeat the
 * uninterrupted run bit for bit.  The reference's CSV format
 * (cmd/sim/fromcsv.go:46-116) holds only the public Body fields; a snapshot
 * adds the private ones a cycle carries over (r, fragmenting and its
 * fragInfo, collided, the stale force a fragmenting body re-applies,
 * body.go:49-52,152-155), the NextId counter (body.go:316-329), the cycle
 * index that keys the fragment generator, its seed, the host adds staged
 * for the next Cycle, the collections' sizes, the precision form, kernel
 * shape and options, and in the mixed form the bodies' current Morton order.
 *
 * nbg_save_state: *size receives the snapshot's bytes; with buf NULL that is
 * all it does (a size query).  A cap below the size returns NBG_E_OVERFLOW.
 * nbg_load_state replaces the context's bodies, collections, staged adds,
 * counters and options with the snapshot's.  The layout is described in
 * nbg_api.cu; values are in the machine's byte order.
 */
int nbg_save_state(nbg_ctx *ctx, void *buf, int64_t cap, int64_t *size);
int nbg_load_state(nbg_ctx *ctx, const void *buf, int64_t size);

/* ---- the cycle ---------------------------------------------------------- */

/* Runs `nsteps` compute cycles with time step dt (timeScaling) and
 * coefficient of restitution R.  nsteps > 1 replays a CUDA graph of one cycle.
 * On NBG_E_OVERFLOW the context grows the buffer that was short and the
 * interrupted cycle can be re-run: state is left as it was before it.
 * A long call can be stopped: nbg_cancel, or the call's deadline, ends it at
 * a cycle boundary within about two launches (graphs or single cycles) and
 * it returns NBG_E_CANCELLED or NBG_E_TIMEOUT with *info filled and the
 * state that after the info->steps_done cycles it ran. */
int nbg_step(nbg_ctx *ctx, double dt, double R, int nsteps, nbg_step_info *info);

/* Asks the nbg_step running on ctx - or, if none is, the next one - to stop
 * at the next cycle boundary.  Safe to call from any thread: it is the one
 * call that may overlap another call on the same context (the reference's
 * runner stops between cycles the same way, computation-runner.go:225-245). */
int nbg_cancel(nbg_ctx *ctx);

/* Runs only the force + collision-detection pass of a cycle on the current
 * state: the forces of bodies that exist and are not fragmenting are
 * recomputed; nothing else changes and the detected events are discarded.
 * For diagnostics and accuracy measurements. */
int nbg_force_pass(nbg_ctx *ctx);

/* Renderables written by the last cycle's Update (one per body in the array
 * before compaction; renderable.go:22-40). */
int nbg_get_renderables(nbg_ctx *ctx, nbg_renderable *host, int64_t cap, int64_t *n);

/* Header of one slot of a render ring. */
typedef struct nbg_ring_slot {
    int64_t cycle;   /* cycle whose renderables the slot holds (-1: none yet) */
    int64_t count;   /* renderables of that cycle */
    int64_t written; /* of them in the slot: min(count, slot capacity) */
    int64_t pad;
} nbg_ring_slot;

/* Bytes of a render ring of `slots` slots of `slot_cap` renderables: the
 * slots' headers, then each slot's renderables. */
#define NBG_RING_BYTES(slots, slot_cap) \
    ((int64_t)(slots) * (int64_t)sizeof(nbg_ring_slot) + \
     (int64_t)(slots) * (int64_t)(slot_cap) * (int64_t)sizeof(nbg_renderable))

/* Renderables written straight into host memory by every cycle's Update, the
 * path of the reference's result queue (computation-runner.go:316-321,
 * resultqueue.go:97-129) without a copy call.  `ring` (NBG_RING_BYTES of
 * memory the caller owns) is pinned and mapped here; cycle c writes slot
 * c mod slots: its renderables first, then the header's count and written,
 * then its cycle, each after a system-wide fence, so a reader that sees a
 * slot's cycle change finds the slot complete.  A reader must copy a slot
 * out before `slots` more cycles overwrite it.  NULL detaches (and unpins). */
int nbg_set_render_ring(nbg_ctx *ctx, void *ring, int64_t slot_cap, int slots);

/* Events resolved by the last cycle, in resolution order.  Self-collisions
 * (b1 == b2), which the reference enqueues and then resolves as no-ops
 * (collisioncalc.go:89-92), are not reported. */
int nbg_get_events(nbg_ctx *ctx, nbg_event *host, int64_t cap, int64_t *n);

/* Net force of the last cycle's force pass for every body (fx, fy, fz of
 * body.go:49).  Any pointer may be NULL. */
int nbg_get_forces(nbg_ctx *ctx, double *fx, double *fy, double *fz, int64_t cap, int64_t *n);

/* Total energy (kinetic + pairwise potential, FP64) and momentum of the bodies
 * that exist, summed over the collections (pairs within each collection); a
 * diagnostic, O(N^2) on the device. */
int nbg_energy(nbg_ctx *ctx, double *kinetic, double *potential, double momentum[3]);

/* ---- force pass without device allocation ------------------------------ */

/*
 * No counterpart in the reference: an entry point for callers that cannot
 * allocate device memory (a host framework whose pool owns the device, a
 * real-time loop that must not block in the allocator).  It runs the
 * mixed-precision force pass of nbg_force_pass on caller-owned device arrays:
 * x, y, z, mass, radius (FP64), flags (NBG_F_*; bodies that exist and are not
 * fragmenting get a force), and writes fx, fy, fz of those bodies.  Every
 * intermediate buffer lives in one static device array of NBG_NOALLOC_BYTES
 * that each GPU loading the library holds until exit; no cudaMalloc or
 * cudaFree is called.  Collision events are not reported.
 *  - n may be at most NBG_NOALLOC_MAX_BODIES; larger n returns NBG_E_ARG.
 *  - The work is queued on `stream` (a cudaStream_t; NULL is the default
 *    stream) and the call returns without waiting.
 *  - The first call on a device looks up the static array's device address
 *    (and makes the device's primary context current if no context is);
 *    make that first call before any stream capture.  The address is kept
 *    with the id of the context it was found in: after a device reset
 *    (cudaDeviceReset) the next call, in the new context, looks it up again,
 *    and that call too belongs before any capture.
 *  - All calls on one device share the array: calls that may overlap on the
 *    GPU (other streams, other host threads) race and must be serialised by
 *    the caller.
 * Errors are reported through nbg_last_error(NULL).
 */
#define NBG_NOALLOC_MAX_BODIES 65536
#define NBG_NOALLOC_BYTES 10521856
int nbg_forces_mixed_noalloc(const double *x, const double *y, const double *z, const double *mass,
                             const double *radius, const uint32_t *flags, int64_t n, double *fx, double *fy,
                             double *fz, void *stream);

/* ---- measurement ------------------------------------------------------- */

/* Device time of the kernels of the last nbg_step call, summed over its
 * cycles, measured with CUDA events on the context's stream.  Slot 0 is the
 * pair (force + detection) kernel, 1 everything else of the cycle. */
typedef struct nbg_timing {
    double pair_ms;
    double other_ms;
    int64_t pair_launches;
    int64_t kernel_launches; /* all kernels of this library launched */
} nbg_timing;
int nbg_enable_timing(nbg_ctx *ctx, int on);
int nbg_get_timing(nbg_ctx *ctx, nbg_timing *t);

/* Tuning knobs of the pair kernels (0 = default). */
#define NBG_OPT_SPLIT 1      /* mixed: most chunks the pair work is cut into (0 = 32 per resident CTA) */
#define NBG_OPT_GRAPH 2      /* 0 = launch each cycle directly, 1 = CUDA graph */
#define NBG_OPT_EV_CAP 3     /* event-list capacity (rounded up to a power of two) */
#define NBG_OPT_FRAG_CAP 4   /* fragments one cycle may emit */
#define NBG_OPT_GRAPH_CYCLES 6 /* cycles captured in one CUDA graph (default 1) */
#define NBG_OPT_MIX_SHAPE 7    /* shape of the mixed pair kernel, 0..NBG_MIX_SHAPES-1 (see nbg_autotune) */
#define NBG_MIX_SHAPES 19
/* 1: forces from the Barnes-Hut octree of cmd/body/octree.go (opening angle
 * 0.3, softening 1e-4, suns summed directly) with the FP64 arithmetic of the
 * plain form, in either precision; collisions stay exact.  This is the
 * reference's --barnes-hut path with its missing Octree.Build call made
 * (body_collection.go:298-300).  With several collections each gets its own
 * tree, the one a context holding it alone would build. */
#define NBG_OPT_BARNES_HUT 8
/* mixed Barnes-Hut walk: registers capped for 3, 4 or 5 CTAs per SM (0..2) */
#define NBG_OPT_BH_SHAPE 9
/* mixed: cycles between Morton sorts of the i-tiles (1..1000, default 4).
   Bodies move far less than a tile per cycle, so an older order still gives
   compact tiles.  Compaction carries the order along (kept bodies keep their
   places, arrivals follow); loads and host edits sort again at the next
   cycle.  The order affects FP32 rounding, never the event set.  1 sorts
   every cycle. */
#define NBG_OPT_SORT_INTERVAL 10
/* plain form, one collection: up to this capacity (default 65536) the pair
   terms of all (i, j) are computed at once and each body adds its own in j
   order; above it one thread walks each body's j.  Identical results; the
   first keeps the FP64 pipes busy when there are few bodies, at the cost of
   a 48 MB-per-thousand-bodies term buffer. */
#define NBG_OPT_P64_SPLIT_MAX 11
/* wall-clock limit of one nbg_step call in milliseconds (0 = none): the call
   launches no further cycle once it has passed, and returns NBG_E_TIMEOUT */
#define NBG_OPT_STEP_DEADLINE_MS 12
/* ordering of a cycle's detected events (ProcessMods' order): up to 4,096
   are sorted by one block in shared memory; more by a multi-block radix sort
   when the cycle's launches include it, else by that one block in global
   memory.  0 (default): include it in the calls after one whose busiest cycle
   had more than 4,096 events, until a call stays under 1,024; 1: always;
   2: never.  The order, and so every result, is the same either way. */
#define NBG_OPT_EVENT_SORT 13
/* test hook for the bounded device waits: 1 makes the bulk-copy shapes (17,
   18) arm each mbarrier for 16 bytes more than their copies bring, so no
   wait completes; every wait gives up after about 2 s of SM clock, the CTA
   waits (bounded again) for its copies and leaves, and the cycle fails with
   NBG_E_TIMEOUT.  The context stays usable; 0 (default) turns it off. */
#define NBG_OPT_TEST_WAIT_STALL 14
/* test hook for a failed capacity growth: 1 makes the next growth of the
   body capacity fail as a device out of memory would, after the old
   buffers were released.  The call fails with NBG_E_CUDA and the context
   is left with no bodies (one empty collection, no staged adds); it stays
   usable, and the next load allocates again.  The hook clears itself. */
#define NBG_OPT_TEST_FAIL_GROWTH 15
#define NBG_OPT_NEAR_PPM 5   /* mixed: pairs closer than (value * 1e-6) x the i-body's
                                distance from its tile origin take the near-pair
                                pass: the exact hi/lo difference, FP64 for a
                                possible overlap (default 50000; twice the
                                value in collections of at most 2,048 bodies,
                                where a tile spans the collection) */
int nbg_set_option(nbg_ctx *ctx, int key, int64_t value);

/* Autotuner of the mixed pair kernel.  Nineteen shapes are compiled, the first fifteen each
 * threads per CTA x i-bodies per thread, j per shared-memory tile, unroll,
 * CTAs per SM, in three kinds: sums in registers (R), sums in shared memory
 * (S), and shared memory with two j-tile buffers filled a tile ahead (D):
 *   0: R 128x4, 256, 2, 3 (default)  1: R 128x4, 256, 1, 3  2: R 128x2, 256, 2, 4
 *   3: R 256x2, 256, 2, 2            4: R 128x4, 512, 2, 3  5: R 64x4, 256, 2, 6
 *   6: R 128x2, 128, 4, 4            7: S 128x2, 256, 2, 5  8: S 128x3, 256, 2, 4
 *   9: S 128x4, 256, 2, 4           10: S 128x4, 128, 4, 4 11: D 128x2, 128, 4, 4
 *  12: D 128x2, 256, 2, 4           13: D 128x2, 128, 2, 4 14: D 128x4, 128, 2, 3
 * two of the symmetric kernel, which computes each unordered pair once
 * and adds its term to both bodies (512-body blocks, 4 i-bodies per thread,
 * j pairs rotated through each warp's lanes):
 *  15: 128x4, 4 CTAs/SM              16: 128x4, 5 CTAs/SM
 * and two more one-sided shapes of kind B, sums in shared memory with the
 * raw j tiles brought into shared memory by bulk copies (cp.async.bulk on an
 * mbarrier) issued two tiles ahead and re-centred from there:
 *  17: B 128x2, 256, 2, 5           18: B 128x4, 256, 2, 4
 * nbg_autotune times the pair kernel of each on the context's current
 * collection (the best of three force passes after one warm-up) and keeps the
 * fastest.  cache_path (may be NULL) names a text file of earlier results
 * keyed by GPU name, SM count, body-count bucket (power of two) and
 * collection-count bucket: a matching entry is used without measuring, and a
 * new measurement is appended. */
int nbg_autotune(nbg_ctx *ctx, const char *cache_path, int *shape, double *best_ms);

/* Peak probes: FFMA (FP32) and DFMA (FP64) throughput of the device in
 * FLOP/s (an FMA counts 2), measured with dependent-chain kernels. */
int nbg_probe_peaks(int device, double *fp32_flops, double *fp64_flops, double *sm_clock_mhz);

#ifdef __cplusplus
}
#endif

#endif /* NBGPU_H */
