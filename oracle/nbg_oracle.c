/*
 * nbg_oracle.c - CPU oracle of the nbodygo direct-sum compute cycle.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU kernels and the timed CPU
 * baseline of bench.py.  Nothing in the product links or calls it.
 *
 * Pinning: the reference's own tests for this path hold almost no numbers,
 * and Go is not installed where this runs, so parity with the reference
 * itself is pinned only through restatements of those tests
 * (tests/test_oracle_reference_kat.py), an independent pure-Python
 * restatement's fixtures (tests/golden/) and a platform-libm variant of this
 * file that bounds the one numeric substitution below
 * (tests/test_oracle_libm_bound.py).
 *
 * It restates, function by function, the reference's Go code with the same
 * data shapes: one heap record per body and an array of pointers
 * (cmd/body/body_collection.go:16), two O(N) passes per body (force, then
 * collision detection), an event queue, single-threaded resolution,
 * integration and compaction.  Floating-point expressions keep Go's
 * evaluation order; the file must be compiled with -ffp-contract=off so no
 * multiply-add is fused (Go on amd64 fuses none).
 *
 * Canonical order.  The reference's event order depends on goroutine
 * scheduling (worker arrival order, an asynchronous channel drain that may
 * drop events when 1000 are in flight).  The oracle fixes the order a single
 * worker with a fully drained, never-dropping channel produces: events arrive
 * body by body in array order and, within a body, in array order of the other
 * body; ProcessMods handles them newest first (PushFront + walk from Front,
 * body_collection.go:93-104,212-233); Cycle appends adds newest first.
 * Multi-threaded compute (slices as computation-runner.go:284-305) collects
 * each slice's events separately and concatenates them in slice order, so
 * every thread count gives the same result.
 *
 * Substitutions (documented, shared with the GPU so both agree bit for bit):
 *  - acos/atan2/sin/cos/asin/tan come from nbg_math.h instead of Go's math.
 *  - fragment positions come from the seeded generator of nbg_shared.h
 *    instead of the wall-clock-seeded math/rand (cmd/util/vectorutil.go:34).
 */
#include "nbg_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "../nbodygo_gb300/csrc/nbg_math.h"
#include "../nbodygo_gb300/csrc/nbg_shared.h"

/* The transcendentals of calcElasticCollision (cmd/body/collisioncalc.go:
 * 104-160).  The shipping oracle uses nbg_math.h, the functions the GPU uses,
 * so the two agree bit for bit.  Built with -DNBG_ORACLE_LIBM (as
 * libnbg_oracle_libm.so) it takes the platform libm's instead: a second
 * instrument that bounds how far that shared substitution can move a
 * trajectory, since Go's math package cannot run here. */
#ifdef NBG_ORACLE_LIBM
#define O_SIN sin
#define O_COS cos
#define O_TAN tan
#define O_ASIN asin
#define O_ACOS acos
#define O_ATAN2 atan2
#else
#define O_SIN nbg_sin
#define O_COS nbg_cos
#define O_TAN nbg_tan
#define O_ASIN nbg_asin
#define O_ACOS nbg_acos
#define O_ATAN2 nbg_atan2
#endif

/* ---- body record: cmd/body/body.go:26-52 -------------------------------- */

typedef struct ob_frag {
    double radius, new_radius, mass;
    int64_t fragments;
    double cx, cy, cz;
} ob_frag;

typedef struct ob_body {
    int64_t id;
    double x, y, z, vx, vy, vz, radius, mass;
    double frag_factor, frag_step;
    int32_t behavior;
    int is_sun, exists, telemetry, pinned;
    double r;
    int fragmenting;
    ob_frag frag;
    double fx, fy, fz;
    int collided;
} ob_body;

/* ---- events: cmd/body/event.go:18-111 ----------------------------------- */

enum { EV_COLLISION = 0, EV_SUBSUME = 1, EV_ADD = 2 };

typedef struct ob_event {
    int type;
    ob_body *b1, *b2;
} ob_event;

typedef struct ev_vec {
    ob_event *v;
    int64_t n, cap;
} ev_vec;

static void ev_push(ev_vec *q, int type, ob_body *b1, ob_body *b2)
{
    if (q->n == q->cap) {
        int64_t nc = q->cap ? q->cap * 2 : 64;
        q->v = (ob_event *)realloc(q->v, (size_t)nc * sizeof(ob_event));
        q->cap = nc;
    }
    q->v[q->n].type = type;
    q->v[q->n].b1 = b1;
    q->v[q->n].b2 = b2;
    q->n++;
}

typedef struct octree octree;

struct nbo_sim {
    ob_body **arr;
    int64_t n;
    int barnes_hut; /* forces from the octree (bc.Tree != nil) */
    octree *tree;
    ev_vec queue; /* arrival order */
    int64_t next_id;
    uint64_t seed;
    uint64_t cycle;
    nbg_event *last_ev;
    int64_t last_nev, last_evcap;
    nbg_step_info info;
};

static ob_body *body_new(void)
{
    ob_body *b = (ob_body *)calloc(1, sizeof(ob_body));
    b->r = 1.0;
    b->exists = 1;
    return b;
}

/* ---- calcForceFrom: body.go:214-225 ------------------------------------- */

static void calc_force_from(ob_body *b, const ob_body *o)
{
    double dx = o->x - b->x;
    double dy = o->y - b->y;
    double dz = o->z - b->z;
    double dist = sqrt(dx * dx + dy * dy + dz * dz);
    if (b->collided || dist > b->radius + o->radius) {
        double force = NBG_G * b->mass * o->mass / (dist * dist);
        b->fx += force * dx / dist;
        b->fy += force * dy / dist;
        b->fz += force * dz / dist;
    }
}

/* ---- Collided: body.go:192-208 ------------------------------------------ */

static int collided_with(const ob_body *b, const ob_body *o, double *dist_out)
{
    if (b->collided) {
        *dist_out = 0;
        return 0;
    }
    double dx = o->x - b->x;
    double dy = o->y - b->y;
    double dz = o->z - b->z;
    double dist = sqrt(dx * dx + dy * dy + dz * dz);
    if (dist > b->radius + o->radius) {
        *dist_out = 0;
        return 0;
    } else if (dist <= b->radius + o->radius) {
        *dist_out = dist;
        return 1;
    }
    *dist_out = 0;
    return 0;
}

/* ---- fragment: fragcalc.go:94-117 --------------------------------------- */

typedef struct slice_out {
    ev_vec ev;           /* collision / subsume / add events of the slice */
    ob_body **gone;      /* fragmenting bodies that finished this cycle */
    int64_t ngone, capgone;
} slice_out;

static void body_fragment(ob_body *b, const nbo_sim *s, slice_out *out)
{
    int cnt = 0;
    uint64_t key = nbg_frag_key(s->seed, b->id, s->cycle);
    while (b->frag.fragments > 0) {
        b->frag.fragments--;
        double px, py, pz;
        nbg_frag_point(key, cnt, b->frag.cx, b->frag.cy, b->frag.cz, b->frag.radius * .9,
                       &px, &py, &pz);
        ob_body *f = (ob_body *)calloc(1, sizeof(ob_body));
        f->id = -1; /* NextId() is called in canonical order after the compute phase */
        f->x = px;
        f->y = py;
        f->z = pz;
        f->vx = b->vx;
        f->vy = b->vy;
        f->vz = b->vz;
        f->mass = b->frag.mass;
        f->radius = b->frag.new_radius;
        f->frag_factor = 0;
        f->frag_step = 0;
        f->behavior = NBG_ELASTIC;
        f->is_sun = 0;
        f->exists = 1;
        f->telemetry = 0;
        f->pinned = 0;
        ev_push(&out->ev, EV_ADD, f, NULL);
        cnt++;
        if (cnt > NBG_MAX_FRAGS_PER_CYCLE) break;
    }
    if (b->frag.fragments <= 0) {
        /* b.Exists = false.  No other body's compute reads this flag in a way
         * that changes its result (fragmenting bodies are skipped by the force
         * pass either way and Collided does not look at Exists), so applying
         * it after the parallel phase is equivalent and race-free. */
        if (out->ngone == out->capgone) {
            out->capgone = out->capgone ? out->capgone * 2 : 16;
            out->gone = (ob_body **)realloc(out->gone, (size_t)out->capgone * sizeof(ob_body *));
        }
        out->gone[out->ngone++] = b;
    }
}

/* ---- Barnes-Hut: cmd/body/octree.go:97-325 --------------------------------
 * The octree the reference builds when Barnes-Hut is on, with its wiring
 * fixed: BuildTree (body_collection.go:298-300) creates the tree but never
 * calls Build, so the reference applies no gravity at all in that mode; here
 * Build runs at the start of every compute phase, as computation-runner.go:
 * 294-296 intends.  Bodies are inserted in array order with the incremental
 * centre-of-mass update, so the tree and every node value are the
 * reference's.  One guard is added: the reference subdivides without end
 * when two bodies share a position; here a leaf at depth BH_MAX_DEPTH keeps
 * every further body it receives (a bucket), and the force pass takes each
 * of its bodies with mass as a leaf. */
#define BH_THETA 0.3
#define BH_SOFTENING 1e-4
#define BH_MAX_DEPTH 64

typedef struct oct_node {
    double cx, cy, cz, half;
    double total_mass, cm_x, cm_y, cm_z;
    const ob_body *body;
    int64_t child[8]; /* -1: nil */
    const ob_body **extra; /* bucket at BH_MAX_DEPTH */
    int64_t nextra;
} oct_node;

struct octree {
    oct_node *pool;
    int64_t used, cap;
    int64_t root; /* -1: no tree */
};

static octree *octree_new(void)
{
    octree *t = (octree *)calloc(1, sizeof(octree));
    t->root = -1;
    return t;
}

static void octree_reset(octree *t)
{
    for (int64_t k = 0; k < t->used; k++) free(t->pool[k].extra);
    t->used = 0;
    t->root = -1;
}

static void octree_free(octree *t)
{
    if (!t) return;
    octree_reset(t);
    free(t->pool);
    free(t);
}

static int64_t oct_alloc(octree *t)
{
    if (t->used == t->cap) {
        t->cap = t->cap ? 2 * t->cap : 16384;
        t->pool = (oct_node *)realloc(t->pool, (size_t)t->cap * sizeof(oct_node));
    }
    oct_node *n = &t->pool[t->used];
    memset(n, 0, sizeof *n);
    for (int c = 0; c < 8; c++) n->child[c] = -1;
    return t->used++;
}

/* octantOf, octree.go:53-65 */
static int oct_octant(const oct_node *n, double x, double y, double z)
{
    int idx = 0;
    if (x >= n->cx) idx |= 1;
    if (y >= n->cy) idx |= 2;
    if (z >= n->cz) idx |= 4;
    return idx;
}

/* updateMass, octree.go:88-95 */
static void oct_update_mass(oct_node *n, double mass, double x, double y, double z)
{
    double newTotal = n->total_mass + mass;
    n->cm_x = (n->cm_x * n->total_mass + x * mass) / newTotal;
    n->cm_y = (n->cm_y * n->total_mass + y * mass) / newTotal;
    n->cm_z = (n->cm_z * n->total_mass + z * mass) / newTotal;
    n->total_mass = newTotal;
}

/* subdivide, octree.go:213-225 (childCenter, octree.go:67-85) */
static void oct_subdivide(octree *t, int64_t ni)
{
    for (int i = 0; i < 8; i++) {
        int64_t c = oct_alloc(t);
        oct_node *n = &t->pool[ni], *ch = &t->pool[c];
        double q = n->half / 2;
        ch->cx = (i & 1) ? n->cx + q : n->cx - q;
        ch->cy = (i & 2) ? n->cy + q : n->cy - q;
        ch->cz = (i & 4) ? n->cz + q : n->cz - q;
        ch->half = n->half / 2;
        n->child[i] = c;
    }
}

static void oct_insert(octree *t, int64_t ni, const ob_body *b, int depth);

/* insertIntoChild, octree.go:228-232 */
static void oct_insert_into_child(octree *t, int64_t ni, const ob_body *b, int depth)
{
    const oct_node *n = &t->pool[ni];
    oct_insert(t, n->child[oct_octant(n, b->x, b->y, b->z)], b, depth + 1);
}

/* insert, octree.go:191-211 */
static void oct_insert(octree *t, int64_t ni, const ob_body *b, int depth)
{
    oct_node *n = &t->pool[ni];
    oct_update_mass(n, b->mass, b->x, b->y, b->z);
    if (n->child[0] < 0) {
        if (n->body == NULL) {
            n->body = b;
            return;
        }
        if (depth >= BH_MAX_DEPTH) {
            n->extra = (const ob_body **)realloc(n->extra, (size_t)(n->nextra + 1) * sizeof(ob_body *));
            n->extra[n->nextra++] = b;
            return;
        }
        const ob_body *existing = n->body;
        n->body = NULL;
        oct_subdivide(t, ni);
        oct_insert_into_child(t, ni, existing, depth);
        oct_insert_into_child(t, ni, b, depth);
        return;
    }
    oct_insert_into_child(t, ni, b, depth);
}

/* Build, octree.go:136-188 */
static void octree_build(octree *t, ob_body *const *bodies, int64_t nb)
{
    octree_reset(t);
    if (nb == 0) return;
    double minX = NBG_DBL_MAX, minY = NBG_DBL_MAX, minZ = NBG_DBL_MAX;
    double maxX = -NBG_DBL_MAX, maxY = -NBG_DBL_MAX, maxZ = -NBG_DBL_MAX;
    int64_t count = 0;
    for (int64_t k = 0; k < nb; k++) {
        const ob_body *b = bodies[k];
        if (!b->exists || b->fragmenting) continue;
        if (b->x < minX) minX = b->x;
        if (b->y < minY) minY = b->y;
        if (b->z < minZ) minZ = b->z;
        if (b->x > maxX) maxX = b->x;
        if (b->y > maxY) maxY = b->y;
        if (b->z > maxZ) maxZ = b->z;
        count++;
    }
    if (count == 0) return;
    t->root = oct_alloc(t);
    oct_node *r = &t->pool[t->root];
    r->cx = (minX + maxX) / 2;
    r->cy = (minY + maxY) / 2;
    r->cz = (minZ + maxZ) / 2;
    r->half = nbg_go_max(maxX - minX, nbg_go_max(maxY - minY, maxZ - minZ)) / 2 * 1.05;
    for (int64_t k = 0; k < nb; k++)
        if (bodies[k]->exists && !bodies[k]->fragmenting) oct_insert(t, t->root, bodies[k], 0);
}

/* the force of a point mass (m at x, y, z) on b, as accumForce applies it
 * (octree.go:286-292) */
static void bh_apply(const ob_body *b, double m, double x, double y, double z, double *fx, double *fy, double *fz)
{
    double dx = x - b->x;
    double dy = y - b->y;
    double dz = z - b->z;
    double distSq = dx * dx + dy * dy + dz * dz + BH_SOFTENING * BH_SOFTENING;
    double dist = sqrt(distSq);
    double force = NBG_G * b->mass * m / distSq;
    *fx += force * dx / dist;
    *fy += force * dy / dist;
    *fz += force * dz / dist;
}

/* accumForce, octree.go:265-305 */
static void bh_accum(const octree *t, int64_t ni, const ob_body *b, double *fx, double *fy, double *fz)
{
    if (ni < 0) return;
    const oct_node *n = &t->pool[ni];
    if (n->total_mass == 0) return;
    double dx = n->cm_x - b->x;
    double dy = n->cm_y - b->y;
    double dz = n->cm_z - b->z;
    double distSq = dx * dx + dy * dy + dz * dz + BH_SOFTENING * BH_SOFTENING;
    double dist = sqrt(distSq);
    const int leaf = n->child[0] < 0;
    if (leaf || (2 * n->half / dist) < BH_THETA) {
        if (leaf && n->nextra > 0) {
            /* bucket: every member as a leaf of its own */
            const ob_body *o0 = n->body;
            if (o0 != b && o0->mass != 0)
                bh_apply(b, o0->mass, o0->x * o0->mass / o0->mass, o0->y * o0->mass / o0->mass,
                         o0->z * o0->mass / o0->mass, fx, fy, fz);
            for (int64_t k = 0; k < n->nextra; k++) {
                const ob_body *o = n->extra[k];
                if (o != b && o->mass != 0)
                    bh_apply(b, o->mass, o->x * o->mass / o->mass, o->y * o->mass / o->mass,
                             o->z * o->mass / o->mass, fx, fy, fz);
            }
            return;
        }
        if (leaf && n->body == b) return;
        double force = NBG_G * b->mass * n->total_mass / distSq;
        *fx += force * dx / dist;
        *fy += force * dy / dist;
        *fz += force * dz / dist;
        return;
    }
    for (int c = 0; c < 8; c++) {
        int64_t ci = n->child[c];
        if (ci >= 0 && t->pool[ci].total_mass > 0) bh_accum(t, ci, b, fx, fy, fz);
    }
}

/* CalcForce, octree.go:236-263: a sun sums every other body directly
 * (directForce, octree.go:310-325), every other body walks the tree */
static void bh_calc_force(const octree *t, const ob_body *b, ob_body *const *arr, int64_t n, double *fx, double *fy,
                          double *fz)
{
    *fx = *fy = *fz = 0;
    if (t->root < 0) return;
    if (b->is_sun) {
        for (int64_t k = 0; k < n; k++) {
            const ob_body *o = arr[k];
            if (o == b || !o->exists || o->fragmenting) continue;
            double dx = o->x - b->x;
            double dy = o->y - b->y;
            double dz = o->z - b->z;
            double distSq = dx * dx + dy * dy + dz * dz + BH_SOFTENING * BH_SOFTENING;
            double dist = sqrt(distSq);
            double force = NBG_G * b->mass * o->mass / distSq;
            *fx += force * dx / dist;
            *fy += force * dy / dist;
            *fz += force * dz / dist;
        }
        return;
    }
    bh_accum(t, t->root, b, fx, fy, fz);
}

/* ---- Compute: body.go:148-187 (bc.Tree == nil: direct sum; else the tree) -- */

static void body_compute(ob_body *b, const nbo_sim *s, slice_out *out)
{
    if (!b->exists) return;
    if (b->fragmenting) {
        body_fragment(b, s, out);
        return;
    }
    b->fx = 0;
    b->fy = 0;
    b->fz = 0;
    ob_body **arr = s->arr;
    int64_t n = s->n;
    if (s->barnes_hut) {
        bh_calc_force(s->tree, b, arr, n, &b->fx, &b->fy, &b->fz);
    } else {
        for (int64_t k = 0; k < n; k++) {
            const ob_body *o = arr[k];
            if (!o->exists || b->fragmenting) continue;
            if (b != o && o->exists && !o->fragmenting) calc_force_from(b, o);
        }
    }
    for (int64_t k = 0; k < n; k++) {
        ob_body *o = arr[k];
        double dist;
        if (collided_with(b, o, &dist)) {
            int bb = b->behavior, obh = o->behavior;
            if ((bb == NBG_ELASTIC || bb == NBG_FRAGMENT) && (obh == NBG_ELASTIC || obh == NBG_FRAGMENT)) {
                ev_push(&out->ev, EV_COLLISION, b, o);
            } else if (bb == NBG_SUBSUME || obh == NBG_SUBSUME) {
                if (b->radius > o->radius && dist <= b->radius)
                    ev_push(&out->ev, EV_SUBSUME, b, o);
                else if (o->radius > b->radius && dist <= o->radius)
                    ev_push(&out->ev, EV_SUBSUME, o, b);
            }
        }
    }
}

/* ---- elastic collision: collisioncalc.go:16-186 -------------------------- */

typedef struct coll_res {
    int collided;
    double vx1, vy1, vz1, vx2, vy2, vz2, vx_cm, vy_cm, vz_cm;
} coll_res;

static coll_res calc_elastic(const ob_body *b, const ob_body *o)
{
    coll_res res;
    memset(&res, 0, sizeof res);
    double r12, m21, d, v, theta2, phi2, st, ct, sp, cp, vx1r, vy1r, vz1r, fvz1r, thetav, phiv, dr,
        alpha, beta, sbeta, cbeta, a, dvz2, vx2r, vy2r, vz2r, x21, y21, z21, vx21, vy21, vz21,
        vx_cm, vy_cm, vz_cm;
    double m1 = b->mass, m2 = o->mass, r1 = b->radius, r2 = o->radius;
    double x1 = b->x, y1 = b->y, z1 = b->z;
    double x2 = o->x, y2 = o->y, z2 = o->z;
    double vx1 = b->vx, vy1 = b->vy, vz1 = b->vz;
    double vx2 = o->vx, vy2 = o->vy, vz2 = o->vz;

    r12 = r1 + r2;
    m21 = m2 / m1;
    x21 = x2 - x1;
    y21 = y2 - y1;
    z21 = z2 - z1;
    vx21 = vx2 - vx1;
    vy21 = vy2 - vy1;
    vz21 = vz2 - vz1;

    vx_cm = (m1 * vx1 + m2 * vx2) / (m1 + m2);
    vy_cm = (m1 * vy1 + m2 * vy2) / (m1 + m2);
    vz_cm = (m1 * vz1 + m2 * vz2) / (m1 + m2);

    d = sqrt(x21 * x21 + y21 * y21 + z21 * z21);
    v = sqrt(vx21 * vx21 + vy21 * vy21 + vz21 * vz21);

    if (v == 0) {
        res.collided = 0;
        return res;
    }
    x2 = x21;
    y2 = y21;
    z2 = z21;
    vx1 = -vx21;
    vy1 = -vy21;
    vz1 = -vz21;

    theta2 = O_ACOS(z2 / d);
    if (x2 == 0 && y2 == 0)
        phi2 = 0;
    else
        phi2 = O_ATAN2(y2, x2);
    st = O_SIN(theta2);
    ct = O_COS(theta2);
    sp = O_SIN(phi2);
    cp = O_COS(phi2);

    vx1r = ct * cp * vx1 + ct * sp * vy1 - st * vz1;
    vy1r = cp * vy1 - sp * vx1;
    vz1r = st * cp * vx1 + st * sp * vy1 + ct * vz1;
    fvz1r = vz1r / v;
    if (fvz1r > 1)
        fvz1r = 1;
    else if (fvz1r < -1)
        fvz1r = -1;
    thetav = O_ACOS(fvz1r);
    if (vx1r == 0 && vy1r == 0)
        phiv = 0;
    else
        phiv = O_ATAN2(vy1r, vx1r);

    dr = d * O_SIN(thetav) / r12;

    if (thetav > NBG_PIO2_HI || fabs(dr) > 1) {
        res.collided = 0;
        return res;
    }
    alpha = O_ASIN(-dr);
    beta = phiv;
    sbeta = O_SIN(beta);
    cbeta = O_COS(beta);

    a = O_TAN(thetav + alpha);
    dvz2 = 2 * (vz1r + a * (cbeta * vx1r + sbeta * vy1r)) / ((1 + a * a) * (1 + m21));

    vz2r = dvz2;
    vx2r = a * cbeta * dvz2;
    vy2r = a * sbeta * dvz2;
    vz1r = vz1r - m21 * vz2r;
    vx1r = vx1r - m21 * vx2r;
    vy1r = vy1r - m21 * vy2r;

    res.collided = 1;
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

static void do_elastic(ob_body *b, ob_body *o, const coll_res *r)
{
    b->vx = (r->vx1 - r->vx_cm) * b->r + r->vx_cm;
    b->vy = (r->vy1 - r->vy_cm) * b->r + r->vy_cm;
    b->vz = (r->vz1 - r->vz_cm) * b->r + r->vz_cm;
    o->vx = (r->vx2 - r->vx_cm) * b->r + r->vx_cm;
    o->vy = (r->vy2 - r->vy_cm) * b->r + r->vy_cm;
    o->vz = (r->vz2 - r->vz_cm) * b->r + r->vz_cm;
    b->collided = 1;
    o->collided = 1;
}

/* ---- fragmentation decision: fragcalc.go:24-85 --------------------------- */

static int should_fragment(const ob_body *b, const ob_body *o, const coll_res *r, double *tf, double *of)
{
    *tf = 0;
    *of = 0;
    if (!(b->behavior == NBG_FRAGMENT || o->behavior == NBG_FRAGMENT)) return 0;
    double vThis = b->vx + b->vy + b->vz;
    double dvThis = fabs(b->vx - ((r->vx1 - r->vx_cm) * b->r + r->vx_cm)) +
                    fabs(b->vy - ((r->vy1 - r->vy_cm) * b->r + r->vy_cm)) +
                    fabs(b->vz - ((r->vz1 - r->vz_cm) * b->r + r->vz_cm));
    double thisFactor = dvThis / fabs(vThis);
    double vOther = o->vx + o->vy + o->vz;
    double dvOther = fabs(o->vx - ((r->vx2 - r->vx_cm) * b->r + r->vx_cm)) +
                     fabs(o->vy - ((r->vy2 - r->vy_cm) * b->r + r->vy_cm)) +
                     fabs(o->vz - ((r->vz2 - r->vz_cm) * b->r + r->vz_cm));
    double otherFactor = dvOther / fabs(vOther);
    if ((b->behavior == NBG_FRAGMENT && thisFactor > b->frag_factor) ||
        (o->behavior == NBG_FRAGMENT && otherFactor > o->frag_factor)) {
        *tf = thisFactor;
        *of = otherFactor;
        return 1;
    }
    return 0;
}

/* Go's int(float64) for a value that is finite and within range truncates
 * toward zero.  For NaN amd64 yields math.MinInt64 and arm64 yields 0; either
 * way no fragment is emitted and the body is removed at its next Compute, so
 * NaN maps to 0 here. */
static int64_t go_int(double f)
{
    if (f != f) return 0;
    return (int64_t)f;
}

static void initiate_fragmentation(ob_body *b, double fragFactor)
{
    double fragDelta;
    if (b->frag_factor > 10)
        fragDelta = 10;
    else
        fragDelta = fragFactor - b->frag_factor;
    double fragments = nbg_go_min(fragDelta * b->frag_step, NBG_MAX_FRAGS);
    if (fragments <= 1) {
        b->behavior = NBG_FRAGMENT;
        return;
    }
    b->fragmenting = 1;
    /* newRadius = max(pow(x, 1/3), .1): Go evaluates the untyped constant 1/3
     * as integer division (0) and Pow(x, 0) == 1 for every x, so newRadius is
     * always 1. */
    double newRadius = 1.0;
    double newMass = b->mass / fragments;
    b->frag.radius = b->radius;
    b->frag.new_radius = newRadius;
    b->frag.mass = newMass;
    b->frag.fragments = go_int(fragments);
    b->frag.cx = b->x;
    b->frag.cy = b->y;
    b->frag.cz = b->z;
}

static void do_fragment(ob_body *b, ob_body *o, double tf, double of)
{
    if (b->behavior == NBG_FRAGMENT && tf > b->frag_factor) initiate_fragmentation(b, tf);
    if (o->behavior == NBG_FRAGMENT && of > o->frag_factor) initiate_fragmentation(o, of);
}

/* ---- ResolveCollision / ResolveSubsume: body.go:228-264 ------------------ */

static void resolve_collision(ob_body *b, ob_body *o)
{
    if (!b->exists || !o->exists) return;
    if (b->behavior == NBG_ELASTIC && (o->behavior == NBG_ELASTIC || o->behavior == NBG_FRAGMENT)) {
        coll_res r = calc_elastic(b, o);
        if (r.collided) {
            double tf, of;
            if (should_fragment(b, o, &r, &tf, &of))
                do_fragment(b, o, tf, of);
            else
                do_elastic(b, o, &r);
        }
    }
}

static void resolve_subsume(ob_body *b, ob_body *o)
{
    double thisMass = b->mass;
    double otherMass = o->mass;
    b->mass = thisMass + otherMass;
    o->mass = 0; /* SetNotExists, body.go:93-96 */
    o->exists = 0;
}

/* ---- the collection ------------------------------------------------------ */

nbo_sim *nbo_create(uint64_t seed)
{
    nbo_sim *s = (nbo_sim *)calloc(1, sizeof(nbo_sim));
    s->seed = seed;
    return s;
}

static void free_bodies(nbo_sim *s)
{
    for (int64_t k = 0; k < s->n; k++) free(s->arr[k]);
    free(s->arr);
    s->arr = NULL;
    s->n = 0;
    for (int64_t k = 0; k < s->queue.n; k++)
        if (s->queue.v[k].type == EV_ADD) free(s->queue.v[k].b1);
    s->queue.n = 0;
}

void nbo_destroy(nbo_sim *s)
{
    if (!s) return;
    octree_free(s->tree);
    free_bodies(s);
    free(s->queue.v);
    free(s->last_ev);
    free(s);
}

static void load_body(ob_body *b, const nbg_soa *in, int64_t k)
{
    b->id = in->id ? in->id[k] : -1;
    b->x = in->x[k];
    b->y = in->y[k];
    b->z = in->z[k];
    b->vx = in->vx[k];
    b->vy = in->vy[k];
    b->vz = in->vz[k];
    b->radius = in->radius[k];
    b->mass = in->mass[k];
    b->frag_factor = in->frag_factor ? in->frag_factor[k] : 0;
    b->frag_step = in->frag_step ? in->frag_step[k] : 0;
    b->behavior = in->collision ? in->collision[k] : NBG_ELASTIC;
    uint32_t f = in->flags ? in->flags[k] : NBG_F_EXISTS;
    b->exists = (f & NBG_F_EXISTS) != 0;
    b->is_sun = (f & NBG_F_IS_SUN) != 0;
    b->pinned = (f & NBG_F_PINNED) != 0;
    b->telemetry = (f & NBG_F_TELEMETRY) != 0;
    b->fragmenting = (f & NBG_F_FRAGMENTING) != 0;
    b->collided = (f & NBG_F_COLLIDED) != 0;
    b->r = in->r ? in->r[k] : 1.0;
    b->fx = in->fx ? in->fx[k] : 0;
    b->fy = in->fy ? in->fy[k] : 0;
    b->fz = in->fz ? in->fz[k] : 0;
    b->frag.radius = in->frag_radius ? in->frag_radius[k] : 0;
    b->frag.new_radius = in->frag_new_radius ? in->frag_new_radius[k] : 0;
    b->frag.mass = in->frag_mass ? in->frag_mass[k] : 0;
    b->frag.fragments = in->frag_fragments ? in->frag_fragments[k] : 0;
    b->frag.cx = in->frag_cx ? in->frag_cx[k] : 0;
    b->frag.cy = in->frag_cy ? in->frag_cy[k] : 0;
    b->frag.cz = in->frag_cz ? in->frag_cz[k] : 0;
}

int nbo_set_bodies(nbo_sim *s, const nbg_soa *in, int64_t n)
{
    if (!s || n < 0 || (n > 0 && !in)) return NBG_E_ARG;
    free_bodies(s);
    s->arr = (ob_body **)malloc((size_t)(n > 0 ? n : 1) * sizeof(ob_body *));
    for (int64_t k = 0; k < n; k++) {
        ob_body *b = body_new();
        load_body(b, in, k);
        s->arr[k] = b;
    }
    s->n = n;
    return NBG_OK;
}

int64_t nbo_count(const nbo_sim *s) { return s->n; }

void nbo_set_barnes_hut(nbo_sim *s, int on)
{
    s->barnes_hut = on != 0;
    if (s->barnes_hut && !s->tree) s->tree = octree_new();
}
void nbo_set_next_id(nbo_sim *s, int64_t id) { s->next_id = id; }
int64_t nbo_get_next_id(const nbo_sim *s) { return s->next_id; }
void nbo_set_cycle(nbo_sim *s, uint64_t cycle) { s->cycle = cycle; }

int nbo_get_state(const nbo_sim *s, nbg_soa *o, int64_t cap)
{
    int64_t n = s->n < cap ? s->n : cap;
    for (int64_t k = 0; k < n; k++) {
        const ob_body *b = s->arr[k];
        if (o->id) o->id[k] = b->id;
        if (o->x) o->x[k] = b->x;
        if (o->y) o->y[k] = b->y;
        if (o->z) o->z[k] = b->z;
        if (o->vx) o->vx[k] = b->vx;
        if (o->vy) o->vy[k] = b->vy;
        if (o->vz) o->vz[k] = b->vz;
        if (o->radius) o->radius[k] = b->radius;
        if (o->mass) o->mass[k] = b->mass;
        if (o->frag_factor) o->frag_factor[k] = b->frag_factor;
        if (o->frag_step) o->frag_step[k] = b->frag_step;
        if (o->collision) o->collision[k] = b->behavior;
        if (o->flags)
            o->flags[k] = (b->exists ? NBG_F_EXISTS : 0u) | (b->is_sun ? NBG_F_IS_SUN : 0u) |
                          (b->pinned ? NBG_F_PINNED : 0u) | (b->telemetry ? NBG_F_TELEMETRY : 0u) |
                          (b->fragmenting ? NBG_F_FRAGMENTING : 0u) | (b->collided ? NBG_F_COLLIDED : 0u);
        if (o->r) o->r[k] = b->r;
        if (o->fx) o->fx[k] = b->fx;
        if (o->fy) o->fy[k] = b->fy;
        if (o->fz) o->fz[k] = b->fz;
        if (o->frag_radius) o->frag_radius[k] = b->frag.radius;
        if (o->frag_new_radius) o->frag_new_radius[k] = b->frag.new_radius;
        if (o->frag_mass) o->frag_mass[k] = b->frag.mass;
        if (o->frag_fragments) o->frag_fragments[k] = b->frag.fragments;
        if (o->frag_cx) o->frag_cx[k] = b->frag.cx;
        if (o->frag_cy) o->frag_cy[k] = b->frag.cy;
        if (o->frag_cz) o->frag_cz[k] = b->frag.cz;
    }
    return NBG_OK;
}

int nbo_add_bodies(nbo_sim *s, const nbg_soa *in, int64_t n, int64_t *ids_out)
{
    if (!s || n < 0 || (n > 0 && !in)) return NBG_E_ARG;
    for (int64_t k = 0; k < n; k++) {
        ob_body *b = body_new();
        load_body(b, in, k);
        if (!in->id || in->id[k] < 0) b->id = s->next_id++;
        if (ids_out) ids_out[k] = b->id;
        ev_push(&s->queue, EV_ADD, b, NULL);
    }
    return NBG_OK;
}

/* processDeletes: computation-runner.go:176-216.  The `return` inside the
 * IterateOnce closure (:206-208) only ends that body's callback, so the walk
 * continues over the whole array and may remove more than `count` bodies. */
int64_t nbo_remove_bodies(nbo_sim *s, int64_t count)
{
    int64_t removed = 0;
    if (count == -1) {
        for (int64_t k = 0; k < s->n; k++) {
            ob_body *b = s->arr[k];
            if (b->exists) {
                b->mass = 0;
                b->exists = 0;
                removed++;
            }
        }
        return removed;
    }
    if (count <= 0) return -1;
    int64_t step = count > s->n ? 1 : s->n / count;
    int64_t iter = 0;
    int should = 0;
    for (int64_t k = 0; k < s->n; k++) {
        ob_body *b = s->arr[k];
        if (iter % step == 0) should = 1;
        iter++;
        if (should && !b->pinned && b->exists) {
            b->mass = 0;
            b->exists = 0;
            should = 0;
            removed++;
        }
    }
    return removed;
}

int32_t nbo_apply_edit(nbo_sim *s, const nbg_edit *e)
{
    int32_t found = 0;
    for (int64_t k = 0; k < s->n; k++) {
        ob_body *b = s->arr[k];
        if (b->id != e->id) continue;
        found++;
        uint32_t m = e->mask;
        if (m & NBG_M_X) b->x = e->x;
        if (m & NBG_M_Y) b->y = e->y;
        if (m & NBG_M_Z) b->z = e->z;
        if (m & NBG_M_VX) b->vx = e->vx;
        if (m & NBG_M_VY) b->vy = e->vy;
        if (m & NBG_M_VZ) b->vz = e->vz;
        if (m & NBG_M_MASS) b->mass = e->mass;
        if (m & NBG_M_RADIUS) b->radius = e->radius;
        if (m & NBG_M_FRAG_FACTOR) b->frag_factor = e->frag_factor;
        if (m & NBG_M_FRAG_STEP) b->frag_step = e->frag_step;
        if (m & NBG_M_COLLISION) b->behavior = e->collision;
        if (m & NBG_M_TELEMETRY) b->telemetry = e->telemetry != 0;
        if (m & NBG_M_EXISTS) b->exists = e->exists != 0;
    }
    return found;
}

int nbo_enqueue_event(nbo_sim *s, int type, int64_t i, int64_t j)
{
    if (i < 0 || j < 0 || i >= s->n || j >= s->n) return NBG_E_ARG;
    if (type != EV_COLLISION && type != EV_SUBSUME) return NBG_E_ARG;
    ev_push(&s->queue, type, s->arr[i], s->arr[j]);
    return NBG_OK;
}

/* ---- compute phase with the worker-pool slicing ------------------------- */

typedef struct worker_arg {
    nbo_sim *s;
    slice_out *outs;
    int64_t nslices, size;
    int tid, nthreads;
} worker_arg;

static void *compute_worker(void *p)
{
    worker_arg *w = (worker_arg *)p;
    for (int64_t sl = w->tid; sl < w->nslices; sl += w->nthreads) {
        int64_t off = sl * w->size;
        int64_t end = off + w->size;
        if (end > w->s->n) end = w->s->n;
        for (int64_t k = off; k < end; k++) body_compute(w->s->arr[k], w->s, &w->outs[sl]);
    }
    return NULL;
}

void nbo_phase_compute(nbo_sim *s, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    if (s->barnes_hut) octree_build(s->tree, s->arr, s->n); /* computation-runner.go:294-296 */
    int64_t max = s->n;
    int64_t size = max / nthreads;
    if (max < 100) size = max;
    if (size < 1) size = 1;
    int64_t nslices = max > 0 ? (max + size - 1) / size : 0;
    slice_out *outs = (slice_out *)calloc((size_t)(nslices > 0 ? nslices : 1), sizeof(slice_out));
    if (nthreads == 1 || nslices <= 1) {
        for (int64_t sl = 0; sl < nslices; sl++) {
            int64_t off = sl * size, end = off + size > max ? max : off + size;
            for (int64_t k = off; k < end; k++) body_compute(s->arr[k], s, &outs[sl]);
        }
    } else {
        int nt = nthreads < nslices ? nthreads : (int)nslices;
        pthread_t *th = (pthread_t *)malloc((size_t)nt * sizeof(pthread_t));
        worker_arg *wa = (worker_arg *)malloc((size_t)nt * sizeof(worker_arg));
        for (int t = 0; t < nt; t++) {
            wa[t].s = s;
            wa[t].outs = outs;
            wa[t].nslices = nslices;
            wa[t].size = size;
            wa[t].tid = t;
            wa[t].nthreads = nt;
            pthread_create(&th[t], NULL, compute_worker, &wa[t]);
        }
        for (int t = 0; t < nt; t++) pthread_join(th[t], NULL);
        free(th);
        free(wa);
    }
    /* concatenate in slice order = single-worker arrival order; NextId for
     * fragments in that order */
    for (int64_t sl = 0; sl < nslices; sl++) {
        for (int64_t k = 0; k < outs[sl].ev.n; k++) {
            ob_event *e = &outs[sl].ev.v[k];
            if (e->type == EV_ADD) {
                e->b1->id = s->next_id++;
                s->info.fragments_emitted++;
            }
            ev_push(&s->queue, e->type, e->b1, e->b2);
        }
        for (int64_t k = 0; k < outs[sl].ngone; k++) outs[sl].gone[k]->exists = 0;
        free(outs[sl].ev.v);
        free(outs[sl].gone);
    }
    free(outs);
}

/* ---- ProcessMods: body_collection.go:212-233 ----------------------------- */

void nbo_phase_process_mods(nbo_sim *s)
{
    s->last_nev = 0;
    for (int64_t k = s->queue.n - 1; k >= 0; k--) {
        ob_event *e = &s->queue.v[k];
        if (e->type == EV_ADD) continue;
        if (e->b1 != e->b2) {
            if (s->last_nev == s->last_evcap) {
                s->last_evcap = s->last_evcap ? s->last_evcap * 2 : 64;
                s->last_ev = (nbg_event *)realloc(s->last_ev, (size_t)s->last_evcap * sizeof(nbg_event));
            }
            nbg_event *r = &s->last_ev[s->last_nev++];
            r->id1 = e->b1->id;
            r->id2 = e->b2->id;
            r->type = e->type == EV_COLLISION ? NBG_EV_COLLISION : NBG_EV_SUBSUME;
            r->pad = 0;
            s->info.events++;
        }
        if (e->type == EV_COLLISION)
            resolve_collision(e->b1, e->b2);
        else
            resolve_subsume(e->b1, e->b2);
    }
    /* handled events leave the list; adds stay for Cycle */
    int64_t w = 0;
    for (int64_t k = 0; k < s->queue.n; k++)
        if (s->queue.v[k].type == EV_ADD) s->queue.v[w++] = s->queue.v[k];
    s->queue.n = w;
}

/* ---- Update: body.go:114-139 -------------------------------------------- */

void nbo_phase_update(nbo_sim *s, double dt, double R)
{
    for (int64_t k = 0; k < s->n; k++) {
        ob_body *b = s->arr[k];
        if (!b->exists) continue;
        if (!b->collided) {
            b->vx += dt * b->fx / b->mass;
            b->vy += dt * b->fy / b->mass;
            b->vz += dt * b->fz / b->mass;
        }
        b->x += dt * b->vx;
        b->y += dt * b->vy;
        b->z += dt * b->vz;
        b->collided = 0;
        b->r = R;
        if (isnan(b->x) || isnan(b->y) || isnan(b->z)) {
            b->exists = 0;
            s->info.nan_removed++;
        }
    }
}

/* ---- Cycle: body_collection.go:253-296 ---------------------------------- */

void nbo_phase_cycle(nbo_sim *s, double R)
{
    int64_t cnt = 0;
    for (int64_t k = 0; k < s->n; k++)
        if (s->arr[k]->exists) cnt++;
    int64_t nadds = 0;
    for (int64_t k = 0; k < s->queue.n; k++)
        if (s->queue.v[k].type == EV_ADD) nadds++;
    ob_body **arr = (ob_body **)malloc((size_t)(cnt + nadds > 0 ? cnt + nadds : 1) * sizeof(ob_body *));
    int64_t j = 0;
    for (int64_t k = 0; k < s->n; k++) {
        if (s->arr[k]->exists)
            arr[j++] = s->arr[k];
        else
            free(s->arr[k]);
    }
    s->info.removed += s->n - cnt;
    for (int64_t k = s->queue.n - 1; k >= 0; k--) {
        if (s->queue.v[k].type == EV_ADD) {
            ob_body *b = s->queue.v[k].b1;
            b->r = R;
            arr[j++] = b;
        }
    }
    free(s->arr);
    s->arr = arr;
    s->n = j;
    s->queue.n = 0; /* events.Init() */
}

int nbo_step(nbo_sim *s, double dt, double R, int nsteps, int nthreads)
{
    memset(&s->info, 0, sizeof s->info);
    for (int k = 0; k < nsteps; k++) {
        s->info.interactions += s->n * (s->n > 0 ? s->n - 1 : 0);
        nbo_phase_compute(s, nthreads);
        nbo_phase_process_mods(s);
        nbo_phase_update(s, dt, R);
        nbo_phase_cycle(s, R);
        s->cycle++;
        s->info.steps_done++;
    }
    s->info.n_bodies = s->n;
    s->info.next_id = s->next_id;
    return NBG_OK;
}

int64_t nbo_last_events(const nbo_sim *s, nbg_event *out, int64_t cap)
{
    int64_t n = s->last_nev < cap ? s->last_nev : cap;
    if (out && n > 0) memcpy(out, s->last_ev, (size_t)n * sizeof(nbg_event));
    return s->last_nev;
}

void nbo_last_info(const nbo_sim *s, nbg_step_info *info) { *info = s->info; }

/* ---- force pass only ------------------------------------------------------ */

typedef struct force_arg {
    const nbo_sim *s;
    double *fx, *fy, *fz;
    int64_t lo, hi;
} force_arg;

static void *force_worker(void *p)
{
    force_arg *a = (force_arg *)p;
    const nbo_sim *s = a->s;
    for (int64_t k = a->lo; k < a->hi; k++) {
        ob_body tmp = *s->arr[k];
        if (s->barnes_hut) {
            if (tmp.exists && !tmp.fragmenting)
                bh_calc_force(s->tree, s->arr[k], s->arr, s->n, &tmp.fx, &tmp.fy, &tmp.fz);
        } else if (tmp.exists && !tmp.fragmenting) {
            tmp.fx = tmp.fy = tmp.fz = 0;
            for (int64_t q = 0; q < s->n; q++) {
                const ob_body *o = s->arr[q];
                if (!o->exists) continue;
                if (q != k && !o->fragmenting) calc_force_from(&tmp, o);
            }
        }
        a->fx[k] = tmp.fx;
        a->fy[k] = tmp.fy;
        a->fz[k] = tmp.fz;
    }
    return NULL;
}

int nbo_forces(const nbo_sim *s, double *fx, double *fy, double *fz, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    if (s->barnes_hut) octree_build(s->tree, s->arr, s->n);
    pthread_t *th = (pthread_t *)malloc((size_t)nthreads * sizeof(pthread_t));
    force_arg *fa = (force_arg *)malloc((size_t)nthreads * sizeof(force_arg));
    int64_t per = (s->n + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; t++) {
        fa[t].s = s;
        fa[t].fx = fx;
        fa[t].fy = fy;
        fa[t].fz = fz;
        fa[t].lo = t * per < s->n ? t * per : s->n;
        fa[t].hi = (t + 1) * per < s->n ? (t + 1) * per : s->n;
        pthread_create(&th[t], NULL, force_worker, &fa[t]);
    }
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    free(th);
    free(fa);
    return NBG_OK;
}

/* ---- math self-test hook ---------------------------------------------------- */

double nbo_math_eval(int which, double a, double b)
{
    switch (which) {
    case 0: return nbg_sin(a);
    case 1: return nbg_cos(a);
    case 2: return nbg_tan(a);
    case 3: return nbg_asin(a);
    case 4: return nbg_acos(a);
    case 5: return nbg_atan(a);
    case 6: return nbg_atan2(a, b);
    case 7: return nbg_go_min(a, b);
    default: return nbg_nan();
    }
}

/* Fragment position generator, exposed so tests can pin it. */
void nbo_frag_point(uint64_t seed, int64_t parent_id, uint64_t cycle, int cnt, double cx, double cy, double cz,
                    double radius, double *out3)
{
    uint64_t key = nbg_frag_key(seed, parent_id, cycle);
    nbg_frag_point(key, cnt, cx, cy, cz, radius, &out3[0], &out3[1], &out3[2]);
}

/* FP64 force of the force pass for the bodies listed in idx (k < m), as
 * nbo_forces computes it; for checking large collections on a sample. */
int nbo_forces_subset(const nbo_sim *s, const int64_t *idx, int64_t m, double *fx, double *fy, double *fz)
{
    for (int64_t q = 0; q < m; q++) {
        int64_t k = idx[q];
        if (k < 0 || k >= s->n) return NBG_E_ARG;
        ob_body tmp = *s->arr[k];
        if (tmp.exists && !tmp.fragmenting) {
            tmp.fx = tmp.fy = tmp.fz = 0;
            for (int64_t j = 0; j < s->n; j++) {
                const ob_body *o = s->arr[j];
                if (!o->exists) continue;
                if (j != k && !o->fragmenting) calc_force_from(&tmp, o);
            }
        }
        fx[q] = tmp.fx;
        fy[q] = tmp.fy;
        fz[q] = tmp.fz;
    }
    return NBG_OK;
}
