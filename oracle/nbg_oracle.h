/*
 * nbg_oracle.h - CPU oracle of the nbodygo compute cycle.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's
 * Go code for the direct-sum cycle, used by the tests as the checker and by
 * bench.py as the timed CPU baseline.  The product (libnbgpu.so) never links,
 * loads or calls it.
 *
 * Parity pin: the reference ships no numeric golden vectors; the oracle is
 * checked against every assertion of the reference's own tests for this path
 * (TestWpCompute, TestCollide, TestSubsume, TestRemove, TestAdds, TestMod) and
 * against an independent pure-Python restatement (tests/golden).
 */
#ifndef NBG_ORACLE_H
#define NBG_ORACLE_H

#include <stdint.h>
#include "../include/nbgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct nbo_sim nbo_sim;

nbo_sim *nbo_create(uint64_t seed);
void nbo_destroy(nbo_sim *s);
int nbo_set_bodies(nbo_sim *s, const nbg_soa *in, int64_t n);
int64_t nbo_count(const nbo_sim *s);
int nbo_get_state(const nbo_sim *s, nbg_soa *out, int64_t cap);
void nbo_set_next_id(nbo_sim *s, int64_t id);
int64_t nbo_get_next_id(const nbo_sim *s);
void nbo_set_cycle(nbo_sim *s, uint64_t cycle);

/* Barnes-Hut forces (cmd/body/octree.go, with BuildTree's missing Build call
 * made): the tree is rebuilt at the start of every compute phase. */
void nbo_set_barnes_hut(nbo_sim *s, int on);

/* Enqueue(NewAdd(b)); ids taken from the counter when id is NULL or < 0. */
int nbo_add_bodies(nbo_sim *s, const nbg_soa *in, int64_t n, int64_t *ids_out);
/* processDeletes (computation-runner.go:176-216). */
int64_t nbo_remove_bodies(nbo_sim *s, int64_t count);
/* ModBody by id with already-parsed values. */
int32_t nbo_apply_edit(nbo_sim *s, const nbg_edit *e);

/* Whole cycles: compute (nthreads workers, slices as computation-runner.go:284-305),
 * ProcessMods, Update, Cycle. */
int nbo_step(nbo_sim *s, double dt, double R, int nsteps, int nthreads);

/* Individual phases, for tests that mirror the reference's unit tests. */
void nbo_phase_compute(nbo_sim *s, int nthreads);
void nbo_phase_process_mods(nbo_sim *s);
void nbo_phase_update(nbo_sim *s, double dt, double R);
void nbo_phase_cycle(nbo_sim *s, double R);
/* bc.Enqueue(newCollision(arr[i], arr[j])) / newSubsume(arr[i], arr[j]). */
int nbo_enqueue_event(nbo_sim *s, int type, int64_t i, int64_t j);

/* Events handled by the last ProcessMods in handling order, self events
 * excluded. Returns the count (may exceed cap). */
int64_t nbo_last_events(const nbo_sim *s, nbg_event *out, int64_t cap);
/* Statistics of the last nbo_step call. */
void nbo_last_info(const nbo_sim *s, nbg_step_info *info);

/* FP64 force of the force pass for every live body, without side effects. */
int nbo_forces(const nbo_sim *s, double *fx, double *fy, double *fz, int nthreads);

/* Force pass for a sample of bodies. */
int nbo_forces_subset(const nbo_sim *s, const int64_t *idx, int64_t m, double *fx, double *fy, double *fz);

/* Test hooks: the shared FP64 functions (0 sin, 1 cos, 2 tan, 3 asin,
 * 4 acos, 5 atan, 6 atan2(a, b), 7 Go's math.Min) and the fragment-position
 * generator. */
double nbo_math_eval(int which, double a, double b);
void nbo_frag_point(uint64_t seed, int64_t parent_id, uint64_t cycle, int cnt, double cx, double cy, double cz,
                    double radius, double *out3);

#ifdef __cplusplus
}
#endif

#endif
