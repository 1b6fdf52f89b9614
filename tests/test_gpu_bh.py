"""Barnes-Hut force pass (cmd/body/octree.go, with BuildTree's missing Build
call made) on the GPU against the oracle's restatement, through the C ABI.

The GPU builds the reference's tree (same nodes, same opening decisions) but
sums each node's centre of mass as sum(m x) / sum(m) rather than by the
reference's running update, and a sun's direct sum as a parallel reduction;
both differ in the last bits only, so forces agree to 1e-12 relative and
whole cycles keep identical event lists."""
import numpy as np
import pytest

from nbodygo_gb300 import _abi as A
from nbodygo_gb300 import workloads as W
from nbodygo_gb300.api import Simulation
from oracle.oracle import OracleSim

from helpers import assert_events_identical, assert_states_identical
from test_gpu_plain_parity import dense_cluster

pytestmark = pytest.mark.gpu
FORCE_RTOL = 1e-12


def bh_pair(bodies, precision="fp64", seed=123):
    sim = Simulation(precision, seed=seed)
    sim.set_option(A.OPT_BARNES_HUT, 1)
    sim.set_bodies(bodies)
    ora = OracleSim(seed=seed, threads=8)
    ora.set_barnes_hut(True)
    ora.set_bodies(bodies)
    return sim, ora


def force_error(got, exp):
    g, e = np.stack(got, 1), np.stack(exp, 1)
    mag = np.linalg.norm(e, axis=1)
    err = np.linalg.norm(g - e, axis=1)
    ok = mag > 0
    assert np.all(err[~ok] == 0)
    return float(np.max(err[ok] / mag[ok])) if ok.any() else 0.0


def with_sun(b, k=0):
    b = {f: np.array(v) for f, v in b.items()}
    b["flags"][k] |= A.F_IS_SUN
    return b


@pytest.mark.parametrize("name,bodies", [
    ("plummer", lambda: W.plummer(3000, seed=7)),
    ("disk_with_sun", lambda: with_sun(W.disk(1500))),
    ("uniform", lambda: W.uniform_ball(2000, R=200.0)),
])
def test_bh_forces_match_oracle(name, bodies):
    b = bodies()
    sim, ora = bh_pair(b)
    got = sim.force_pass()
    exp = ora.forces()
    assert force_error(got, exp) <= FORCE_RTOL, name


def test_bh_forces_differ_from_direct_sum_by_the_approximation_only():
    b = W.plummer(3000, seed=8)
    sim, _ = bh_pair(b)
    bh = np.stack(sim.force_pass(), 1)
    direct = Simulation("fp64")
    direct.set_bodies(b)
    ds = np.stack(direct.force_pass(), 1)
    rel = np.linalg.norm(bh - ds) / np.linalg.norm(ds)
    assert 1e-6 < rel < 5e-3  # theta = 0.3 plus softening, not zero gravity


def test_bh_massless_bodies_keep_the_reference_nan_centre_rule():
    """A node whose first body (array order) is massless has the reference's
    NaN running centre and is always opened."""
    b = W.plummer(800, seed=9)
    b["mass"][0] = 0.0
    b["mass"][5] = 0.0
    b["mass"][100:110] = 0.0
    sim, ora = bh_pair(b)
    assert force_error(sim.force_pass(), ora.forces()) <= FORCE_RTOL


def test_bh_cycles_track_the_oracle_with_collisions():
    """Dense cluster, every behaviour: the tree query finds exactly the
    collisions of the O(N^2) pass, cycle after cycle."""
    b = dense_cluster(400, seed=31)
    sim, ora = bh_pair(b)
    sim.apply_edits([dict(id=int(b["id"][3]), mask=A.M_EXISTS, exists=0)])
    ora.apply_edits([dict(id=int(b["id"][3]), mask=A.M_EXISTS, exists=0)])
    for c in range(12):
        gi = sim.step(0.05, 0.9, 1)
        oi = ora.step(0.05, 0.9, 1)
        assert_events_identical(sim.events(), ora.events(), f"cycle {c}")
        for k in ("n_bodies", "events", "fragments_emitted", "removed", "next_id"):
            assert gi[k] == oi[k], f"cycle {c}: {k} {gi[k]} != {oi[k]}"
        gs, os_ = sim.state(), ora.state()
        assert np.array_equal(gs["id"], os_["id"])
        assert np.array_equal(gs["flags"], os_["flags"])
        for f in ("x", "y", "z", "vx", "vy", "vz", "mass"):
            d = np.abs(gs[f] - os_[f])
            scale = np.maximum(np.abs(os_[f]), 1e-300)
            assert np.all((d <= 1e-9 * scale) | (d <= 1e-12)), f"cycle {c}: {f}"


def test_bh_step_with_a_graph_equals_single_cycles():
    b = W.plummer(2048, seed=11)
    s1 = Simulation("fp64")
    s1.set_option(A.OPT_BARNES_HUT, 1)
    s1.set_bodies(b)
    s1.step(0.01, 1.0, 6)
    s2 = Simulation("fp64")
    s2.set_option(A.OPT_BARNES_HUT, 1)
    s2.set_option(A.OPT_GRAPH, 0)
    s2.set_bodies(b)
    for _ in range(6):
        s2.step(0.01, 1.0, 1)
    a, c = s1.state(), s2.state()
    for f in ("x", "y", "z", "vx", "vy", "vz"):
        assert np.array_equal(a[f].view(np.uint64), c[f].view(np.uint64)), f


def batched_bh_sets():
    return [
        dense_cluster(300, seed=51),                               # collisions of every behaviour
        {k: np.asarray(v)[:0] for k, v in W.plummer(8, seed=1).items()},  # an empty collection
        with_sun(W.disk(n=400, seed=52)),                          # a sun: summed directly
        W.plummer(n=1500, seed=53, radius_range=(0.3, 1.5)),
        dense_cluster(1, seed=54),                                 # a single body
        W.uniform_ball(n=700, seed=55, R=60.0, radius=0.8, behavior=A.ELASTIC),
    ]


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_batched_bh_equals_each_collection_alone(prec):
    """One tree per collection: every collection of a batched Barnes-Hut
    context gets the tree, walk groups, sun sums and collision query it gets
    alone, so its forces and its whole cycles are bit-identical to a context
    holding that collection only (fragment ids aside: a batch draws them from
    one counter)."""
    from test_gpu_batch import split_state

    sets = batched_bh_sets()
    batch = Simulation(prec, seed=8)
    batch.set_option(A.OPT_BARNES_HUT, 1)
    batch.set_collections(sets)
    alone = []
    for b in sets:
        s = Simulation(prec, seed=8)
        s.set_option(A.OPT_BARNES_HUT, 1)
        s.set_bodies(b)
        alone.append(s)
    f = np.array(batch.force_pass())
    o = 0
    for q, (s, b) in enumerate(zip(alone, sets)):
        k = len(b["x"])
        if k:
            g = np.array(s.force_pass())
            assert np.array_equal(f[:, o:o + k].view(np.uint64), g.view(np.uint64)), f"collection {q}"
        o += k
    for c in range(6):
        batch.step(0.05, 0.9, 1)
        for s in alone:
            s.step(0.05, 0.9, 1)
        counts = batch.sim_counts()
        assert list(counts) == [s.count() for s in alone], f"cycle {c}"
        for q, (s, got) in enumerate(zip(alone, split_state(batch.state(), counts))):
            if counts[q]:
                assert_states_identical(got, s.state(), fields=[k for k in got if k != "id"],
                                        where=f"{prec} cycle {c} collection {q}")
    batch.close()
    for s in alone:
        s.close()


@pytest.mark.parametrize("name,bodies", [
    ("plummer", lambda: W.plummer(3000, seed=7)),
    ("disk_with_sun", lambda: with_sun(W.disk(1500))),
    ("uniform", lambda: W.uniform_ball(2000, R=200.0)),
])
def test_mixed_bh_walk_stays_close_to_the_fp64_tree(name, bodies):
    """The mixed walk: FP32 terms on the same tree.  Its error against the
    FP64 tree is far below the tree's own approximation (~1e-3); a body
    whose opening test flips at theta may differ by that approximation."""
    b = bodies()
    sim, ora = bh_pair(b, precision="mixed")
    g = np.stack(sim.force_pass(), 1)
    e = np.stack(ora.forces(), 1)
    rel = np.linalg.norm(g - e) / np.linalg.norm(e)
    mag = np.linalg.norm(e, axis=1)
    per = np.linalg.norm(g - e, axis=1)[mag > 0] / mag[mag > 0]
    assert rel <= 1e-5, (name, rel)
    assert np.median(per) <= 1e-6, name
    assert np.max(per) <= 1e-2, name


def test_mixed_bh_first_cycle_events_are_exact():
    """Collisions come from the FP64 range query in both precisions."""
    b = dense_cluster(400, seed=33)
    sim, ora = bh_pair(b, precision="mixed")
    sim.step(0.05, 0.9, 1)
    ora.step(0.05, 0.9, 1)
    assert_events_identical(sim.events(), ora.events(), "cycle 0")


def test_every_mixed_walk_shape_gives_the_same_forces():
    """The walk shapes differ in the CTAs per SM their registers are capped
    for, not in arithmetic: each group's terms, order and folds are fixed."""
    b = W.plummer(n=5000, seed=61, radius_range=(0.3, 1.5))
    out = []
    for shape in range(3):
        with Simulation("mixed") as s:
            s.set_option(A.OPT_BARNES_HUT, 1)
            s.set_option(A.OPT_BH_SHAPE, shape)
            s.set_bodies(b)
            out.append(np.array(s.force_pass()))
    for shape, f in enumerate(out[1:], 1):
        assert np.array_equal(f.view(np.uint64), out[0].view(np.uint64)), f"shape {shape}"
