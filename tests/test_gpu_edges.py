"""Edge cases of the collection on the GPU, through the C ABI: an empty
collection, a single body, and a collection that merges down to one body,
in both forms and with the Barnes-Hut force pass; the plain form against the
oracle, bit for bit."""
import numpy as np
import pytest

from nbodygo_gb300 import _abi as A
from nbodygo_gb300 import workloads as W
from nbodygo_gb300.api import NbgError, Simulation
from oracle.oracle import OracleSim

from helpers import assert_states_identical, body_set

pytestmark = pytest.mark.gpu

FORMS = [("fp64", False), ("mixed", False), ("fp64", True), ("mixed", True)]


def make(prec, bh, bodies):
    sim = Simulation(prec, seed=7)
    if bh:
        sim.set_option(A.OPT_BARNES_HUT, 1)
    sim.set_bodies(bodies)
    return sim


@pytest.mark.parametrize("prec,bh", FORMS)
def test_empty_collection_steps_and_accepts_adds(prec, bh):
    sim = make(prec, bh, body_set([]))
    info = sim.step(0.01, 1.0, 3)
    assert info["steps_done"] == 3 and info["n_bodies"] == 0 and info["interactions"] == 0
    assert len(sim.state()["x"]) == 0
    sim.force_pass()
    ids = sim.add_bodies(body_set([dict(x=1.0, mass=1e10, radius=0.5), dict(x=-1.0, mass=1e10, radius=0.5)]))
    assert len(ids) == 2
    info = sim.step(0.01, 1.0, 2)
    assert info["n_bodies"] == 2


@pytest.mark.parametrize("prec,bh", FORMS)
def test_single_body_moves_in_a_straight_line(prec, bh):
    b = body_set([dict(x=3.0, y=-2.0, z=1.0, vx=1.5, vy=0.25, vz=-0.5, mass=1e12, radius=1.0)])
    sim = make(prec, bh, b)
    ora = OracleSim(seed=7, threads=2)
    ora.set_bodies(b)
    for _ in range(5):
        info = sim.step(0.01, 1.0, 1)
        ora.step(0.01, 1.0, 1)
        assert info["n_bodies"] == 1 and info["interactions"] == 0
    got, exp = sim.state(), ora.state()
    assert got["fx"][0] == 0.0 and got["fy"][0] == 0.0 and got["fz"][0] == 0.0
    assert_states_identical(got, exp, fields=("x", "y", "z", "vx", "vy", "vz", "mass", "radius"), where=prec)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_merge_down_to_one_body(prec):
    """A large subsume body absorbs the four small ones inside it in the
    first cycle (subsume needs the larger radius to reach the other body);
    the survivor keeps stepping alone.  The plain form follows the oracle bit
    for bit through the merge."""
    rows = [dict(x=0.0, mass=5e9, radius=5.0)] + [dict(x=0.8 * k, y=0.3 * k, vx=0.01 * k, mass=1e9 * k, radius=0.5)
                                                   for k in range(1, 5)]
    b = body_set(rows, behavior=A.SUBSUME)
    sim = make(prec, False, b)
    ora = OracleSim(seed=7, threads=2)
    ora.set_bodies(b)
    for c in range(6):
        sim.step(0.01, 1.0, 1)
        ora.step(0.01, 1.0, 1)
        if prec == "fp64":
            assert_states_identical(sim.state(), ora.state(), where=f"cycle {c}")
    st = sim.state()
    assert len(st["x"]) == 1 == ora.count()
    assert st["mass"][0] == pytest.approx(sum(r["mass"] for r in rows), rel=1e-15)
    info = sim.step(0.01, 1.0, 3)
    assert info["n_bodies"] == 1 and info["interactions"] == 0


def test_invalid_collision_behaviour_is_rejected_before_any_copy():
    """A load with a collision behaviour outside 0..3 fails with NBG_E_ARG and
    leaves the loaded collection as it was."""
    from nbodygo_gb300.api import NbgError

    good = body_set([dict(x=float(k), mass=1e9, radius=0.1) for k in range(100)])
    sim = make("fp64", False, good)
    before = sim.state()
    bad = body_set([dict(x=float(k), mass=1e9, radius=0.1) for k in range(50)])
    bad["collision"][7] = 9
    with pytest.raises(NbgError):
        sim.set_bodies(bad)
    after = sim.state()
    assert_states_identical(after, before, where="after a rejected load")
    bad["collision"][7] = -1
    with pytest.raises(NbgError):
        sim.set_bodies(bad)
    assert sim.count() == 100


@pytest.mark.parametrize("prec,bh,shape", [("fp64", False, None), ("mixed", False, 0), ("mixed", False, 15),
                                           ("fp64", True, None), ("mixed", True, None)])
def test_reloading_other_sizes_leaves_nothing_stale(prec, bh, shape):
    """One context loaded with 3,000 bodies, stepped through a CUDA graph,
    reloaded with 9,000, stepped, then with 500: its force pass and next
    cycles equal a fresh context's on the last set, bit for bit (buffers,
    graphs, the Morton order and the trees are all rebuilt for the new
    bodies)."""
    from nbodygo_gb300 import workloads as W

    def make():
        s = Simulation(prec, seed=4)
        if bh:
            s.set_option(A.OPT_BARNES_HUT, 1)
        if shape is not None:
            s.set_option(A.OPT_MIX_SHAPE, shape)
        s.set_option(A.OPT_GRAPH_CYCLES, 3)
        return s

    last = W.plummer(n=500, seed=33, radius_range=(0.5, 2.0))
    with make() as a:
        a.set_bodies(W.plummer(n=3000, seed=31, radius_range=(0.5, 2.0)))
        a.step(0.01, 1.0, 6)
        a.set_bodies(W.plummer(n=9000, seed=32, radius_range=(0.5, 2.0)))
        a.step(0.01, 1.0, 4)
        a.set_bodies(last)
        fa = np.array(a.force_pass())
        a.step(0.01, 1.0, 5)
        sa = a.state()
    with make() as b:
        b.set_bodies(last)
        fb = np.array(b.force_pass())
        b.step(0.01, 1.0, 5)
        sb = b.state()
    assert np.array_equal(fa.view(np.uint64), fb.view(np.uint64))
    assert_states_identical(sa, sb, where="reloaded vs fresh")


@pytest.mark.parametrize("first,then", [("fp64", "mixed"), ("mixed", "fp64")])
def test_switching_precision_mid_run(first, then):
    """nbg_set_precision on a stepped context: the cycles after the switch
    equal those of a fresh context of the new form loaded with the state
    reached, bit for bit (a switch to the plain form is the oracle's cycle
    from there on)."""
    from nbodygo_gb300 import workloads as W

    b = W.plummer(n=2000, seed=35, radius_range=(0.5, 2.0))
    with Simulation(first, seed=4) as a:
        a.set_bodies(b)
        a.step(0.01, 1.0, 3)
        mid, nid = a.state(), a.next_id()
        a.set_precision(then)
        a.step(0.01, 1.0, 4)
        sa = a.state()
    with Simulation(then, seed=4) as c:
        c.set_bodies(mid)
        c.set_next_id(nid)
        c.step(0.01, 1.0, 4)
        sc = c.state()
    assert_states_identical(sa, sc, where=f"{first} -> {then}")


@pytest.mark.parametrize("prec,bh", [("mixed", False), ("fp64", True), ("mixed", True)])
def test_switching_between_one_and_several_collections(prec, bh):
    """One context loaded with a single collection, then three, then one
    again (the launch sequence changes: per-collection passes of the octree
    sort, collection fields of the Morton keys): each stage equals a fresh
    context's, bit for bit."""
    from nbodygo_gb300 import workloads as W

    def make():
        s = Simulation(prec, seed=4)
        if bh:
            s.set_option(A.OPT_BARNES_HUT, 1)
        s.set_option(A.OPT_GRAPH_CYCLES, 2)
        return s

    one = W.plummer(n=1500, seed=36, radius_range=(0.5, 2.0))
    three = [W.plummer(n=600 + 100 * k, seed=37 + k, radius_range=(0.5, 2.0)) for k in range(3)]
    with make() as a:
        a.set_bodies(one)
        a.step(0.01, 1.0, 4)
        a.set_collections(three)
        a.step(0.01, 1.0, 4)
        s3 = a.state()
        a.set_bodies(one)
        a.step(0.01, 1.0, 4)
        s1 = a.state()
    with make() as b:
        b.set_collections(three)
        b.step(0.01, 1.0, 4)
        assert_states_identical(s3, b.state(), where="three collections after one")
    with make() as c:
        c.set_bodies(one)
        c.step(0.01, 1.0, 4)
        assert_states_identical(s1, c.state(), where="one collection after three")


def test_contexts_stepped_from_two_threads_at_once():
    """Two contexts on one GPU, each driven by its own host thread at the
    same time (ctypes drops the GIL during a call, so the calls overlap):
    each ends exactly where it ends when run alone."""
    import threading

    from nbodygo_gb300 import workloads as W

    jobs = [("mixed", W.plummer(n=6000, seed=41, radius_range=(0.5, 2.0))),
            ("fp64", W.disk(n=1500, seed=42)),
            ("mixed", W.plummer_disk(n_each=4096, seed=43))]

    def run(prec, b, out, k):
        with Simulation(prec, seed=7) as s:
            s.set_bodies(b)
            for _ in range(4):
                s.step(0.01, 1.0, 3)
            out[k] = s.state()

    alone = [None] * len(jobs)
    for k, (prec, b) in enumerate(jobs):
        run(prec, b, alone, k)
    together = [None] * len(jobs)
    threads = [threading.Thread(target=run, args=(prec, b, together, k)) for k, (prec, b) in enumerate(jobs)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for k in range(len(jobs)):
        assert_states_identical(together[k], alone[k], where=f"context {k} from a thread")


def test_failed_capacity_growth_leaves_an_empty_usable_context():
    """A growth of the body capacity that fails after the old buffers were
    released (the host-side hook stands in for a device out of memory)
    leaves one empty collection; stepping it is harmless, and the next load
    runs as in a fresh context."""
    small, big = W.plummer(n=1000, seed=31), W.plummer(n=5000, seed=32)
    for prec in ("fp64", "mixed"):
        with Simulation(prec) as ref:
            ref.set_bodies(big)
            ref.step(0.01, 1.0, 2)
            exp = ref.state()
        with Simulation(prec) as s:
            s.set_bodies(small)
            s.step(0.01, 1.0, 1)
            s.add_bodies(W.plummer(n=3, seed=33))
            s.set_option(A.OPT_TEST_FAIL_GROWTH, 1)
            with pytest.raises(NbgError) as e:
                s.set_bodies(big)
            assert e.value.code == A.NBG_E_CUDA and "no bodies" in str(e.value)
            assert s.count() == 0 and list(s.sim_counts()) == [0]
            s.step(0.01, 1.0, 2)
            assert s.count() == 0
            s.set_bodies(big)
            s.step(0.01, 1.0, 2)
            assert_states_identical(s.state(), exp, where=f"{prec}: after a failed growth")
