"""Plain FP64 form on the GPU against the CPU oracle: bit-identical state and
events, cycle after cycle, through the C ABI (libnbgpu.so)."""
import numpy as np
import pytest

from nbodygo_gb300 import _abi as A
from nbodygo_gb300 import workloads as W
from nbodygo_gb300.api import Simulation
from oracle.oracle import OracleSim

from helpers import assert_events_identical, assert_states_identical, body_set

pytestmark = pytest.mark.gpu
THREADS = 8


def run_both(bodies, dt, R, steps, per_step_check=True, seed=123, gpu_opts=None):
    sim = Simulation("fp64", seed=seed)
    for k, v in (gpu_opts or {}).items():
        sim.set_option(k, v)
    sim.set_bodies(bodies)
    ora = OracleSim(seed=seed, threads=THREADS)
    ora.set_bodies(bodies)
    if per_step_check:
        for s in range(steps):
            gi = sim.step(dt, R, 1)
            oi = ora.step(dt, R, 1)
            where = f"cycle {s}"
            assert_events_identical(sim.events(), ora.events(), where)
            assert_states_identical(sim.state(), ora.state(), where=where)
            for k in ("n_bodies", "events", "fragments_emitted", "removed", "nan_removed", "next_id",
                      "interactions"):
                assert gi[k] == oi[k], f"{where}: info {k} {gi[k]} != {oi[k]}"
    else:
        gi = sim.step(dt, R, steps)
        oi = ora.step(dt, R, steps)
        assert_states_identical(sim.state(), ora.state(), where=f"after {steps} cycles")
        for k in ("n_bodies", "events", "fragments_emitted", "removed", "next_id", "interactions"):
            assert gi[k] == oi[k], f"info {k} {gi[k]} != {oi[k]}"
    return sim, ora


def test_disk_workload_200_cycles_bit_exact():
    """Workload 0 (N=1,000 disk, elastic, dt=0.005): 20 cycles checked one by
    one, then 180 more as one graph replay, then the final state."""
    b = W.disk()
    sim, ora = run_both(b, 0.005, 1.0, 20)
    gi = sim.step(0.005, 1.0, 180)
    oi = ora.step(0.005, 1.0, 180)
    assert gi["steps_done"] == 180
    assert_states_identical(sim.state(), ora.state(), where="after 200 cycles")
    assert gi["events"] == oi["events"]


@pytest.mark.parametrize("split_max", [0, 1 << 20])
def test_plummer_workload_bit_exact(split_max):
    """Workload 1 (N=16,384 Plummer, elastic, dt=0.01): the first cycles,
    through the one-thread-per-body kernel and through the split pass."""
    b = W.plummer()
    run_both(b, 0.01, 1.0, 3, gpu_opts={A.OPT_P64_SPLIT_MAX: split_max})


def test_split_and_direct_pair_passes_agree():
    """The two plain pair passes on the same collision-heavy cluster: the same
    events and the same state, bit for bit, cycle after cycle."""
    b = dense_cluster(3000, seed=17)
    a = Simulation("fp64", seed=4)
    a.set_option(A.OPT_P64_SPLIT_MAX, 0)
    a.set_bodies(b)
    c = Simulation("fp64", seed=4)
    c.set_option(A.OPT_P64_SPLIT_MAX, 1 << 20)
    c.set_bodies(b)
    for s in range(6):
        ia, ic = a.step(0.05, 0.9, 1), c.step(0.05, 0.9, 1)
        assert ia == ic, f"cycle {s}"
        assert_events_identical(a.events(), c.events(), f"cycle {s}")
        assert_states_identical(a.state(), c.state(), where=f"cycle {s}")


def test_graph_replay_equals_single_cycles():
    b = W.plummer(n=2048, seed=9)
    s1 = Simulation("fp64")
    s1.set_bodies(b)
    s1.step(0.01, 1.0, 12)
    s2 = Simulation("fp64")
    s2.set_bodies(b)
    for _ in range(12):
        s2.step(0.01, 1.0, 1)
    assert_states_identical(s1.state(), s2.state(), where="graph vs direct")


def dense_cluster(n, seed, behaviors=(A.NONE, A.SUBSUME, A.ELASTIC, A.FRAGMENT)):
    rng = W.SplitMix64(seed)
    b = body_set([{}] * n)
    b["x"][:] = rng.uniform(n, -30, 30)
    b["y"][:] = rng.uniform(n, -30, 30)
    b["z"][:] = rng.uniform(n, -30, 30)
    b["vx"][:] = rng.normal(n, 0, 3)
    b["vy"][:] = rng.normal(n, 0, 3)
    b["vz"][:] = rng.normal(n, 0, 3)
    b["mass"][:] = rng.log_uniform(n, 1e8, 1e12)
    b["radius"][:] = rng.uniform(n, 0.5, 3.0)
    beh = np.array(behaviors, dtype=np.int32)
    b["collision"][:] = beh[np.floor(rng.uniform(n, 0, len(beh))).astype(int)]
    b["frag_factor"][:] = rng.uniform(n, 0.0, 2.0)
    # a few fragments per impact: a fragmenting body's pieces all overlap, so
    # F fragments make O(F^2) collision events per cycle
    b["frag_step"][:] = rng.uniform(n, 0.0, 6.0)
    return b


def test_dense_cluster_all_behaviours_bit_exact():
    """Many collisions of every kind (elastic, subsume, fragmentation with
    fragments emitted over several cycles), compaction and adds."""
    b = dense_cluster(400, seed=31)
    sim, ora = run_both(b, 0.05, 0.9, 25)
    # the cluster really collides: subsumed bodies left and fragments arrived
    # (the oracle resolves 89,290 events, emits 172 fragments and removes 49
    # bodies over these 25 cycles), so the count moved off 400
    assert ora.count() == sim.count() and ora.count() != 400


def test_dense_cluster_elastic_fragment_bit_exact():
    b = dense_cluster(300, seed=32, behaviors=(A.ELASTIC, A.FRAGMENT))
    run_both(b, 0.05, 1.0, 25)


def test_head_on_elastic_pair():
    b = body_set([
        dict(x=-5.0, vx=3.0, mass=1e10, radius=1.0),
        dict(x=5.0, vx=-3.0, mass=2e10, radius=1.5),
    ])
    sim, ora = run_both(b, 0.5, 1.0, 8)


def test_simtest_three_body():
    """SimTest (cmd/sim/simgen.go:382-407): a stationary body and two bodies
    heading down at it, 9e29 kg, radius 60, plus a distant sun."""
    rows = [dict(x=20000, y=20000, z=20000, vx=-3, vy=-3, vz=-5, mass=1, radius=500, collision=A.SUBSUME,
                 flags=A.F_EXISTS | A.F_IS_SUN | A.F_PINNED),
            dict(mass=9e29, radius=60),
            dict(x=-350, y=350, vx=530000000, vy=-500000000, mass=9e29, radius=60),
            dict(x=350, y=350, vx=-530000000, vy=-500000000, mass=9e29, radius=60)]
    b = body_set(rows)
    run_both(b, 1e-9, 1.0, 10)


def test_subsume_triple():
    b = body_set([
        dict(x=0.0, mass=1e9, radius=5.0),
        dict(x=0.5, mass=1e3, radius=0.2),
        dict(x=1.0, mass=2e9, radius=4.0),
        dict(x=50.0, mass=1e3, radius=0.2),
    ], behavior=A.SUBSUME)
    run_both(b, 0.01, 1.0, 3)


def test_fragment_impact_emits_fragments_over_cycles():
    b = body_set([
        dict(x=-2.0, vx=40.0, vy=1.0, mass=1e6, radius=1.0, collision=A.ELASTIC),
        dict(x=0.5, vx=-5.0, vy=0.3, vz=0.2, mass=5e6, radius=2.0, collision=A.FRAGMENT, frag_factor=0.1,
             frag_step=4.0),
    ])
    sim, ora = run_both(b, 0.01, 1.0, 6)
    assert ora.count() > 2, "the impact should have fragmented the second body"


def test_coincident_bodies_nan_path():
    """TestCollide's geometry inside a full cycle: coincident elastic bodies
    get NaN velocities, then NaN positions, and Update removes them."""
    b = body_set([dict(x=500.0, y=500.0, z=500.0, vx=1.0, mass=1.0, radius=1.0),
                  dict(x=500.0, y=500.0, z=500.0, vx=-1.0, mass=2.0, radius=1.0),
                  dict(x=900.0, mass=1.0, radius=1.0)])
    sim, ora = run_both(b, 0.1, 1.0, 2)


def test_cycle_boundary_edits():
    """AddBody, ModBody, RemoveBodies and GetBody between cycles."""
    b = dense_cluster(200, seed=41)
    sim = Simulation("fp64")
    sim.set_bodies(b)
    ora = OracleSim(threads=THREADS)
    ora.set_bodies(b)
    for s in range(6):
        if s == 1:
            add = dense_cluster(5, seed=99)
            add["id"][:] = -1
            assert np.array_equal(sim.add_bodies(add), ora.add_bodies(add))
        if s == 2:
            edits = [dict(id=3, mask=A.M_X | A.M_VX | A.M_COLLISION, x=1.5, vx=-2.0, collision=A.SUBSUME),
                     dict(id=7, mask=A.M_EXISTS, exists=0),
                     dict(id=12, mask=A.M_MASS | A.M_RADIUS, mass=5e12, radius=4.0),
                     dict(id=100000, mask=A.M_X, x=0.0)]
            assert np.array_equal(sim.apply_edits(edits), ora.apply_edits(edits))
        if s == 3:
            assert sim.remove_bodies(9) == ora.remove_bodies(9)
        if s == 4:
            got = sim.get_body(12)
            st = ora.state()
            k = int(np.flatnonzero(st["id"] == 12)[0]) if 12 in st["id"] else None
            if k is not None:
                assert got is not None and got["mass"] == st["mass"][k]
            assert sim.get_body(10 ** 9) is None
        sim.step(0.05, 1.0, 1)
        ora.step(0.05, 1.0, 1)
        assert_states_identical(sim.state(), ora.state(), where=f"cycle {s}")


def test_overflow_retry_gives_identical_result():
    """An event list of capacity 1 and a fragment buffer of capacity 1: the
    cycle stops before mutating, the buffers grow, the cycle re-runs, and the
    result is the oracle's."""
    b = dense_cluster(300, seed=32, behaviors=(A.ELASTIC, A.FRAGMENT))
    run_both(b, 0.05, 1.0, 10, gpu_opts={A.OPT_EV_CAP: 1, A.OPT_FRAG_CAP: 1})


def test_renderables_match_state():
    b = W.disk(n=500, seed=5)
    sim = Simulation("fp64")
    sim.set_bodies(b)
    sim.step(0.005, 1.0, 1)
    st = sim.state()
    r = sim.renderables()
    assert len(r) == len(st["x"])
    assert np.array_equal(r["id"], st["id"])
    assert np.array_equal(r["x"], st["x"].astype(np.float32))
    assert np.array_equal(r["z"], st["z"].astype(np.float32))
    assert np.array_equal(r["radius"], st["radius"])


def test_energy_diagnostic():
    b = W.plummer(n=512, seed=3)
    sim = Simulation("fp64")
    sim.set_bodies(b)
    ke, pe, mom = sim.energy()
    m, vx, vy, vz = b["mass"], b["vx"], b["vy"], b["vz"]
    ke_ref = float(np.sum(0.5 * m * (vx * vx + vy * vy + vz * vz)))
    x, y, z = b["x"], b["y"], b["z"]
    dx = x[None, :] - x[:, None]
    dy = y[None, :] - y[:, None]
    dz = z[None, :] - z[:, None]
    r = np.sqrt(dx * dx + dy * dy + dz * dz)
    iu = np.triu_indices(len(x), 1)
    pe_ref = float(-np.sum(6.673e-11 * m[:, None] * m[None, :] / np.where(r > 0, r, 1.0) * (r > 0))[()] / 1.0)
    pe_ref = float(-np.sum((6.673e-11 * m[:, None] * m[None, :] / np.where(r > 0, r, np.inf))[iu]))
    assert abs(ke - ke_ref) <= 1e-12 * abs(ke_ref)
    assert abs(pe - pe_ref) <= 1e-12 * abs(pe_ref)
    assert abs(mom[0] - float(np.sum(m * vx))) <= 1e-9 * float(np.sum(np.abs(m * vx)))


@pytest.mark.parametrize("seed,n,split_max", [(101, 60, 0), (102, 250, 1 << 20), (103, 700, 0), (104, 1500, 1 << 20),
                                              (105, 333, 1 << 20), (106, 2049, 0)])
def test_randomized_clusters_bit_exact(seed, n, split_max):
    """Seeded random clusters of every behaviour and size, through either
    plain pair pass: state, events and step counters equal the oracle's, cycle
    after cycle."""
    rng = np.random.default_rng(seed)
    b = dense_cluster(n, seed=seed)
    dt = float(rng.choice([0.01, 0.03, 0.05]))
    R = float(rng.choice([1.0, 0.8]))
    run_both(b, dt, R, 8, gpu_opts={A.OPT_P64_SPLIT_MAX: split_max}, seed=seed)


def test_plummer_workload_full_run_bit_exact():
    """Workload 1 for its full length (N = 16,384, elastic, dt = 0.01, 100
    cycles, replayed as CUDA graphs of 10): the final state, event and
    removal counts equal the oracle's bit for bit."""
    b = W.plummer()
    sim = Simulation("fp64", seed=123)
    sim.set_option(A.OPT_GRAPH_CYCLES, 10)
    sim.set_bodies(b)
    ora = OracleSim(seed=123, threads=THREADS)
    ora.set_bodies(b)
    gi = sim.step(0.01, 1.0, 100)
    oi = ora.step(0.01, 1.0, 100)
    assert gi["steps_done"] == 100
    for k in ("n_bodies", "events", "fragments_emitted", "removed", "interactions"):
        assert gi[k] == oi[k], f"info {k} {gi[k]} != {oi[k]}"
    assert_states_identical(sim.state(), ora.state(), where="after 100 cycles")
