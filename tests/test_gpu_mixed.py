"""Mixed-precision form: FP32 pair terms, FP64 elsewhere.  Forces within
1e-6 relative L2 of the FP64 force pass; the collision set is exact."""
import numpy as np
import pytest

from nbodygo_gb300 import _abi as A
from nbodygo_gb300 import workloads as W
from nbodygo_gb300.api import Simulation
from oracle.oracle import OracleSim

from helpers import rel_l2
from test_gpu_plain_parity import dense_cluster

pytestmark = pytest.mark.gpu
TOL = 1e-6  # relative L2 acceleration error against FP64


def mixed_forces(bodies):
    sim = Simulation("mixed")
    sim.set_bodies(bodies)
    return sim, sim.force_pass()


def live(b):
    return (b["flags"] & (A.F_EXISTS | A.F_FRAGMENTING)) == A.F_EXISTS


@pytest.mark.parametrize("n,seed", [(100, 1), (257, 2), (1000, 3), (4096, 4)])
def test_plummer_forces(n, seed):
    b = W.plummer(n=n, seed=seed)
    _, f = mixed_forces(b)
    ora = OracleSim(threads=8)
    ora.set_bodies(b)
    g = ora.forces()
    err = rel_l2(f, g)
    assert err <= TOL, f"rel L2 {err:.3e}"


def test_disk_forces_and_events():
    """Central body + disk: the dt = 0 cycle resolves the same events as the
    oracle's compute pass on the same state."""
    b = W.disk(n=1000, seed=8)
    sim, f = mixed_forces(b)
    ora = OracleSim(threads=8)
    ora.set_bodies(b)
    g = ora.forces()
    assert rel_l2(f, g) <= TOL
    sim.step(0.0, 1.0, 1)
    ora.step(0.0, 1.0, 1)
    ev_g, ev_o = sim.events(), ora.events()
    assert len(ev_g) == len(ev_o)
    assert np.array_equal(ev_g["id1"], ev_o["id1"]) and np.array_equal(ev_g["id2"], ev_o["id2"])


def test_dense_cluster_events_exact():
    """Overlapping pairs are decided in FP64: the event list of the first
    cycle is identical to the oracle's."""
    b = dense_cluster(400, seed=31)
    sim = Simulation("mixed", seed=5)
    sim.set_bodies(b)
    sim.step(0.05, 0.9, 1)
    ora = OracleSim(seed=5, threads=8)
    ora.set_bodies(b)
    ora.step(0.05, 0.9, 1)
    ev_g, ev_o = sim.events(), ora.events()
    assert len(ev_o) > 10
    for f in ("id1", "id2", "type"):
        assert np.array_equal(ev_g[f], ev_o[f])


def test_plummer_disk_subset_forces():
    """Workload 2's distribution at 1/8 size, against the FP64 oracle."""
    b = W.plummer_disk(n_each=8192, seed=3)
    _, f = mixed_forces(b)
    ora = OracleSim(threads=8)
    ora.set_bodies(b)
    g = ora.forces()
    assert rel_l2(f, g) <= TOL


def test_full_size_plummer_disk_against_fp64_gpu():
    """Workload 2 at full size (N = 131,072): mixed forces against the plain
    FP64 GPU forces (themselves bit-identical to the oracle), plus a sampled
    check of the plain forces against the oracle."""
    b = W.plummer_disk()
    _, f = mixed_forces(b)
    plain = Simulation("fp64")
    plain.set_bodies(b)
    g = plain.force_pass()
    err = rel_l2(f, g)
    assert err <= TOL, f"rel L2 {err:.3e}"
    ora = OracleSim(threads=8)
    ora.set_bodies(b)
    idx = np.arange(0, len(b["x"]), 4099)
    ox, oy, oz = ora.forces_subset(idx)
    assert np.array_equal(g[0][idx], ox) and np.array_equal(g[1][idx], oy) and np.array_equal(g[2][idx], oz)


def test_full_size_uniform_sampled():
    """Workload 4 at full size (N = 1,048,576), one cycle: a sample of 64
    bodies against the FP64 oracle, and Newton's third law on the total."""
    b = W.uniform_ball()
    _, f = mixed_forces(b)
    ora = OracleSim(threads=8)
    ora.set_bodies(b)
    idx = np.arange(0, len(b["x"]), 16411)[:64]
    g = ora.forces_subset(idx)
    err = rel_l2([c[idx] for c in f], g)
    assert err <= TOL, f"rel L2 {err:.3e}"
    tot = np.sqrt(sum(np.sum(c) ** 2 for c in f))
    mag = np.sum(np.sqrt(f[0] ** 2 + f[1] ** 2 + f[2] ** 2))
    assert tot <= 1e-5 * mag


def test_mixed_is_deterministic():
    """Persistent CTAs take work items in any order; the sums do not depend
    on it (per-item slots, fixed-order reduction)."""
    b = W.plummer_disk(n_each=4096, seed=9)
    _, f1 = mixed_forces(b)
    _, f2 = mixed_forces(b)
    for a, c in zip(f1, f2):
        assert np.array_equal(a, c)


def test_near_pairs_in_fp64_keep_error_down():
    """With the near-pair radius off, only overlap candidates go to FP64 and
    the error of close encounters grows; with it on the gate holds."""
    b = W.plummer_disk(n_each=8192, seed=3)
    ora = OracleSim(threads=8)
    ora.set_bodies(b)
    g = ora.forces()
    errs = {}
    for ppm in (0, 50000, 100000):  # off, the default, twice the default
        sim = Simulation("mixed")
        sim.set_option(A.OPT_NEAR_PPM, ppm)
        sim.set_bodies(b)
        errs[ppm] = rel_l2(sim.force_pass(), g)
    assert errs[50000] <= TOL and errs[100000] <= TOL
    assert errs[100000] <= errs[50000] <= errs[0]


def test_every_body_within_1e6_of_its_term_scale():
    """The per-body reading of the 1e-6 bound: each body's error against the
    FP64 force, relative to the sum of the magnitudes of its terms
    sum_j |f_ij| (the scale FP32 rounding acts on; in a dense core the terms
    cancel and |f_i| is far smaller).  Since sum_j |f_ij| >= |f_i|, only
    bodies whose plain relative error exceeds the bound need the sum."""
    b = W.plummer_disk(n_each=8192, seed=3)
    ora = OracleSim(threads=8)
    ora.set_bodies(b)
    g = np.array(ora.forces())
    with Simulation("mixed") as sim:
        sim.set_bodies(b)
        f = np.array(sim.force_pass())
    err = np.linalg.norm(f - g, axis=0)
    mag = np.linalg.norm(g, axis=0)
    worst = np.argsort(err / mag)[::-1][:512]
    assert (err / mag)[worst[-1]] <= TOL, "more than 512 bodies above the bound: widen the sample"
    x = np.stack([b["x"], b["y"], b["z"]])
    G = 6.673e-11
    for i in worst:
        d = np.linalg.norm(x - x[:, i:i + 1], axis=0)
        far = d > b["radius"] + b["radius"][i]
        far[i] = False
        scale = G * b["mass"][i] * np.sum(b["mass"][far] / d[far] ** 2)
        assert err[i] <= TOL * scale, f"body {i}: {err[i] / scale:.3e} of its term scale"


def test_every_kernel_shape_gives_the_same_physics():
    """All compiled shapes of the mixed pair kernel agree with FP64 within
    the tolerance and detect the same events; the autotuner picks one."""
    b = dense_cluster(300, seed=51)
    ora = OracleSim(threads=8)
    ora.set_bodies(b)
    g = ora.forces()
    for shape in range(A.MIX_SHAPES):
        sim = Simulation("mixed")
        sim.set_option(A.OPT_MIX_SHAPE, shape)
        sim.set_bodies(b)
        assert rel_l2(sim.force_pass(), g) <= TOL, f"shape {shape}"
        sim.step(0.05, 1.0, 1)
        assert len(sim.events()) > 0
    big = W.plummer_disk(n_each=4096, seed=7)
    sim = Simulation("mixed")
    sim.set_bodies(big)
    shape, ms = sim.autotune()
    assert 0 <= shape < A.MIX_SHAPES and ms > 0
    ora = OracleSim(threads=8)
    ora.set_bodies(big)
    assert rel_l2(sim.force_pass(), ora.forces()) <= TOL


def fp64_forces_by_id(pre, ids):
    """FP64 force pass on the state `pre`, as (3, len(ids)) for the bodies
    `ids` (all of which are in `pre`)."""
    ref = Simulation("fp64")
    ref.set_bodies(pre)
    f = np.array(ref.force_pass())
    ref.close()
    order = np.argsort(pre["id"])
    at = order[np.searchsorted(pre["id"], ids, sorter=order)]
    return f[:, at]


def step_and_check(sim, cycles, dt, tol=TOL):
    """Each cycle: the mixed forces it computed (read from the state after
    it) against FP64 forces of the state before it, body by body (by id;
    bodies a cycle created have no reference and are skipped).  Returns the
    bodies removed over the cycles."""
    removed = 0
    for _ in range(cycles):
        pre = sim.state()
        info = sim.step(dt, 1.0, 1)
        removed += info["removed"]
        post = sim.state()
        keep = np.isin(post["id"], pre["id"]) & live(post)
        ids = post["id"][keep]
        got = np.array([post["fx"][keep], post["fy"][keep], post["fz"][keep]])
        exp = fp64_forces_by_id(pre, ids)
        err = rel_l2(got, exp)
        assert err <= tol, f"rel L2 {err:.3e}"
    return removed


@pytest.mark.parametrize("interval", [1, 8, 1000])
def test_sort_interval_keeps_forces_accurate(interval):
    """Cycles that keep an older Morton order (the bodies have moved since)
    stay within the FP64 tolerance."""
    b = W.plummer_disk(2048, seed=21)
    sim = Simulation("mixed")
    sim.set_option(A.OPT_SORT_INTERVAL, interval)
    sim.set_bodies(b)
    step_and_check(sim, 10, 0.5)


def test_sort_interval_resorts_after_compaction_and_edits():
    """With a 1000-cycle interval, compaction (merged bodies) and a host edit
    that moves a body far away each force a new order: a stale permutation
    would pair forces with the wrong bodies.  No fragmentation here: a cycle
    emits fragments and shrinks their parents before its pair pass, so its
    forces belong to a state that is never read back."""
    sim = Simulation("mixed", seed=3)
    sim.set_option(A.OPT_SORT_INTERVAL, 1000)
    sim.set_bodies(dense_cluster(400, seed=31, behaviors=(A.NONE, A.SUBSUME, A.ELASTIC)))
    removed = step_and_check(sim, 6, 0.05)
    assert removed > 0
    st = sim.state()
    sim.apply_edits([dict(id=int(st["id"][5]), mask=A.M_X | A.M_Y, x=5000.0, y=-4000.0)])
    step_and_check(sim, 2, 0.05)
    with pytest.raises(Exception):
        sim.set_option(A.OPT_SORT_INTERVAL, 0)


@pytest.mark.parametrize("kind,n,seed", [("uniform", 3000, 1), ("plummer", 2500, 2), ("disk", 3500, 3),
                                         ("cluster", 1200, 4), ("uniform", 700, 5), ("plummer", 4096, 6)])
def test_randomized_forces_within_gate(kind, n, seed):
    """Mixed forces of seeded collections of several distributions and sizes
    stay within 1e-6 relative L2 of the oracle."""
    if kind == "uniform":
        b = W.uniform_ball(n=n, seed=seed, R=0.5 * n ** (1 / 3) * 10, radius=0.3)
    elif kind == "plummer":
        b = W.plummer(n=n, seed=seed)
    elif kind == "disk":
        b = W.disk(n=n, seed=seed)
    else:
        b = dense_cluster(n, seed=seed)
    _, f = mixed_forces(b)
    ora = OracleSim(threads=8)
    ora.set_bodies(b)
    err = rel_l2(f, ora.forces())
    assert err <= TOL, f"{kind} n={n}: rel L2 {err:.3e}"


def _net_force_ratio(f, lo=0, hi=None):
    fx, fy, fz = (np.asarray(c[lo:hi], dtype=np.float64) for c in f)
    net = np.sqrt(fx.sum() ** 2 + fy.sum() ** 2 + fz.sum() ** 2)
    scale = np.sqrt(fx ** 2 + fy ** 2 + fz ** 2).sum()
    return net / scale


def test_full_size_uniform_forces_cancel():
    """Config 4 at full size (2^20 bodies): gravity is pairwise antisymmetric,
    so the forces of the mixed pass sum to zero up to rounding."""
    b = W.uniform_ball()
    sim = Simulation("mixed", capacity=len(b["x"]))
    sim.set_bodies(b)
    ratio = _net_force_ratio(sim.force_pass())
    assert ratio <= 1e-6, f"net force {ratio:.3e} of the summed magnitudes"


def test_full_size_ensemble_forces_cancel_per_collection():
    """Config 3 at full size (512 collections, 3.3 M bodies): each
    collection's forces sum to zero up to rounding, so no pair crosses
    collections and none is counted once."""
    sims = W.ensemble()
    sim = Simulation("mixed", capacity=sum(len(s["x"]) for s in sims))
    sim.set_collections(sims)
    f = sim.force_pass()
    o, worst = 0, 0.0
    for s in sims:
        n = len(s["x"])
        worst = max(worst, _net_force_ratio(f, o, o + n))
        o += n
    assert worst <= 1e-5, f"worst net force {worst:.3e} of a collection's summed magnitudes"


def test_autotune_cache_file(tmp_path):
    """The first tuning of a collection appends its result to the cache
    file; a context of the same size bucket takes the shape from the file
    without measuring (the same shape and time come back)."""
    path = str(tmp_path / "tune.txt")
    b = W.plummer(n=9000, seed=17)
    with Simulation("mixed") as s1:
        s1.set_bodies(b)
        shape1, ms1 = s1.autotune(path)
    lines = open(path).read().split("\n")
    assert len([ln for ln in lines if ln.strip()]) == 1 and lines[0].split()[1] == str(shape1)
    with Simulation("mixed") as s2:
        s2.set_bodies(W.plummer(n=10000, seed=18))  # the same power-of-two bucket
        shape2, ms2 = s2.autotune(path)
    assert (shape2, round(ms2, 4)) == (shape1, round(ms1, 4))
    assert len([ln for ln in open(path).read().split("\n") if ln.strip()]) == 1
