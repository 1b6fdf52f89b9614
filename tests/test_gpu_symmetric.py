"""The symmetric mixed pair kernel (the last two shapes, k_pair_sym with
registers capped for 4 and 5 CTAs per SM):
each unordered pair computed once and added to both bodies.  It must give
the FP64 forces within the mixed tolerance on collections of several
512-body blocks (where pairs rotate through the warps), ragged last blocks,
several collections, bodies that exert no force, and dense clusters whose
near pairs fall across blocks; the events must be the oracle's; the result
must not depend on scheduling."""
import numpy as np
import pytest

from nbodygo_gb300 import _abi as A
from nbodygo_gb300 import workloads as W
from nbodygo_gb300.api import Simulation
from oracle.oracle import OracleSim

from helpers import rel_l2
from test_gpu_plain_parity import dense_cluster

pytestmark = pytest.mark.gpu
TOL = 1e-6
SYM = A.MIX_SYM
SHAPES = (A.MIX_SYM, A.MIX_SYM + 1)


def forces(b, shape=SYM, sims=None):
    with Simulation("mixed") as s:
        s.set_option(A.OPT_MIX_SHAPE, shape)
        if sims is None:
            s.set_bodies(b)
        else:
            s.set_collections(sims)
        return np.array(s.force_pass())


def oracle_forces(b):
    o = OracleSim(threads=8)
    o.set_bodies(b)
    return np.array(o.forces())


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("n", [513, 1023, 1025, 4096, 5000])
def test_plummer_against_the_oracle(n, shape):
    b = W.plummer(n=n, seed=n)
    f = forces(b, shape=shape)
    assert rel_l2(f, oracle_forces(b)) <= TOL


@pytest.mark.parametrize("shape", SHAPES)
def test_plummer_disk_against_the_oracle_and_the_one_sided_kernel(shape):
    b = W.plummer_disk(n_each=8192, seed=3)
    f = forces(b, shape=shape)
    g = oracle_forces(b)
    assert rel_l2(f, g) <= TOL
    assert rel_l2(f, forces(b, shape=7)) <= TOL


def test_bodies_that_exert_no_force():
    """Non-existent, fragmenting and non-finite bodies: no term from them
    reaches any other body."""
    b = W.plummer(n=3000, seed=11)
    b["flags"][::7] = 0                              # do not exist
    b["flags"][3::11] |= A.F_FRAGMENTING              # fragmenting
    b["x"][5::97] = np.nan                            # non-finite position
    live = (b["flags"] & (A.F_EXISTS | A.F_FRAGMENTING)) == A.F_EXISTS
    ok = live & np.isfinite(b["x"])
    f = forces(b)
    g = oracle_forces(b)
    assert np.all(np.isfinite(f[:, ok]))
    assert rel_l2(f[:, ok], g[:, ok]) <= TOL
    assert rel_l2(f[:, ok], forces(b, shape=7)[:, ok]) <= TOL


def test_several_collections():
    sims = [W.plummer(n=1500, seed=1), W.disk(n=700, seed=2), W.uniform_ball(n=2100, seed=3, R=300.0),
            W.plummer(n=1, seed=4), W.plummer(n=512, seed=5)]
    f = forces(None, sims=sims)
    o = 0
    for b in sims:
        k = len(b["x"])
        if k > 1:
            assert rel_l2(f[:, o:o + k], oracle_forces(b)) <= TOL
        o += k


@pytest.mark.parametrize("shape", SHAPES)
def test_dense_cluster_events_and_forces(shape):
    """Near and overlapping pairs in every block pair: exact FP64 terms on
    both sides, and the oracle's event list."""
    b = dense_cluster(3000, seed=61)
    with Simulation("mixed", seed=5) as s:
        s.set_option(A.OPT_MIX_SHAPE, shape)
        s.set_bodies(b)
        f = np.array(s.force_pass())
        s.step(0.05, 0.9, 1)
        ev = s.events()
    assert rel_l2(f, oracle_forces(b)) <= TOL
    ora = OracleSim(seed=5, threads=8)
    ora.set_bodies(b)
    ora.step(0.05, 0.9, 1)
    eo = ora.events()
    assert len(eo) > 1000
    for k in ("id1", "id2", "type"):
        assert np.array_equal(ev[k], eo[k]), k


def test_deterministic():
    b = W.plummer_disk(n_each=4096, seed=9)
    a, c = forces(b), forces(b)
    assert np.array_equal(a, c)


def test_cycles_through_the_symmetric_kernel_match_one_sided_events():
    """Several cycles of a colliding workload: the same events and removals
    as the one-sided kernel, cycle by cycle."""
    b = W.plummer_disk(n_each=4096, seed=13)
    runs = []
    for shape in (SYM, 7):
        s = Simulation("mixed", seed=2)
        s.set_option(A.OPT_MIX_SHAPE, shape)
        s.set_bodies(b)
        runs.append(s)
    for c in range(5):
        i1, i2 = runs[0].step(0.01, 1.0, 1), runs[1].step(0.01, 1.0, 1)
        assert (i1["events"], i1["removed"]) == (i2["events"], i2["removed"]), f"cycle {c}"
    for s in runs:
        s.close()
