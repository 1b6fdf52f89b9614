"""The oracle's restatement of the reference's Barnes-Hut octree
(cmd/body/octree.go) on the CPU: known answers for small cases and the size
of the approximation on a Plummer sphere."""
import math

import numpy as np

from nbodygo_gb300 import _abi as A
from nbodygo_gb300 import workloads as W
from oracle.oracle import OracleSim

from helpers import body_set

G = 6.673e-11
SOFT2 = 1e-4 * 1e-4


def bh_forces(b):
    o = OracleSim()
    o.set_bodies(b)
    o.set_barnes_hut(True)
    return np.stack(o.forces(), 1)


def test_two_bodies_are_two_leaves_with_softening():
    """Two bodies: each is a leaf of the other's walk, so the force is the
    softened point-mass term of octree.go:286-292 exactly."""
    b = body_set([dict(x=-3.0, y=1.0, mass=5e10, radius=0.1), dict(x=4.0, y=-2.0, z=0.5, mass=2e9, radius=0.1)])
    f = bh_forces(b)
    for i, j in ((0, 1), (1, 0)):
        # the leaf's centre is x * m / m, as the running update leaves it
        cm = [b[c][j] * b["mass"][j] / b["mass"][j] for c in "xyz"]
        d = [cm[k] - b[c][i] for k, c in enumerate("xyz")]
        dsq = d[0] * d[0] + d[1] * d[1] + d[2] * d[2] + SOFT2
        dist = math.sqrt(dsq)
        force = G * b["mass"][i] * b["mass"][j] / dsq
        assert list(f[i]) == [force * d[k] / dist for k in range(3)]


def test_sun_sums_every_body_directly():
    b = W.disk(300)
    b["flags"][0] |= A.F_IS_SUN
    f = bh_forces(b)
    x = np.stack([b["x"], b["y"], b["z"]], 1)
    d = x[1:] - x[0]
    dsq = np.sum(d * d, 1) + SOFT2
    force = G * b["mass"][0] * b["mass"][1:] / dsq
    exp = np.sum((force / np.sqrt(dsq))[:, None] * d, 0)
    assert np.allclose(f[0], exp, rtol=1e-12, atol=0)


def test_plummer_approximation_is_small_but_not_zero():
    """The reference's default force path as built (BuildTree never calls
    Build) applies no gravity; with the tree built, theta = 0.3 stays within
    a few 1e-3 of the direct sum."""
    b = W.plummer(4096, seed=2)
    bh = bh_forces(b)
    o = OracleSim(threads=4)
    o.set_bodies(b)
    direct = np.stack(o.forces(), 1)
    rel = np.linalg.norm(bh - direct) / np.linalg.norm(direct)
    assert 1e-5 < rel < 5e-3


def test_dead_and_fragmenting_bodies_stay_out_of_the_tree():
    b = W.plummer(500, seed=3)
    b["flags"][7] = 0  # not existing
    f = bh_forces(b)
    b2 = {k: np.delete(v, 7) for k, v in b.items()}
    f2 = bh_forces(b2)
    assert np.array_equal(np.delete(f, 7, axis=0), f2)
