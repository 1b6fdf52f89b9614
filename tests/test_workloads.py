"""Seeded synthetic workloads: deterministic, right sizes and distributions."""
import numpy as np

from nbodygo_gb300 import _abi as A
from nbodygo_gb300 import workloads as W


def test_splitmix_reference_values():
    # SplitMix64 with seed 0: published first outputs
    r = W.SplitMix64(0)
    assert [int(v) for v in r.u64(3)] == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]


def test_deterministic():
    a, b = W.disk(seed=5), W.disk(seed=5)
    for k in a:
        assert np.array_equal(a[k], b[k])


def test_disk():
    b = W.disk()
    assert len(b["x"]) == 1000 and b["mass"][0] == 5e15 and b["radius"][0] == 20
    r = np.hypot(b["x"][1:], b["y"][1:])
    assert r.min() >= 100 and r.max() <= 1000
    assert 1e3 <= b["mass"][1:].min() and b["mass"][1:].max() <= 1e5
    assert np.all(b["collision"] == A.ELASTIC)
    assert abs(np.std(b["z"][1:]) - 5.0) < 0.5


def test_plummer():
    b = W.plummer(n=4096)
    r = np.sqrt(b["x"] ** 2 + b["y"] ** 2 + b["z"] ** 2)
    # half-mass radius of a Plummer sphere: a / sqrt(2^(2/3) - 1) = 1.305 a
    assert abs(np.median(r) / 200.0 - 1.305) < 0.08
    assert np.all(r <= 2000.0)
    assert np.allclose(b["mass"], 1e16 / 4096)
    # virial ratio 2T/|U| = 1 for the Plummer model; T from the samples
    t = 0.5 * np.sum(b["mass"] * (b["vx"] ** 2 + b["vy"] ** 2 + b["vz"] ** 2))
    u = 3 * np.pi / 32 * W.G * 1e16 ** 2 / 200.0
    assert abs(2 * t / u - 1.0) < 0.15


def test_plummer_disk_and_uniform_sizes():
    b = W.plummer_disk(n_each=1024)
    assert len(b["x"]) == 2048 and np.all(b["collision"] == A.SUBSUME)
    assert b["radius"].min() >= 0.1 and b["radius"].max() <= 0.5
    assert np.array_equal(b["id"], np.arange(2048))
    u = W.uniform_ball(n=10000)
    r = np.sqrt(u["x"] ** 2 + u["y"] ** 2 + u["z"] ** 2)
    assert r.max() <= 20000 and abs(np.mean((r / 20000) ** 3) - 0.5) < 0.02


def test_ensemble_sizes():
    s = W.ensemble_sizes()
    assert len(s) == 512 and s.min() >= 256 and s.max() <= 32768
    assert abs(np.mean(np.log(s)) - 0.5 * (np.log(256) + np.log(32768))) < 0.2
