"""The mixed form at the full sizes of the measured workloads, each against an
FP64 reference:

- the 512-collection ensemble (3.3 M bodies): mixed forces against the plain
  FP64 GPU forces (bit-identical to the oracle), relative L2 <= 1e-6 over all
  of them, and every body's error against the sum of its terms' magnitudes:
  the 99.9th percentile within 1e-6 and the worst body within the far-pair
  bound at the default near-pair factor, every body within 1e-6 at factor
  0.15;
- the 2^20-body uniform ball: 1,024 bodies spread over the ball against the
  CPU oracle's FP64 forces;
- the 131,072-body Plummer sphere + disk over its stated 1,000 cycles: the
  subsume events conserve mass to 1e-12, and the first 10 cycles resolve the
  same events and remove the same bodies as the plain FP64 form.
"""
import numpy as np
import pytest

from nbodygo_gb300 import _abi as A
from nbodygo_gb300 import workloads as W
from nbodygo_gb300.api import Simulation
from oracle.oracle import OracleSim

from helpers import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-6
G = 6.673e-11


def term_scale(sims):
    """Each body's sum_j |f_ij| = G m_i sum_j m_j / d_ij^2 over the pairs the
    force pass sums (j != i, d_ij > r_i + r_j: calcForceFrom's overlap skip,
    cmd/body/body.go:214-225), in FP64 on the GPU, in the flat body order."""
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    out = []
    for b in sims:
        x = torch.tensor(np.stack([b["x"], b["y"], b["z"]], 1), device=dev, dtype=torch.float64)
        m = torch.tensor(b["mass"], device=dev, dtype=torch.float64)
        r = torch.tensor(b["radius"], device=dev, dtype=torch.float64)
        k = len(b["x"])
        o = torch.empty(k, device=dev, dtype=torch.float64)
        for i0 in range(0, k, 1024):
            i1 = min(k, i0 + 1024)
            d2 = ((x[None, :, :] - x[i0:i1, None, :]) ** 2).sum(2)
            far = d2.sqrt() > r[i0:i1, None] + r[None, :]
            far[torch.arange(i1 - i0, device=dev), torch.arange(i0, i1, device=dev)] = False
            w = torch.where(far, m[None, :] / torch.where(far, d2, torch.ones_like(d2)), torch.zeros_like(d2))
            o[i0:i1] = G * m[i0:i1] * w.sum(1)
        out.append(o.cpu().numpy())
    return np.concatenate(out)


def test_ensemble_mixed_against_fp64_body_by_body():
    sims = W.ensemble()
    n = sum(len(s["x"]) for s in sims)
    with Simulation("fp64", capacity=n) as p:
        p.set_collections(sims)
        g = np.array(p.force_pass())
    scale = term_scale(sims)

    def mixed(ppm=None):
        with Simulation("mixed", capacity=n) as m:
            if ppm is not None:
                m.set_option(A.OPT_NEAR_PPM, ppm)
            m.set_collections(sims)
            return np.array(m.force_pass())

    f = mixed()
    assert rel_l2(f, g) <= TOL
    # A collection's relative L2 can exceed 1e-6 where its bodies' forces
    # cancel (disks: |f_i| near a fifth of sum_j |f_ij|), which scales the
    # FP32 rounding of the terms up against |f_i|.
    o = 0
    for s, b in enumerate(sims):
        k = len(b["x"])
        e = rel_l2(f[:, o:o + k], g[:, o:o + k])
        assert e <= 2 * TOL, f"collection {s}: relative L2 {e:.3e}"
        o += k
    # Body by body against the cancellation-free scale.  A pair beyond the
    # near-pair radius kappa |x' - c| (kappa 0.05) carries a dx error of at
    # most sqrt(3) 2^-24 (1 + 2 / kappa) of its distance and a term error of
    # twice that; in sparse disks a single such neighbour can carry most of
    # a body's force, which is the tail above 1e-6.
    e = np.linalg.norm(f - g, axis=0) / scale
    assert np.quantile(e, 0.999) <= TOL, f"99.9th percentile {np.quantile(e, 0.999):.3e}"
    bound = 2 * np.sqrt(3.0) * 2.0 ** -24 * (1 + 2 / 0.05) + TOL
    assert e.max() <= bound, f"worst body {e.max():.3e} of its term scale, bound {bound:.3e}"
    # with the near-pair factor at 0.15 every body is within 1e-6
    e = np.linalg.norm(mixed(150000) - g, axis=0) / scale
    assert e.max() <= TOL, f"factor 0.15: worst body {e.max():.3e} of its term scale"


@pytest.mark.parametrize("shape", [0, A.MIX_SYM])
def test_uniform_ball_1024_bodies_against_the_oracle(shape):
    """The default one-sided shape, and the symmetric kernel the autotuner
    picks for this workload (2.1 M block pairs, 13 GB of j partials)."""
    b = W.uniform_ball()
    with Simulation("mixed", capacity=len(b["x"])) as m:
        m.set_option(A.OPT_MIX_SHAPE, shape)
        m.set_bodies(b)
        f = m.force_pass()
    ora = OracleSim(threads=8)
    ora.set_bodies(b)
    idx = np.arange(1024) * (len(b["x"]) // 1024) + 511
    g = ora.forces_subset(idx)
    err = rel_l2([c[idx] for c in f], g)
    assert err <= TOL, f"rel L2 {err:.3e}"


def test_plummer_disk_1000_cycles_conserve_mass_and_match_fp64_events():
    b = W.plummer_disk()
    dt = 0.01
    m = Simulation("mixed", capacity=len(b["x"]) + 4096)
    p = Simulation("fp64", capacity=len(b["x"]) + 4096)
    m.set_bodies(b)
    p.set_bodies(b)
    m0 = float(np.sum(b["mass"]))
    for c in range(10):
        im, ip = m.step(dt, 1.0, 1), p.step(dt, 1.0, 1)
        assert (im["events"], im["removed"], im["n_bodies"]) == (ip["events"], ip["removed"], ip["n_bodies"]), \
            f"cycle {c}"
        em, ep = m.events(), p.events()
        assert np.array_equal(em["id1"], ep["id1"]) and np.array_equal(em["id2"], ep["id2"]), f"cycle {c}"
    p.close()
    m.set_option(A.OPT_GRAPH_CYCLES, 10)
    done, events = 10, 0
    while done < 1000:
        info = m.step(dt, 1.0, 10)
        done += info["steps_done"]
        events += info["events"]
    st = m.state()
    live = (st["flags"] & A.F_EXISTS) != 0
    drift = abs(float(np.sum(st["mass"][live])) - m0) / m0
    assert events > 100
    assert drift <= 1e-12, f"mass drift {drift:.3e} over 1,000 cycles"
    m.close()
