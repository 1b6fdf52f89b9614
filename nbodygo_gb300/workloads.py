"""Seeded synthetic body sets for the benchmark workloads.

No public dataset is involved: each workload is a documented distribution
drawn from a SplitMix64 stream (uniform doubles with 53 random bits, normals by
Box-Muller), so the same seed gives the same bodies on every machine and every
numpy version.  All workloads use G = 6.673e-11 (cmd/body/body.go:19).

  disk        central body (m=5e15, r=20) + annulus r in [100,1000] (uniform
              in area), z ~ N(0, 5^2), circular speed sqrt(G M / r) plus
              N(0, 0.5^2) per component, m log-uniform [1e3, 1e5], radius
              U(0.5, 2), elastic                                  (N = 1,000)
  plummer     Plummer sphere (Aarseth, Henon & Wielen 1974 sampling; radius
              truncated at 10 a; speeds by von Neumann rejection on
              q^2 (1-q^2)^(7/2)); equal masses                   (N = 16,384)
  plummer_disk  65,536 Plummer (a=300, M=1e16) + 65,536 disk bodies orbiting
              it (r in [400, 4000]); radii U(0.1, 0.5); subsume  (N = 131,072)
  uniform     uniform ball R = 20,000, m = 1e10, radius 0.05, v ~ N(0, 1),
              no collisions                                    (N = 1,048,576)
  ensemble    512 independent sims, N log-uniform [256, 32768], each one of
              {uniform ball R = 0.5 N^(1/3) 10, Plummer a = 200, disk};
              behaviour cycles none / elastic / subsume; m log-uniform
              [1e3, 1e6]; radius U(0.1, 1)
"""
import numpy as np

from . import _abi as A

G = 6.673e-11
_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


class SplitMix64:
    """SplitMix64 (Steele, Lea & Flood 2014) as a vectorised stream."""

    def __init__(self, seed):
        self.state = np.uint64(int(seed) & (2 ** 64 - 1))

    def u64(self, n):
        with np.errstate(over="ignore"):
            idx = np.arange(1, n + 1, dtype=np.uint64)
            z = self.state + idx * _GOLDEN
            self.state = self.state + np.uint64(n) * _GOLDEN
            z = (z ^ (z >> np.uint64(30))) * _M1
            z = (z ^ (z >> np.uint64(27))) * _M2
            return z ^ (z >> np.uint64(31))

    def uniform(self, n, lo=0.0, hi=1.0):
        u = (self.u64(n) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)
        return lo + (hi - lo) * u

    def normal(self, n, mu=0.0, sigma=1.0):
        u1 = self.uniform(n)
        u2 = self.uniform(n)
        return mu + sigma * np.sqrt(-2.0 * np.log1p(-u1)) * np.cos(2.0 * np.pi * u2)

    def log_uniform(self, n, lo, hi):
        return np.exp(self.uniform(n, np.log(lo), np.log(hi)))

    def unit_vectors(self, n):
        cz = self.uniform(n, -1.0, 1.0)
        ph = self.uniform(n, 0.0, 2.0 * np.pi)
        s = np.sqrt(1.0 - cz * cz)
        return s * np.cos(ph), s * np.sin(ph), cz


def _bodies(n):
    b = {f: np.zeros(n, dtype=A.FIELD_DTYPES[f]) for f in
         ("id", "x", "y", "z", "vx", "vy", "vz", "radius", "mass", "frag_factor", "frag_step", "collision", "flags")}
    b["id"][:] = np.arange(n, dtype=np.int64)
    b["flags"][:] = A.F_EXISTS
    b["collision"][:] = A.ELASTIC
    return b


def _concat(parts):
    out = {k: np.concatenate([p[k] for p in parts]) for k in parts[0]}
    out["id"] = np.arange(len(out["x"]), dtype=np.int64)
    return out


def disk(n=1000, seed=1, r_in=100.0, r_out=1000.0, central_mass=5e15, central_radius=20.0,
         radius_lo=0.5, radius_hi=2.0, enclosed_mass=None, with_central=True, behavior=A.ELASTIC):
    """Central body + disk annulus (workload 0 and the disk half of workload 2)."""
    rng = SplitMix64(seed)
    nd = n - 1 if with_central else n
    b = _bodies(n)
    r = np.sqrt(rng.uniform(nd, r_in * r_in, r_out * r_out))
    phi = rng.uniform(nd, 0.0, 2.0 * np.pi)
    z = rng.normal(nd, 0.0, 5.0)
    m_enc = central_mass if enclosed_mass is None else enclosed_mass(r)
    vt = np.sqrt(G * m_enc / r)
    vx = -vt * np.sin(phi) + rng.normal(nd, 0.0, 0.5)
    vy = vt * np.cos(phi) + rng.normal(nd, 0.0, 0.5)
    vz = rng.normal(nd, 0.0, 0.5)
    o = 1 if with_central else 0
    b["x"][o:] = r * np.cos(phi)
    b["y"][o:] = r * np.sin(phi)
    b["z"][o:] = z
    b["vx"][o:], b["vy"][o:], b["vz"][o:] = vx, vy, vz
    b["mass"][o:] = rng.log_uniform(nd, 1e3, 1e5)
    b["radius"][o:] = rng.uniform(nd, radius_lo, radius_hi)
    if with_central:
        b["mass"][0] = central_mass
        b["radius"][0] = central_radius
    b["collision"][:] = behavior
    return b


def plummer(n=16384, seed=2, a=200.0, total_mass=1e16, radius=0.2, r_max_factor=10.0, behavior=A.ELASTIC,
            radius_range=None):
    """Plummer sphere with isotropic velocities from its distribution function."""
    rng = SplitMix64(seed)
    b = _bodies(n)
    r = np.empty(0)
    while len(r) < n:
        x1 = rng.uniform(2 * (n - len(r)) + 16)
        x1 = x1[x1 > 0]
        rr = a / np.sqrt(x1 ** (-2.0 / 3.0) - 1.0)
        r = np.concatenate([r, rr[rr <= r_max_factor * a]])
    r = r[:n]
    ux, uy, uz = rng.unit_vectors(n)
    q = np.empty(0)
    while len(q) < n:
        m = 2 * (n - len(q)) + 64
        qq = rng.uniform(m)
        yy = rng.uniform(m, 0.0, 0.1)
        q = np.concatenate([q, qq[yy < qq * qq * (1.0 - qq * qq) ** 3.5]])
    q = q[:n]
    vesc = np.sqrt(2.0 * G * total_mass) * (r * r + a * a) ** -0.25
    v = q * vesc
    wx, wy, wz = rng.unit_vectors(n)
    b["x"][:], b["y"][:], b["z"][:] = r * ux, r * uy, r * uz
    b["vx"][:], b["vy"][:], b["vz"][:] = v * wx, v * wy, v * wz
    b["mass"][:] = total_mass / n
    if radius_range is None:
        b["radius"][:] = radius
    else:
        b["radius"][:] = rng.uniform(n, radius_range[0], radius_range[1])
    b["collision"][:] = behavior
    return b


def plummer_disk(n_each=65536, seed=3):
    """Workload 2: Plummer (a=300, M=1e16) + a disk orbiting it, subsume."""
    a, M = 300.0, 1e16
    p = plummer(n_each, seed=seed, a=a, total_mass=M, behavior=A.SUBSUME, radius_range=(0.1, 0.5))

    def m_enc(r):
        return M * r ** 3 / (r * r + a * a) ** 1.5

    d = disk(n_each, seed=seed + 1000, r_in=400.0, r_out=4000.0, radius_lo=0.1, radius_hi=0.5,
             enclosed_mass=m_enc, with_central=False, behavior=A.SUBSUME)
    return _concat([p, d])


def uniform_ball(n=1048576, seed=4, R=20000.0, mass=1e10, radius=0.05, behavior=A.NONE):
    """Workload 4: uniform ball, equal masses, v ~ N(0, 1), no collisions."""
    rng = SplitMix64(seed)
    b = _bodies(n)
    r = R * np.cbrt(rng.uniform(n))
    ux, uy, uz = rng.unit_vectors(n)
    b["x"][:], b["y"][:], b["z"][:] = r * ux, r * uy, r * uz
    b["vx"][:], b["vy"][:], b["vz"][:] = rng.normal(n), rng.normal(n), rng.normal(n)
    b["mass"][:] = mass
    b["radius"][:] = radius
    b["collision"][:] = behavior
    return b


def ensemble_sizes(count=512, seed=5, lo=256, hi=32768):
    rng = SplitMix64(seed)
    return np.floor(rng.log_uniform(count, lo, hi)).astype(np.int64)


def ensemble(count=512, seed=5, lo=256, hi=32768):
    """Workload 3: list of independent body sets of uneven size."""
    sizes = ensemble_sizes(count, seed, lo, hi)
    rng = SplitMix64(seed + 77)
    kinds = np.floor(rng.uniform(count, 0, 3)).astype(int)
    behaviors = [A.NONE, A.ELASTIC, A.SUBSUME]
    sims = []
    for s, (n, kind) in enumerate(zip(sizes, kinds)):
        beh = behaviors[s % 3]
        sub_seed = seed * 100003 + s
        if kind == 0:
            b = uniform_ball(int(n), seed=sub_seed, R=0.5 * n ** (1.0 / 3.0) * 10.0, mass=1.0, radius=0.1,
                             behavior=beh)
        elif kind == 1:
            b = plummer(int(n), seed=sub_seed, a=200.0, total_mass=1e16, behavior=beh)
        else:
            b = disk(int(n), seed=sub_seed, behavior=beh)
        r2 = SplitMix64(sub_seed + 5)
        b["mass"][:] = r2.log_uniform(int(n), 1e3, 1e6)
        b["radius"][:] = r2.uniform(int(n), 0.1, 1.0)
        sims.append(b)
    return sims


WORKLOADS = {
    "disk": dict(fn=disk, n=1000, dt=0.005, steps=200, precision="fp64"),
    "plummer": dict(fn=plummer, n=16384, dt=0.01, steps=100, precision="fp64"),
    "plummer_disk": dict(fn=plummer_disk, n=131072, dt=0.01, steps=1000, precision="mixed"),
    "uniform": dict(fn=uniform_ball, n=1048576, dt=0.01, steps=20, precision="mixed"),
}
