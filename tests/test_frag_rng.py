"""The seeded fragment-position generator (stand-in for the reference's
wall-clock-seeded util.GetVectorEven, cmd/util/vectorutil.go:32-42): an
independent pure-Python restatement agrees bit for bit, and the points are
uniform in the ball."""
import numpy as np

from oracle.oracle import frag_point

MASK = (1 << 64) - 1
GOLDEN = 0x9E3779B97F4A7C15


def mix(z):
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK
    return z ^ (z >> 31)


def key(seed, parent, cycle):
    k = mix((seed + GOLDEN) & MASK)
    k = mix(k ^ ((parent * 0xD1B54A32D192ED03) & MASK))
    return mix(k ^ ((cycle * 0xAEF17502108EF2D9 + 0x632BE59BD9B4E019) & MASK))


def uniform(k, ctr):
    return (mix((k + (ctr + 1) * GOLDEN) & MASK) >> 11) * 2.0 ** -53


def py_point(seed, parent, cycle, cnt, c, radius):
    k = key(seed, parent, cycle)
    x = y = z = 0.0
    for a in range(85):
        base = cnt * 256 + 3 * a
        x = uniform(k, base) * 2 - 1
        y = uniform(k, base + 1) * 2 - 1
        z = uniform(k, base + 2) * 2 - 1
        if not (x * x + y * y + z * z > 1):
            break
    else:
        x = y = z = 0.0
    return (x * radius) + c[0], (y * radius) + c[1], (z * radius) + c[2]


def test_matches_python_restatement():
    for seed in (0, 1, 0xDEADBEEF):
        for parent in (0, 7, 123456789):
            for cycle in (0, 3, 1000):
                for cnt in (0, 1, 100):
                    c = (1.5, -2.25, 1e3)
                    assert frag_point(seed, parent, cycle, cnt, c, 0.9) == py_point(seed, parent, cycle, cnt, c, 0.9)


def test_uniform_in_ball():
    pts = np.array([frag_point(42, 5, 0, k, (0.0, 0.0, 0.0), 1.0) for k in range(101)] +
                   [frag_point(42, p, 1, 0, (0.0, 0.0, 0.0), 1.0) for p in range(3000)])
    r = np.sqrt((pts ** 2).sum(axis=1))
    assert np.all(r <= 1.0)
    # uniform in the ball: P(r <= 0.5) = 1/8, mean r = 3/4
    assert abs(np.mean(r <= 0.5) - 0.125) < 0.03
    assert abs(np.mean(r) - 0.75) < 0.02
    assert np.all(np.abs(pts.mean(axis=0)) < 0.06)
