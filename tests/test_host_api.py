"""Host-side logic of the Python API that needs no GPU."""
import numpy as np

from nbodygo_gb300.api import _adjacent


def test_adjacent_parts_become_one_view():
    buf = np.arange(10.0)
    sims = [{"x": buf[0:3]}, {"x": buf[3:7]}, {"x": buf[7:10]}]
    v = _adjacent(sims, "x")
    assert np.shares_memory(v, buf) and np.array_equal(v, buf)


def test_adjacent_views_of_a_byte_buffer():
    raw = np.zeros(80, dtype=np.uint8)
    f = raw.view(np.float64)
    f[:] = np.arange(10)
    v = _adjacent([{"x": f[:4]}, {"x": f[4:]}], "x")
    assert np.shares_memory(v, raw) and np.array_equal(v, np.arange(10.0))


def test_non_adjacent_parts_are_concatenated():
    buf = np.arange(10.0)
    v = _adjacent([{"x": buf[0:3]}, {"x": buf[4:7]}], "x")
    assert not np.shares_memory(v, buf)
    assert np.array_equal(v, [0, 1, 2, 4, 5, 6])
    v = _adjacent([{"x": buf[3:6]}, {"x": buf[0:3]}], "x")  # adjacent, wrong order
    assert np.array_equal(v, [3, 4, 5, 0, 1, 2])
    v = _adjacent([{"x": np.ones(2)}, {"x": np.zeros(2, dtype=np.float32)}], "x")
    assert np.array_equal(v, [1, 1, 0, 0])
