"""Shared helpers of the parity tests."""
import numpy as np

from nbodygo_gb300 import _abi as A

STATE_FIELDS = ("id", "x", "y", "z", "vx", "vy", "vz", "radius", "mass", "frag_factor", "frag_step",
                "collision", "flags", "r", "fx", "fy", "fz", "frag_radius", "frag_new_radius", "frag_mass",
                "frag_fragments", "frag_cx", "frag_cy", "frag_cz")


def assert_states_identical(got, exp, fields=STATE_FIELDS, where=""):
    assert len(got["x"]) == len(exp["x"]), f"{where}: body count {len(got['x'])} != {len(exp['x'])}"
    for f in fields:
        a, b = np.asarray(got[f]), np.asarray(exp[f])
        if a.dtype.kind == "f":
            same = (a.view(np.uint64) == b.view(np.uint64)) | (np.isnan(a) & np.isnan(b))
        else:
            same = a == b
        if not np.all(same):
            k = int(np.flatnonzero(~same)[0])
            raise AssertionError(f"{where}: field {f} differs first at body {k}: {a[k]!r} != {b[k]!r}")


def assert_events_identical(got, exp, where=""):
    assert len(got) == len(exp), f"{where}: {len(got)} events != {len(exp)}"
    for f in ("id1", "id2", "type"):
        assert np.array_equal(got[f], exp[f]), f"{where}: event field {f} differs"


def body_set(rows, behavior=A.ELASTIC):
    """Bodies from a list of dicts (x, y, z, vx, vy, vz, mass, radius, ...)."""
    n = len(rows)
    b = {f: np.zeros(n, dtype=A.FIELD_DTYPES[f]) for f in
         ("id", "x", "y", "z", "vx", "vy", "vz", "radius", "mass", "frag_factor", "frag_step", "collision", "flags")}
    b["id"][:] = np.arange(n)
    b["flags"][:] = A.F_EXISTS
    b["collision"][:] = behavior
    for k, row in enumerate(rows):
        for key, v in row.items():
            b[key][k] = v
    return b


def rel_l2(a, b):
    num = np.sqrt(sum(np.sum((x - y) ** 2) for x, y in zip(a, b)))
    den = np.sqrt(sum(np.sum(y ** 2) for y in b))
    return num / den
