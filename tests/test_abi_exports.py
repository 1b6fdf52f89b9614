"""libnbgpu.so loads without a GPU and exports every function include/*.h
declares; the ctypes binding declares exactly those."""
import ctypes
import glob
import os
import re

from nbodygo_gb300 import _abi, api

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DECL = re.compile(r"^\s*(?:const\s+)?(?:int|void|char|double|int64_t)\s*\*?\s*(nbg_\w+)\s*\(", re.M)


def declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        names |= set(DECL.findall(open(h).read()))
    return names


def test_header_declares_functions():
    names = declared()
    for must in ("nbg_create", "nbg_destroy", "nbg_set_bodies", "nbg_apply_edits", "nbg_step", "nbg_get_state",
                 "nbg_get_renderables", "nbg_get_events", "nbg_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(api.LIB_PATH)
    missing = [n for n in sorted(declared()) if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_binding_covers_header():
    lib = ctypes.CDLL(api.LIB_PATH)
    bound = set(_abi.declare(lib))
    assert bound == declared(), f"header-only: {declared() - bound}, binding-only: {bound - declared()}"


def test_struct_sizes_match_header_layout():
    # nbg_soa: 24 pointers; nbg_edit: 8 + 4 + 4 + 10 doubles + 2 ints
    assert ctypes.sizeof(_abi.NbgSoa) == 24 * ctypes.sizeof(ctypes.c_void_p)
    assert ctypes.sizeof(_abi.NbgEdit) == 8 + 4 + 4 + 80 + 8
    assert ctypes.sizeof(_abi.NbgStepInfo) == 9 * 8
    assert ctypes.sizeof(_abi.NbgRenderable) == 32
    assert ctypes.sizeof(_abi.NbgEvent) == 24
