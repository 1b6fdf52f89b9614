"""The C++ host mirror (include/nbodygo.hpp) against the reference's own Go
tests of the body collection and the runner, restated in tests/cpp/test_mirror.cpp.

The program is compiled with g++ and linked to libnbgpu.so.  Without a GPU
only its host part runs (ApplyMods, the parsing helpers and the CSV loader,
cmd/body/body_test.go:9-47, cmd/globals/globals.go:41-102,
cmd/sim/fromcsv.go:46-131); on a GPU every test runs through the C ABI.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "nbodygo_gb300")


def _compile(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "test_mirror")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "test_mirror.cpp"), "-L", LIBDIR, "-lnbgpu",
           "-Wl,-rpath," + LIBDIR, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _run(exe, mode, timeout):
    r = subprocess.run([exe, mode], capture_output=True, text=True, timeout=timeout, cwd=os.path.dirname(exe))
    assert r.returncode == 0 and r.stdout.strip().endswith("PASSED"), r.stdout + r.stderr
    return r.stdout


def test_mirror_host_part(tmp_path):
    out = _run(_compile(tmp_path), "host", 60)
    assert "ok   TestMod" in out and "ok   TestParse" in out and "ok   TestFromCsv" in out


@pytest.mark.gpu
def test_mirror_against_reference_tests(tmp_path):
    out = _run(_compile(tmp_path), "gpu", 600)
    for name in ("TestInitSize", "TestRemove", "TestGetByID", "TestGetByName", "TestModByID",
                 "TestModByIDNoMatch", "TestModByName", "TestModByClass", "TestAdds", "TestRunnerSetters",
                 "TestRunnerBarnesHut", "TestRunnerCycle", "TestRunnerSnapshot"):
        assert "ok   " + name in out, out
