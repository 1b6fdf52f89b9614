"""The guided cut of the mixed pair work into chunks (nbg_internal.cuh),
checked on the host: built with nvcc as a host program, no GPU needed."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_chunk_cut_covers_every_unit(tmp_path):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if nvcc is None:
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "chunk_cut")
    cmd = [nvcc, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "nbodygo_gb300", "csrc"), "-I",
           os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp", "chunk_cut.cu"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "bad 0" in r.stdout
