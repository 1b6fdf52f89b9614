"""Builds libnbgpu.so (CUDA, sm_103a) in the source tree, and the CPU oracle.

    python -m nbodygo_gb300.build            # build what is out of date
    python -m nbodygo_gb300.build --force    # rebuild everything

The translation units compile in parallel.  k_cycle.cu and k_bh.cu are
compiled with --fmad=false: their FP64 arithmetic must round after every
operation to match the reference's Go code (and the oracle, compiled with
-ffp-contract=off).
"""
import argparse
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libnbgpu.so")
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "libnbg_oracle.so")
# the same oracle with the platform libm's sin/cos/tan/asin/acos/atan2 in
# place of nbg_math.h: bounds the effect of that substitution (tests only)
ORACLE_LIBM_LIB = os.path.join(ORACLE_DIR, "libnbg_oracle_libm.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
               "-Xcompiler", "-ffp-contract=off", "-I", CSRC, "-I", os.path.join(ROOT, "include")]
UNITS = {
    "k_cycle.cu": ["--fmad=false", "-DNBG_NO_FMAD"],
    "k_bh.cu": ["--fmad=false", "-DNBG_NO_FMAD"],
    "k_mixed.cu": [],
    "k_sort.cu": [],
    "k_probe.cu": [],
    "nbg_api.cu": [],
    "nbg_noalloc.cu": [],
}
HEADERS = ["nbg_internal.cuh", "nbg_math.h", "nbg_shared.h"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _mtime(p):
    try:
        return os.path.getmtime(p)
    except OSError:
        return -1.0


def _stale(target, deps):
    t = _mtime(target)
    return t < 0 or any(_mtime(d) > t for d in deps)


def build_oracle(force=False, verbose=False):
    src = os.path.join(ORACLE_DIR, "nbg_oracle.c")
    deps = [src, os.path.join(ORACLE_DIR, "nbg_oracle.h"), os.path.join(ROOT, "include", "nbgpu.h"), __file__]
    deps += [os.path.join(CSRC, h) for h in ("nbg_math.h", "nbg_shared.h")]
    procs = []
    for lib, defs in ((ORACLE_LIB, []), (ORACLE_LIBM_LIB, ["-DNBG_ORACLE_LIBM"])):
        if not force and not _stale(lib, deps):
            continue
        cmd = [os.environ.get("CC", "gcc"), "-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
               "-shared", "-pthread", "-D_GNU_SOURCE"] + defs + [src, "-o", lib, "-lm"]
        if verbose:
            print(" ".join(cmd))
        procs.append((cmd, subprocess.Popen(cmd)))
    for cmd, p in procs:
        if p.wait() != 0:
            raise RuntimeError("oracle build failed: " + " ".join(cmd))
    return ORACLE_LIB


def build_lib(force=False, verbose=False, ptxas_verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "nbgpu.h")]
    objs, procs = [], []
    for unit, flags in UNITS.items():
        src = os.path.join(CSRC, unit)
        obj = os.path.join(BUILD, unit.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs + [__file__]):
            cmd = [_nvcc()] + ARCH + NVCC_COMMON + flags + ["-c", src, "-o", obj]
            if ptxas_verbose:
                cmd += ["-Xptxas", "-v"]
            if verbose:
                print(" ".join(cmd))
            procs.append((unit, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    failed = []
    for unit, p in procs:
        out, _ = p.communicate()
        if out and (verbose or ptxas_verbose or p.returncode != 0):
            print(f"--- {unit}\n{out}")
        if p.returncode != 0:
            failed.append(unit)
    if failed:
        raise RuntimeError("nvcc failed for " + ", ".join(failed))
    if force or procs or _stale(LIB, objs):
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True)
    return LIB


def build(force=False, verbose=False, ptxas_verbose=False):
    build_oracle(force=force, verbose=verbose)
    return build_lib(force=force, verbose=verbose, ptxas_verbose=ptxas_verbose)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    ap.add_argument("--ptxas", action="store_true", help="print register / spill / smem usage")
    a = ap.parse_args(argv)
    build(force=a.force, verbose=a.verbose, ptxas_verbose=a.ptxas)
    return 0


if __name__ == "__main__":
    sys.exit(main())
