"""Benchmark of the nbodygo compute cycle on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload plummer_disk|ensemble|uniform|plummer|disk]

A "step" is one compute cycle: force and collision detection, resolution,
integration, compaction.  The metric is pair interactions/s: N(N-1) per cycle,
with N taken at the start of the cycle (summed over the simulations of an
ensemble).

Default workload `plummer_disk`:

- N = 131,072 bodies: 65,536 in a Plummer sphere (a = 300, M = 1e16) plus
  65,536 disk bodies.
- Radii 0.1-0.5, subsume collisions, dt = 0.01, mixed precision.

Other workloads:

- `ensemble`: 512 independent simulations of 256-32,768 bodies in one
  context, 10 cycles per CUDA graph.
- `uniform`: N = 1,048,576.
- `plummer`: N = 16,384, FP64.
- `disk`: N = 1,000, FP64.

Timing:

- `value` is device time, taken with CUDA events on the stream the library
  runs on, with the collection resident in HBM.  L2 is flushed (a 512 MB
  write) before every timed cycle, or before every graph of cycles for the
  ensemble.
- `e2e` is the same metric through the C ABI with host buffers.  Every cycle
  (or graph) uploads the full body state from pinned host memory, runs it,
  and reads the full state back, timed on the host clock.

`--impl reference` times the CPU restatement of the reference's cycle
(oracle/), with every host thread, as the reference's worker pool would use
them.  On the default workload each step is one full cycle of the same
131,072-body collection (about 10 s on 16 Grace cores); the larger workloads
(ensemble, uniform, Barnes-Hut) are timed on a stated sample.

Under torchrun (N > 1) each rank runs on its own GPU.  The direct sum of one
collection is not sharded: each rank runs an independent replica.  The
ensemble's 512 independent collections are split across the ranks instead
(shard_collections), one job with no exchange.  `value` is the sum over ranks
of the work done, divided by the slowest rank's time.
"""
import argparse
import json
import os
import re
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "pair interactions/s, 1 GB300: mixed vs FP64 plain at <=1e-6 rel accel error"
UNIT = "interactions/s"
FLOPS_PER_PAIR = 20  # Nyland, Harris & Prins (GPU Gems 3, ch. 31) convention

# workload -> (precision, dt, description)
WORKLOADS = {
    "plummer_disk": ("mixed", 0.01, "Plummer a=300 M=1e16 + disk r 400-4000, radii 0.1-0.5, subsume"),
    "ensemble": ("mixed", 0.01, "512 sims, N log-uniform 256-32768, {uniform ball, Plummer, disk}, "
                                "none/elastic/subsume, 10 cycles per CUDA graph"),
    "uniform": ("mixed", 0.01, "uniform ball R=20000, m=1e10, radius 0.05, v~N(0,1), no collisions"),
    "plummer": ("fp64", 0.01, "Plummer a=200 M=1e16, radius 0.2, elastic"),
    "disk": ("fp64", 0.005, "central body 5e15 + disk r 100-1000, elastic"),
    "plummer_bh": ("fp64", 0.01, "Plummer a=200 M=1e16, 131072 bodies, radius 0.2, elastic; Barnes-Hut octree "
                                 "forces (theta 0.3, softening 1e-4, FP64), exact collisions"),
    "plummer_bh_mixed": ("mixed", 0.01, "Plummer a=200 M=1e16, 131072 bodies, radius 0.2, elastic; Barnes-Hut "
                                        "octree, mixed walk (FP32 terms), exact collisions"),
    "uniform_bh_mixed": ("mixed", 0.01, "uniform ball R=20000, m=1e10, radius 0.05, 1048576 bodies, no collisions; "
                                        "Barnes-Hut octree, mixed walk"),
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="plummer_disk", choices=sorted(WORKLOADS))
    ap.add_argument("--n-each", type=int, default=65536, help="plummer_disk: bodies per component")
    ap.add_argument("--bodies", type=int, default=None,
                    help="uniform, uniform_bh_mixed: bodies in the ball (default 1,048,576), e.g. a smaller case "
                         "for a profiler")
    ap.add_argument("--no-plain", action="store_true", help="skip the FP64 comparison run")
    ap.add_argument("--with-plain", action="store_true",
                    help="run the FP64 comparison on the uniform ball too (one FP64 force pass, ~2 min at 1M bodies)")
    ap.add_argument("--near-ppm", type=int, default=None,
                    help="mixed: near-pair radius factor in parts per million (library default 50000)")
    ap.add_argument("--chunks", type=int, default=None,
                    help="mixed: most chunks the pair work is cut into (library default 32 per resident CTA)")
    ap.add_argument("--p64-split-max", type=int, default=None,
                    help="plain FP64: largest capacity for the split pair pass (library default 65536)")
    ap.add_argument("--sort-interval", type=int, default=None,
                    help="mixed: cycles between Morton sorts of the i-tiles (library default 4)")
    ap.add_argument("--drift-cycles", type=int, default=0,
                    help="after the timed run, step a fresh copy of the workload this many cycles and report the "
                         "relative energy and momentum drift (untimed)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default kernel shape")
    ap.add_argument("--shape", type=int, default=None,
                    help="use this shape of the mixed pair kernel, or of the mixed Barnes-Hut walk (no autotune)")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Barrier / max / sum over ranks (torch.distributed) when WORLD_SIZE > 1:
    NCCL between GPUs, gloo when asked (the CPU tests of the replica path)."""

    def __init__(self, ws, local, backend="nccl"):
        self.ws = ws
        self.backend = backend
        if ws > 1:
            import torch
            import torch.distributed as td

            if backend == "nccl":
                torch.cuda.set_device(local)
            td.init_process_group(backend)
            self.td, self.torch = td, torch

    def barrier(self):
        if self.ws > 1:
            self.td.barrier()

    def _reduce(self, v, op):
        if self.ws == 1:
            return v
        dev = "cuda" if self.backend == "nccl" else "cpu"
        t = self.torch.tensor([float(v)], dtype=self.torch.float64, device=dev)
        self.td.all_reduce(t, op=op)
        return float(t.item())

    def max(self, v):
        return v if self.ws == 1 else self._reduce(v, self.td.ReduceOp.MAX)

    def sum(self, v):
        return v if self.ws == 1 else self._reduce(v, self.td.ReduceOp.SUM)

    def close(self):
        if self.ws > 1:
            self.td.destroy_process_group()


def aggregate(dist, interactions, t_ms):
    """Whole-job rate of N replicas: the work of all ranks over the slowest
    rank's time.  Returns (value per second, slowest ms, total work)."""
    t_max = dist.max(t_ms)
    work = dist.sum(interactions)
    return work / (t_max * 1e-3), t_max, work


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        fd, self.path = tempfile.mkstemp(prefix=f"nbg_clocks_gpu{gpu}_", suffix=".csv")
        os.close(fd)

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as fh:
            for line in fh:
                p = [x.strip() for x in line.split(",")]
                if len(p) < 9:
                    continue
                try:
                    sm.append(float(p[1]))
                    smax = float(p[2])
                except ValueError:
                    continue
                for nm, v in zip(names, p[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        try:
            os.unlink(self.path)
        except OSError:
            pass
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def traffic_from_profiles(workload, kernel="k_pair_mixed"):
    """DRAM bytes per launch of the pair kernel from the committed ncu summary
    (pair_mixed_<workload>.md, or pair_sym_<workload>.md for the symmetric
    kernel)."""
    stem = "pair_sym" if kernel == "k_pair_sym" else "pair_mixed"
    p = os.path.join(ROOT, "profiles", f"{stem}_{workload}.md")
    try:
        txt = open(p).read()
    except OSError:
        return None
    m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", txt)
    return float(m.group(1)) if m else None


def measured_hbm():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def shard_collections(sizes, ws):
    """The collections each of ws ranks runs: largest pair work n (n - 1)
    first, each to the rank with the least work so far (ties to the lower
    rank).  Deterministic, so every rank derives the same split without an
    exchange; every collection goes to exactly one rank."""
    load = [0] * ws
    shards = [[] for _ in range(ws)]
    for s in sorted(range(len(sizes)), key=lambda k: (-sizes[k] * (sizes[k] - 1), k)):
        r = min(range(ws), key=lambda q: (load[q], q))
        shards[r].append(s)
        load[r] += sizes[s] * (sizes[s] - 1)
    return [sorted(x) for x in shards]


def make_workload(name, n_each, rank, ws=1, bodies=None):
    """(list of body dicts, one per simulation) for a workload.  The ensemble
    is one job split across the ranks (its collections are independent);
    every other workload is one replica per rank with its own seed."""
    from nbodygo_gb300 import workloads as W

    seed_off = 1000 * rank
    if name == "plummer_disk":
        return [W.plummer_disk(n_each=n_each, seed=3 + seed_off)]
    if name == "ensemble":
        sims = W.ensemble(seed=5)
        if ws > 1:
            mine = shard_collections([len(b["x"]) for b in sims], ws)[rank]
            sims = [sims[k] for k in mine]
        return sims
    if name == "uniform":
        return [W.uniform_ball(seed=4 + seed_off) if bodies is None else W.uniform_ball(bodies, seed=4 + seed_off)]
    if name == "plummer":
        return [W.plummer(seed=2 + seed_off)]
    if name in ("plummer_bh", "plummer_bh_mixed"):
        return [W.plummer(131072, seed=2 + seed_off)]
    if name == "uniform_bh_mixed":
        return [W.uniform_ball(seed=4 + seed_off) if bodies is None else W.uniform_ball(bodies, seed=4 + seed_off)]
    return [W.disk(seed=1 + seed_off)]


def load(sim, sims):
    if len(sims) == 1:
        sim.set_bodies(sims[0])
    else:
        sim.set_collections(sims)


# workloads whose full collection the CPU restatement runs per timed cycle in
# seconds (plummer_disk: ~10 s per cycle on 16 Grace cores); the others are
# timed on a sample drawn from their own generator
CPU_FULL = ("plummer_disk", "plummer", "disk")


def config_of(workload, n0, nsims, ws):
    """The `config` object of a bench line: the workload, identical in both
    arms so their lines describe the same job."""
    prec, dt, desc = WORKLOADS[workload]
    return {"workload": f"{workload}: {n0} bodies in {nsims} simulation(s) ({desc}), dt={dt}",
            "n_bodies": n0, "n_sims": nsims, "dt": dt,
            "l2": "GPU arm: flushed (512 MB write) before every timed cycle"
                  + (" graph" if workload == "ensemble" else "") + "; CPU arm: not applicable",
            "parallelism": (f"collections split over {ws} ranks" if workload == "ensemble" and ws > 1
                            else f"replicas x{ws}")}


def cpu_sample(workload, n_each=65536):
    """(list of body sets, description): what the CPU restatement is timed on.
    The full workload where a cycle takes seconds (CPU_FULL), otherwise a
    bounded sample drawn from the workload's own generator."""
    from nbodygo_gb300 import workloads as W

    if workload in CPU_FULL:
        sims = make_workload(workload, n_each, 0)
        n = int(sum(len(b["x"]) for b in sims))
        return sims, f"{workload} with {n:,} bodies (the full workload)"
    if workload == "ensemble":
        sims, total = [], 0
        for b in W.ensemble(seed=5):
            if sims and total + len(b["x"]) > 49152:
                continue
            sims.append(b)
            total += len(b["x"])
            if total >= 32768:
                break
        return sims, f"{len(sims)} collections of the ensemble, {total:,} bodies"
    if workload == "uniform":
        return [W.uniform_ball(32768, seed=4)], "uniform ball of the same radius with 32,768 bodies (a sample)"
    return [W.plummer(32768, seed=2)], ("plummer with 32,768 bodies, Barnes-Hut (the reference's octree, "
                                        "built once per cycle; a sample)")


def cpu_cycles(workload, dt, warmup, steps, sample=None):
    """Times `steps` cycles of the CPU restatement on every body set of the
    workload's CPU sample, all host threads: (interactions, seconds,
    description)."""
    from oracle.oracle import OracleSim

    sets, what = sample or cpu_sample(workload)
    cores = os.cpu_count() or 1
    inter, t = 0, 0.0
    for b in sets:
        o = OracleSim(threads=cores)
        if "_bh" in workload:
            o.set_barnes_hut(True)
        o.set_bodies(b)
        for _ in range(warmup):
            o.step(dt, 1.0, 1)
        for _ in range(steps):
            t0 = time.perf_counter()
            info = o.step(dt, 1.0, 1)
            t += time.perf_counter() - t0
            inter += info["interactions"]
    return inter, t, what


def cpu_baseline_sample(workload, dt, n_each=65536):
    """CPU restatement of the reference cycle, all host threads: one cycle of
    the full workload where that takes seconds, else cycles of a sample."""
    cores = os.cpu_count() or 1
    sample = cpu_sample(workload, n_each)
    steps = 1 if sum(len(b["x"]) for b in sample[0]) > 10000 else 20
    inter, t, what = cpu_cycles(workload, dt, 0, steps, sample)
    return {"value": inter / t, "unit": UNIT, "cores": cores, "kind": "port",
            "full_workload": workload in CPU_FULL,
            "sample": f"{what}, {steps} cycle(s), {t:.2f} s; C restatement of the reference's Go cycle (oracle/)"}


def run_reference(args, ws, rank):
    """--impl reference: the CPU restatement of the reference's cycle (its
    worker-pool slicing over every host thread), each step one cycle of the
    workload.  Under torchrun only rank 0 runs."""
    if rank != 0:
        return 0
    prec, dt, desc = WORKLOADS[args.workload]
    cores = os.cpu_count() or 1
    sample = cpu_sample(args.workload, args.n_each)
    sets = sample[0]
    n = int(sum(len(b["x"]) for b in sets))
    full = args.workload in CPU_FULL
    total_int, total_t, what = cpu_cycles(args.workload, dt, args.warmup, args.steps, sample)
    v = total_int / total_t
    if full:
        config = config_of(args.workload, n, len(sets), ws)
    else:
        config = {"workload": f"{args.workload} sample: {n} bodies in {len(sets)} collection(s) ({desc})",
                  "n_bodies": n, "n_sims": len(sets), "dt": dt}
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total_t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": config,
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "full_workload": full,
                             "sample": f"{what}, one cycle per step; the C restatement of the reference's Go "
                                       "cycle (oracle/) with the worker-pool slicing"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


G_CONST = 6.673e-11  # cmd/globals/globals.go


def force_scale(torch, sims, idx, device):
    """For the bodies at flat indices idx: the sum over j of |f_ij| =
    G m_i m_j / d_ij^2 over the pairs the force pass sums (j in the same
    collection, j != i, j live, d > r_i + r_j: calcForceFrom's overlap skip,
    cmd/body/body.go:214-225), in FP64 on the GPU.  It is the scale of a
    body's force with no cancellation between terms."""
    out = np.zeros(len(idx))
    off = np.cumsum([0] + [len(b["x"]) for b in sims])
    idx = np.asarray(idx, dtype=np.int64)
    sim_of = np.searchsorted(off, idx, side="right") - 1
    for s in np.unique(sim_of):
        b = sims[s]
        live = (np.asarray(b["flags"]) & 0x11) == 0x01  # exists, not fragmenting
        T = {k: torch.as_tensor(np.asarray(b[k], dtype=np.float64), device=device) for k in ("x", "y", "z", "mass",
                                                                                             "radius")}
        mj = T["mass"] * torch.as_tensor(live, device=device)
        sel = np.nonzero(sim_of == s)[0]
        loc = idx[sel] - off[s]
        for a in range(0, len(loc), 64):
            li = torch.as_tensor(loc[a:a + 64], device=device)
            d2 = ((T["x"][None, :] - T["x"][li, None]) ** 2 + (T["y"][None, :] - T["y"][li, None]) ** 2
                  + (T["z"][None, :] - T["z"][li, None]) ** 2)
            far = d2.sqrt() > (T["radius"][None, :] + T["radius"][li, None])
            far[torch.arange(len(li), device=device), li] = False
            w = torch.where(far, mj[None, :] / torch.where(far, d2, torch.ones_like(d2)), torch.zeros_like(d2))
            out[sel[a:a + 64]] = (G_CONST * T["mass"][li] * w.sum(dim=1)).cpu().numpy()
    return out


def accuracy_block(torch, sims, fm, fp, device, limit=1e-6, top=2048):
    """Mixed forces fm against the FP64 forces fp (both (fx, fy, fz) over the
    flat body order).  Besides relative L2 and the plain per-body relative
    error, each body's error is normalised by the sum of the magnitudes of its
    terms, sum_j |f_ij|: in a dense core the terms cancel and |f_i| is far
    smaller than the terms the FP32 arithmetic rounds.  Since
    sum_j |f_ij| >= |f_i|, the normalised error of a body is at most its plain
    relative error, so the normalised error is computed for the `top` bodies
    with the largest plain error, and every other body is bounded by the
    largest plain error outside them."""
    mag = np.sqrt(fp[0] ** 2 + fp[1] ** 2 + fp[2] ** 2)
    err = np.sqrt((fm[0] - fp[0]) ** 2 + (fm[1] - fp[1]) ** 2 + (fm[2] - fp[2]) ** 2)
    num = np.sqrt(np.sum(err ** 2))
    den = np.sqrt(np.sum(mag ** 2))
    ok = np.nonzero(mag > 0)[0]
    rel = err[ok] / mag[ok]
    order = np.argsort(rel)[::-1]
    k = min(top, len(order))
    worst = ok[order[:k]]
    scale = force_scale(torch, sims, worst, device)
    norm = np.where(scale > 0, err[worst] / np.where(scale > 0, scale, 1.0), 0.0)
    rest = float(rel[order[k]]) if k < len(order) else 0.0
    max_norm = max(float(norm.max()) if k else 0.0, rest)
    by_norm = np.argsort(norm)[::-1][:8]
    rel_l2 = float(num / den)
    return {
        "rel_l2_vs_fp64": rel_l2, "max_rel": float(rel.max()), "median_rel": float(np.median(rel)),
        "p99_9_rel": float(np.quantile(rel, 0.999)), "bodies_above_1e-6_rel": int(np.sum(rel > 1e-6)),
        "max_rel_normalised": max_norm,
        "normalised": f"|f_mixed - f_fp64| / sum_j |f_ij| (FP64 term magnitudes) for the {k} bodies with the "
                      f"largest plain relative error; every other body is bounded by the plain relative error "
                      f"{rest:.3e} of the next one",
        "worst_bodies": [{"index": int(worst[q]), "rel": float(err[worst[q]] / mag[worst[q]]),
                          "normalised": float(norm[q]), "cancellation": float(mag[worst[q]] / scale[q])}
                         for q in by_norm],
        "gate": {"limit": limit, "rel_l2_pass": rel_l2 <= limit, "max_normalised_pass": max_norm <= limit,
                 "reading": "relative L2 over all bodies, and every body's error relative to the sum of its "
                            "terms' magnitudes"},
        "reference": "plain FP64 GPU forces (bit-identical to the oracle)"}


def pinned_like(torch, st, extra):
    out, keep = {}, []
    for k, v in st.items():
        tdt = torch.int32 if v.dtype == np.uint32 else getattr(torch, str(v.dtype))
        t = torch.empty(len(v) + extra, dtype=tdt, pin_memory=True)
        keep.append(t)
        arr = t.numpy().view(v.dtype)
        arr[: len(v)] = v
        out[k] = arr
    return out, keep


def main():
    args = parse()
    ws, rank, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, ws, rank)

    from nbodygo_gb300 import build as B

    B.build()
    import torch

    from nbodygo_gb300 import _abi as A
    from nbodygo_gb300.api import Simulation, probe_peaks

    prec, DT, desc = WORKLOADS[args.workload]
    dist = Dist(ws, local)
    torch.cuda.set_device(local)
    # a dedicated stream: the library's kernels, the L2 flush and the timing
    # events are ordered on it (torch's default stream is the legacy NULL
    # stream, which nbg_set_stream does not take)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sims = make_workload(args.workload, args.n_each, rank, ws, args.bodies)
    sharded = args.workload == "ensemble" and ws > 1
    n0 = int(sum(len(b["x"]) for b in sims))
    chunk = 10 if args.workload == "ensemble" else 1
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    bh = "_bh" in args.workload
    sim = Simulation(prec, device=local, capacity=n0 + 4096)
    sim.set_stream(stream.cuda_stream)
    sim.set_option(A.OPT_GRAPH_CYCLES, chunk)
    if bh:
        sim.set_option(A.OPT_BARNES_HUT, 1)
    if args.sort_interval is not None:
        sim.set_option(A.OPT_SORT_INTERVAL, args.sort_interval)
    if args.near_ppm is not None:
        sim.set_option(A.OPT_NEAR_PPM, args.near_ppm)
    if args.p64_split_max is not None:
        sim.set_option(A.OPT_P64_SPLIT_MAX, args.p64_split_max)
    if args.chunks is not None:
        sim.set_option(A.OPT_SPLIT, args.chunks)
    load(sim, sims)
    tuned = None
    if prec == "mixed" and args.shape is not None:
        # Barnes-Hut: the shape of the mixed walk (CTAs per SM it is built for)
        sim.set_option(A.OPT_BH_SHAPE if bh else A.OPT_MIX_SHAPE, args.shape)
        tuned = {"shape": args.shape, "pair_kernel_ms": None, "candidates": 3 if bh else A.MIX_SHAPES,
                 "fixed": True, "kernel": "k_bh_force_mixed" if bh else
                 "k_pair_sym" if args.shape in (A.MIX_SYM, A.MIX_SYM + 1) else "k_pair_mixed"}
    elif prec == "mixed" and not args.no_autotune and not bh:
        shape, tms = sim.autotune()
        tuned = {"shape": shape, "pair_kernel_ms": tms, "candidates": A.MIX_SHAPES}
    sim.step(DT, 1.0, max(args.warmup, 3) * chunk)

    # ---- timed: K cycles, L2 flushed before each chunk, device time ----
    nchunks = max(1, args.steps // chunk)
    clocks = Clocks(local)
    clocks.start()
    dist.barrier()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nchunks)]
    interactions, cycles = 0, 0
    for k in range(nchunks):
        flush.fill_(float(k))
        ev[k][0].record(stream)
        info = sim.step(DT, 1.0, chunk)
        ev[k][1].record(stream)
        interactions += info["interactions"]
        cycles += info["steps_done"]
    torch.cuda.synchronize()
    dist.barrier()
    clk = clocks.stop()
    per_chunk = [a.elapsed_time(b) for a, b in ev]
    t_ms = sum(per_chunk)
    value, t_max, work = aggregate(dist, interactions, t_ms)
    # the job's size: one replica's, or the whole ensemble split over ranks
    job_bodies = int(dist.sum(n0)) if sharded else n0
    job_sims = int(dist.sum(len(sims))) if sharded else len(sims)

    # ---- pair-kernel time (library timing mode, same stream) ----
    sim.enable_timing(True)
    flush.fill_(1.0)
    tsteps = min(cycles, 10)
    info_t = sim.step(DT, 1.0, tsteps)
    tm = sim.timing()
    sim.enable_timing(False)
    inter_t = info_t["interactions"] / max(1, info_t["steps_done"])
    bh_terms_t = info_t["bh_terms"] / max(1, info_t["steps_done"])
    pair_ms = tm["pair_ms"] / max(1, tm["pair_launches"])
    launches = tm["kernel_launches"] / max(1, info_t["steps_done"]) * cycles

    # ---- e2e through the C ABI with host buffers ----
    st = sim.state()
    counts = sim.sim_counts()
    pinned, keep = pinned_like(torch, st, 4096)
    n_h = len(st["x"])
    e2e_int, e2e_t, h2d, d2h, e2e_chunks = 0, 0.0, 0, 0, max(1, min(nchunks, 10))
    # each call returns once its copies and cycles are done, so the host
    # clock between the calls splits the step into its phases
    phase = {"load": 0.0, "step": 0.0, "read": 0.0}
    per_call = []
    # call 0 is an untimed warm-up of the host path (first use of the pinned
    # arrays by the copy kernel)
    for k in range(e2e_chunks + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        host = {f: a[:n_h] for f, a in pinned.items()}
        if len(counts) == 1:
            sim.set_bodies(host)
        else:
            sim.set_collections_flat(host, counts)
        t1 = time.perf_counter()
        info = sim.step(DT, 1.0, chunk)
        t2 = time.perf_counter()
        out = sim.state(out=pinned)
        # several collections: their sizes after the step; one collection:
        # the length of what was read
        counts = sim.sim_counts() if len(counts) > 1 else [len(out["x"])]
        t3 = time.perf_counter()
        n_h = len(out["x"])
        per_call.append(round(1e3 * (t3 - t0), 3))
        if k == 0:
            continue
        h2d += sum(a.nbytes for a in host.values())
        phase["load"] += t1 - t0
        phase["step"] += t2 - t1
        phase["read"] += t3 - t2
        e2e_t += t3 - t0
        d2h += sum(a.nbytes for a in out.values())
        e2e_int += info["interactions"]
    e2e = {"value": dist.sum(e2e_int) / dist.max(e2e_t), "unit": UNIT,
           "h2d_bytes_per_step": int(h2d // (e2e_chunks * chunk)),
           "d2h_bytes_per_step": int(d2h // (e2e_chunks * chunk)),
           "phases_ms_per_call": {k: round(1e3 * v / e2e_chunks, 3) for k, v in phase.items()},
           "ms_per_call": per_call[1:], "warmup_call_ms": per_call[0],
           "path": "nbg_set_bodies / nbg_set_collections (full state, pinned host, collections one after another) "
                   "+ nbg_step + nbg_get_state "
                   "(full state)" + (f", {chunk} cycles per call" if chunk > 1 else "")}

    # ---- FP32 / FP64 peaks, plain FP64 comparison, accuracy ----
    f32, f64, mhz = probe_peaks(local)
    result_extra = {}
    plain_ok = (prec == "mixed" and (args.workload != "uniform" or args.with_plain) and not bh
                and not args.no_plain and rank == 0)
    if plain_ok:
        # above this size the plain comparison is one timed FP64 force pass
        # (no stepping, no O(N^2) FP64 energy sums)
        big = n0 > 262144
        plain = Simulation("fp64", device=local, capacity=n0 + 4096)
        plain.set_stream(stream.cuda_stream)
        load(plain, sims)
        pe0, pe1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        pe0.record(stream)
        fp = plain.force_pass()
        pe1.record(stream)
        torch.cuda.synchronize()
        force_ms = pe0.elapsed_time(pe1)
        mixed0 = Simulation("mixed", device=local, capacity=n0 + 4096)
        mixed0.set_stream(stream.cuda_stream)
        if args.near_ppm is not None:
            mixed0.set_option(A.OPT_NEAR_PPM, args.near_ppm)
        if tuned is not None:
            # the forces of the kernel shape that was timed
            mixed0.set_option(A.OPT_MIX_SHAPE, tuned["shape"])
        load(mixed0, sims)
        fm = mixed0.force_pass()
        accuracy = accuracy_block(torch, sims, fm, fp, f"cuda:{local}")
        accuracy["kernel_shape"] = tuned["shape"] if tuned is not None else 0
        if big:
            pairs = sum(len(b["x"]) * (len(b["x"]) - 1) for b in sims)
            plain_rate = pairs / (1e-3 * force_ms)
            drift = {"skipped": f"{n0} bodies: the FP64 energy sum is O(N^2) in FP64"}
            result_extra["plain_fp64"] = {
                "value": plain_rate, "unit": UNIT, "ms_per_step": None, "force_pass_ms": force_ms,
                "pair_kernel_ms": force_ms,
                "roofline_frac_fp64": plain_rate * FLOPS_PER_PAIR / f64 if f64 else None,
                "steps": 0, "timed": "one FP64 force pass (pair kernel and set-up), CUDA events"}
        else:
            # energy over the same cycles from the same state, both forms
            e0 = sum(plain.energy()[:2])
            plain.enable_timing(True)
            pi = plain.step(DT, 1.0, 2)
            ptm = plain.timing()
            plain.enable_timing(False)
            mixed0.step(DT, 1.0, 2)
            ep, em = sum(plain.energy()[:2]), sum(mixed0.energy()[:2])
            p_ms = (ptm["pair_ms"] + ptm["other_ms"]) / max(1, ptm["pair_launches"])
            plain_rate = pi["interactions"] / (1e-3 * (ptm["pair_ms"] + ptm["other_ms"]))
            drift = {"fp64": abs(ep - e0) / abs(e0), "mixed": abs(em - e0) / abs(e0),
                     "mixed_vs_fp64": abs(em - ep) / abs(e0)}
            result_extra["plain_fp64"] = {
                "value": plain_rate, "unit": UNIT, "ms_per_step": p_ms,
                "pair_kernel_ms": ptm["pair_ms"] / max(1, ptm["pair_launches"]),
                "roofline_frac_fp64": plain_rate * FLOPS_PER_PAIR / f64 if f64 else None,
                "steps": 2}
        result_extra["mixed_over_plain"] = value / plain_rate / ws if plain_rate else None
        accuracy["energy_drift_2_cycles"] = drift
        result_extra["accuracy"] = accuracy
        plain.close()
        mixed0.close()

    if args.drift_cycles > 0 and rank == 0:
        ds = Simulation(prec, device=local, capacity=n0 + 4096)
        ds.set_stream(stream.cuda_stream)
        ds.set_option(A.OPT_GRAPH_CYCLES, 10)
        if bh:
            ds.set_option(A.OPT_BARNES_HUT, 1)
        load(ds, sims)
        ke0, pe0_, p0 = ds.energy()
        st0 = ds.state()
        pscale = float(np.sum(st0["mass"] * np.sqrt(st0["vx"] ** 2 + st0["vy"] ** 2 + st0["vz"] ** 2)))
        done, events = 0, 0
        while done < args.drift_cycles:
            k = min(10, args.drift_cycles - done)
            di = ds.step(DT, 1.0, k)
            done += di["steps_done"]
            events += di.get("events", 0)
        ke1, pe1_, p1 = ds.energy()
        st1 = ds.state()
        result_extra["drift"] = {
            "cycles": done, "form": prec, "bodies_start": n0, "bodies_end": int(len(st1["x"])), "events": events,
            "mass_rel": abs(float(np.sum(st1["mass"])) - float(np.sum(st0["mass"]))) / float(np.sum(st0["mass"])),
            "energy_rel": abs((ke1 + pe1_) - (ke0 + pe0_)) / abs(ke0 + pe0_),
            "momentum_rel": float(np.sqrt(sum((a - b) ** 2 for a, b in zip(p1, p0)))) / pscale,
            "note": "mass is conserved; energy and momentum are not: a subsume keeps the absorbing body's velocity "
                    "and an elastic collision with fragments moves mass between bodies as the reference does"}
        ds.close()

    if bh:
        # the whole tree pass (build, walk, collision query) against the FP64
        # peak, counting only the point-mass terms the walk summed
        achieved = bh_terms_t * FLOPS_PER_PAIR / (pair_ms * 1e-3) / 1e12
        if prec == "mixed":
            peak, kernel, bound = f32 / 1e12, "k_bh_* (tree build + k_bh_force_mixed + k_bh_collide)", "fp32_fma"
            peak_src = f"FFMA-chain probe on this GPU at {mhz:.0f} MHz (MEASURED_PEAKS.json has no FP32 figure)"
        else:
            peak, kernel, bound = f64 / 1e12, "k_bh_* (tree build + k_bh_force + k_bh_collide)", "fp64_fma"
            peak_src = f"DFMA-chain probe on this GPU at {mhz:.0f} MHz (MEASURED_PEAKS.json has no FP64 figure)"
    elif prec == "mixed":
        achieved = inter_t * FLOPS_PER_PAIR / (pair_ms * 1e-3) / 1e12
        # shapes MIX_SYM and MIX_SYM + 1 are the symmetric kernel
        sym = tuned is not None and tuned.get("shape") in (A.MIX_SYM, A.MIX_SYM + 1)
        peak, kernel, bound = f32 / 1e12, "k_pair_sym" if sym else "k_pair_mixed", "fp32_fma"
        peak_src = f"FFMA-chain probe on this GPU at {mhz:.0f} MHz (MEASURED_PEAKS.json has no FP32 figure)"
    else:
        achieved = inter_t * FLOPS_PER_PAIR / (pair_ms * 1e-3) / 1e12
        peak, kernel, bound = f64 / 1e12, "k_pair_fp64", "fp64_fma"
        peak_src = f"DFMA-chain probe on this GPU at {mhz:.0f} MHz (MEASURED_PEAKS.json has no FP64 figure)"
    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline_sample(args.workload, DT, args.n_each)
    sim.close()
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": cycles,
            "warmup": args.warmup, "ms_per_step": t_max / cycles,
            "ms_per_chunk_each": [round(v, 4) for v in per_chunk], "cycles_per_chunk": chunk,
            "higher_is_better": True, "scaling": "strong" if sharded else "weak", "vs_baseline": None,
            "dtype": "fp32 pair terms, fp64 state" if prec == "mixed" else "f64",
            "data": "synthetic",
            "config": config_of(args.workload, job_bodies, job_sims, ws),
            "form": {"precision": prec, "barnes_hut": bh,
                     "sort_interval": (args.sort_interval or 4) if prec == "mixed" and not bh else None},
            "e2e": e2e,
            "gpu_launches": int(launches),
            "roofline": {"bound": bound, "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak if peak else None,
                         "traffic": traffic_from_profiles(args.workload, kernel) if prec == "mixed" else None,
                         "kernel": kernel, "flops_per_pair": FLOPS_PER_PAIR, "pair_kernel_ms": pair_ms,
                         "peak_source": peak_src},
            "peaks": {"fp32_tflops": f32 / 1e12, "fp64_tflops": f64 / 1e12, "probe_sm_mhz": mhz,
                      "hbm_gbs_measured": measured_hbm().get("hbm_gbs")},
            "clocks": clk,
            "cpu_baseline": cpu,
            "autotune": tuned,
        }
        if bh:
            line["barnes_hut"] = {
                "point_mass_terms_per_cycle": bh_terms_t,
                "terms_per_body": bh_terms_t / max(1, n0),
                "tree_pass_ms": pair_ms,
                "note": "value counts N(N-1) per cycle, the direct sum the tree replaces; the roofline counts "
                        "the terms the walk summed"}
        line.update(result_extra)
        print(json.dumps(line), flush=True)
    dist.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
