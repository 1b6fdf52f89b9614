"""Benchmark of the nbodygo compute cycle on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (one "step" = one compute cycle: force + collision detection,
resolution, integration, compaction): `plummer_disk`, N = 131,072 bodies
(65,536 Plummer a=300 M=1e16 + 65,536 disk bodies, radii 0.1-0.5, subsume,
dt = 0.01), mixed precision.  Metric: pair interactions/s (N(N-1) per cycle,
N at the start of the cycle).

`value` is device time (CUDA events on the stream the library runs on) with
the collection resident in HBM; L2 is flushed (a 512 MB write) before every
timed cycle.  `e2e` is the same metric through the C ABI with host buffers:
every cycle uploads the full body state from pinned host memory
(nbg_set_bodies), runs nbg_step and reads the full state back
(nbg_get_state), timed on the host clock.

`--impl reference` times the CPU restatement of the reference's cycle
(oracle/, with every host thread as the reference's worker pool would use)
on a 32,768-body sample of the same distribution per step.

Under torchrun (N > 1) each rank runs an independent replica on its own GPU
(the direct sum of one collection is not sharded: replicas only); value is the
sum over ranks of the work done divided by the slowest rank's time.
"""
import argparse
import json
import os
import re
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "pair interactions/s, 1 GB300: mixed vs FP64 plain at <=1e-6 rel accel error"
UNIT = "interactions/s"
WORKLOAD = "plummer_disk"
DT = 0.01
FLOPS_PER_PAIR = 20  # Nyland, Harris & Prins (GPU Gems 3, ch. 31) convention


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n-each", type=int, default=65536, help="bodies per component (default: the workload)")
    ap.add_argument("--no-plain", action="store_true", help="skip the FP64 comparison run")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Barrier / max-reduction over ranks (torch.distributed) when WORLD_SIZE > 1."""

    def __init__(self, ws, local):
        self.ws = ws
        self.pg = None
        if ws > 1:
            import torch
            import torch.distributed as td

            torch.cuda.set_device(local)
            td.init_process_group("nccl")
            self.td, self.torch = td, torch

    def barrier(self):
        if self.ws > 1:
            self.td.barrier()

    def max(self, v):
        if self.ws == 1:
            return v
        t = self.torch.tensor([float(v)], device="cuda")
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v):
        if self.ws == 1:
            return v
        t = self.torch.tensor([float(v)], device="cuda")
        self.td.all_reduce(t, op=self.td.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.td.destroy_process_group()


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_gpu{gpu}.csv")

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
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
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def traffic_from_profiles():
    """DRAM bytes per launch of the mixed pair kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "pair_mixed_plummer_disk.md")
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


def cpu_baseline_sample(n_each_sample=16384, steps=1):
    """CPU restatement of the reference cycle, all host threads, on a sample."""
    from nbodygo_gb300 import workloads as W
    from oracle.oracle import OracleSim

    cores = os.cpu_count() or 1
    b = W.plummer_disk(n_each=n_each_sample, seed=3)
    o = OracleSim(threads=cores)
    o.set_bodies(b)
    t0 = time.perf_counter()
    info = o.step(DT, 1.0, steps)
    t = time.perf_counter() - t0
    return {"value": info["interactions"] / t, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"plummer_disk with {2 * n_each_sample} bodies, {steps} cycle(s), {t:.2f} s"}


def run_reference(args, ws, rank):
    """--impl reference: the CPU restatement, timed per cycle on a sample."""
    if rank != 0:
        return 0
    from nbodygo_gb300 import workloads as W
    from oracle.oracle import OracleSim

    cores = os.cpu_count() or 1
    n_each = 16384
    b = W.plummer_disk(n_each=n_each, seed=3)
    o = OracleSim(threads=cores)
    o.set_bodies(b)
    for _ in range(args.warmup):
        o.step(DT, 1.0, 1)
    total_int, total_t = 0, 0.0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        info = o.step(DT, 1.0, 1)
        total_t += time.perf_counter() - t0
        total_int += info["interactions"]
    v = total_int / total_t
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total_t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": f"{WORKLOAD} sample: {2 * n_each} bodies (full workload: 131,072)",
                       "n_bodies": 2 * n_each, "dt": DT, "collision": "subsume"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"plummer_disk with {2 * n_each} bodies per cycle; the C restatement of "
                                       "the reference's Go cycle (oracle/), worker-pool slicing"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    ws, rank, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, ws, rank)

    from nbodygo_gb300 import build as B

    B.build()
    import torch

    from nbodygo_gb300 import _abi as A
    from nbodygo_gb300 import workloads as W
    from nbodygo_gb300.api import Simulation, probe_peaks

    dist = Dist(ws, local)
    torch.cuda.set_device(local)
    # a dedicated stream: the library's kernels, the L2 flush and the timing
    # events are ordered on it (torch's default stream is the legacy NULL
    # stream, which nbg_set_stream does not take)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    bodies = W.plummer_disk(n_each=args.n_each, seed=3 + 1000 * rank)
    n0 = len(bodies["x"])
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    sim = Simulation("mixed", device=local, capacity=n0 + 4096)
    sim.set_stream(stream.cuda_stream)
    sim.set_bodies(bodies)
    for _ in range(max(args.warmup, 3)):
        sim.step(DT, 1.0, 1)

    # ---- timed: K cycles, L2 flushed before each, device time ----
    clocks = Clocks(local)
    clocks.start()
    dist.barrier()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    interactions = 0
    for k in range(args.steps):
        flush.fill_(float(k))
        ev[k][0].record(stream)
        info = sim.step(DT, 1.0, 1)
        ev[k][1].record(stream)
        interactions += info["interactions"]
    torch.cuda.synchronize()
    dist.barrier()
    clk = clocks.stop()
    per_step = [a.elapsed_time(b) for a, b in ev]
    t_ms = sum(per_step)
    t_max = dist.max(t_ms)
    work = dist.sum(interactions)
    value = work / (t_max * 1e-3)

    # ---- pair-kernel time (library timing mode, same stream) ----
    sim.enable_timing(True)
    flush.fill_(1.0)
    info_t = sim.step(DT, 1.0, args.steps)
    tm = sim.timing()
    sim.enable_timing(False)
    n_now = info_t["interactions"] / max(1, info_t["steps_done"])
    pair_ms = tm["pair_ms"] / max(1, tm["pair_launches"])
    launches = tm["kernel_launches"]

    # ---- e2e through the C ABI with host buffers ----
    st = sim.state()
    pinned, keep = {}, []
    for k, v in st.items():
        tdt = torch.int32 if v.dtype == np.uint32 else getattr(torch, str(v.dtype))
        t = torch.empty(len(v) + 4096, dtype=tdt, pin_memory=True)
        keep.append(t)
        arr = t.numpy().view(v.dtype)
        arr[: len(v)] = v
        pinned[k] = arr
    host = {k: a[: len(st["x"])] for k, a in pinned.items()}
    e2e_int, e2e_t, h2d, d2h, e2e_steps = 0, 0.0, 0, 0, max(1, min(args.steps, 5))
    for k in range(e2e_steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sim.set_bodies(host)
        info = sim.step(DT, 1.0, 1)
        host = sim.state(out=pinned)
        e2e_t += time.perf_counter() - t0
        e2e_int += info["interactions"]
        h2d += sum(a.nbytes for a in host.values())
        d2h += sum(a.nbytes for a in host.values())
    e2e = {"value": dist.sum(e2e_int) / dist.max(e2e_t), "unit": UNIT, "h2d_bytes_per_step": int(h2d // e2e_steps),
           "d2h_bytes_per_step": int(d2h // e2e_steps),
           "path": "nbg_set_bodies (full state, pinned host) + nbg_step + nbg_get_state (full state)"}

    # ---- FP32 / FP64 peaks, plain FP64 comparison, accuracy ----
    f32, f64, mhz = probe_peaks(local)
    result_extra = {}
    if not args.no_plain and rank == 0:
        plain = Simulation("fp64", device=local, capacity=n0 + 4096)
        plain.set_stream(stream.cuda_stream)
        plain.set_bodies(bodies)
        fp = plain.force_pass()
        mixed0 = Simulation("mixed", device=local, capacity=n0 + 4096)
        mixed0.set_bodies(bodies)
        fm = mixed0.force_pass()
        num = np.sqrt(sum(np.sum((a - b) ** 2) for a, b in zip(fm, fp)))
        den = np.sqrt(sum(np.sum(b ** 2) for b in fp))
        mag = np.sqrt(fp[0] ** 2 + fp[1] ** 2 + fp[2] ** 2)
        err = np.sqrt((fm[0] - fp[0]) ** 2 + (fm[1] - fp[1]) ** 2 + (fm[2] - fp[2]) ** 2)
        ok = mag > 0
        plain.enable_timing(True)
        pi = plain.step(DT, 1.0, 2)
        ptm = plain.timing()
        p_ms = (ptm["pair_ms"] + ptm["other_ms"]) / max(1, ptm["pair_launches"])
        plain_rate = pi["interactions"] / (1e-3 * (ptm["pair_ms"] + ptm["other_ms"]))
        result_extra["plain_fp64"] = {
            "value": plain_rate, "unit": UNIT, "ms_per_step": p_ms,
            "pair_kernel_ms": ptm["pair_ms"] / max(1, ptm["pair_launches"]),
            "roofline_frac_fp64": plain_rate * FLOPS_PER_PAIR / f64 if f64 else None,
            "steps": 2}
        result_extra["mixed_over_plain"] = value / plain_rate / ws if plain_rate else None
        result_extra["accuracy"] = {"rel_l2_vs_fp64": float(num / den), "max_rel": float(np.max(err[ok] / mag[ok])),
                                    "median_rel": float(np.median(err[ok] / mag[ok])),
                                    "reference": "plain FP64 GPU forces (bit-identical to the oracle)"}
        plain.close()
        mixed0.close()
        ke0, pe0, _ = sim.energy()
        result_extra["energy"] = {"kinetic": ke0, "potential": pe0}

    achieved = n_now * FLOPS_PER_PAIR / (pair_ms * 1e-3) / 1e12
    peak = f32 / 1e12
    traffic = traffic_from_profiles()
    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline_sample()
    sim.close()
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max / args.steps,
            "ms_per_step_each": [round(v, 4) for v in per_step], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32 pair terms, fp64 state",
            "data": "synthetic",
            "config": {"workload": f"{WORKLOAD}: {n0} bodies (Plummer a=300 M=1e16 + disk r 400-4000), subsume, "
                                   f"dt={DT}, mixed precision", "n_bodies": n0, "dt": DT,
                       "l2": "flushed (512 MB write) before every timed cycle", "parallelism": f"replicas x{ws}"},
            "e2e": e2e,
            "gpu_launches": int(launches),
            "roofline": {"bound": "fp32_fma", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak if peak else None, "traffic": traffic,
                         "kernel": "k_pair_mixed", "flops_per_pair": FLOPS_PER_PAIR,
                         "pair_kernel_ms": pair_ms,
                         "peak_source": f"FFMA-chain probe on this GPU at {mhz:.0f} MHz (MEASURED_PEAKS.json "
                                        "has no FP32 figure)"},
            "peaks": {"fp32_tflops": f32 / 1e12, "fp64_tflops": f64 / 1e12, "probe_sm_mhz": mhz,
                      "hbm_gbs_measured": measured_hbm().get("hbm_gbs")},
            "clocks": clk,
            "cpu_baseline": cpu,
        }
        line.update(result_extra)
        print(json.dumps(line), flush=True)
    dist.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
