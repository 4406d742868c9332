#!/usr/bin/env python
"""CTMRG-step benchmark of the GB300 backend.

Workload (U(1) iPEPS, 1x1 unit cell): physical q in {-1,+1} (dim 2), virtual
D=4 with q in {-1,0,1} and degeneracies [1,2,1], chi=32, site tensor N(0,1)
from a fixed seed, environment initialised FROM_A and grown for `warmup`
steps (so chi is saturated) before timing.  One step = grow_all (left, right,
top, bottom moves), all tensor work on the GPU in FP64.

Arms:
  default            this backend on cuda:LOCAL_RANK
  --impl reference   the CPU restatement of the reference algorithm (oracle
                     port; the reference itself cannot be built here), all
                     host cores, same workload and metric.
Replicas only across GPUs: each rank runs the same workload independently.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

AUX = [(-1, 1), (0, 2), (1, 1)]
PHYS = [(-1, 1), (1, 1)]
CHI = 32
SEED = 1234
METRIC = "CTMRG step throughput, U(1) iPEPS D=4 chi=32, plain FP64"
WORKLOAD = "u1_ipeps_D4_chi32_ctmrg_step"


def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def make_site_tensor_data(sizes_by_sector):
    rng = np.random.default_rng(SEED)
    return [rng.standard_normal(n) for n in sizes_by_sector]


# ----------------------------------------------------------------------------- GPU arm
def run_gpu(args):
    import ctypes as C

    from xped_gb300 import CTM, Basis, Tensor, ensure_device, lib
    from xped_gb300._lib import profile_read

    rank, world, local = dist_info()
    ensure_device(local)
    L = lib()
    aux = Basis.from_pairs("U1", AUX)
    phys = Basis.from_pairs("U1", PHYS)
    A = Tensor.zeros([aux, aux], [aux, aux, phys])
    qs, rs, cs = A.sectors()
    A.set_data(np.concatenate(make_site_tensor_data([r * c for r, c in zip(rs, cs)])))
    ctm = CTM(A, CHI).init()
    for _ in range(args.warmup):
        ctm.grow_all()
    L.xgb_synchronize()

    # L2 flush buffer (> 129 MB L2), written between timed steps outside the events
    flush_bytes = 512 << 20
    flush = C.c_void_p()
    L.xgb_malloc(C.byref(flush), flush_bytes)

    def flush_l2():
        L.xgb_memset_zero(flush, flush_bytes)

    # ---- device-resident timing
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.4)
    step_ms = []
    launches0 = L.xgb_launch_count()
    for _ in range(args.steps):
        flush_l2()
        L.xgb_synchronize()
        L.xgb_event_record(0)
        ctm.grow_all()
        L.xgb_event_record(1)
        step_ms.append(L.xgb_event_elapsed_ms(0, 1))
    launches = (L.xgb_launch_count() - launches0) / max(args.steps, 1)
    clocks = sampler.stop()

    # ---- end to end: env + site tensor from pinned host buffers, result back to host
    names = ["C1", "C2", "C3", "C4", "T1", "T2", "T3", "T4"]
    env = ctm.env()
    try:
        import torch
        pin = lambda n: torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
    except Exception:
        pin = lambda n: np.empty(n, dtype=np.float64)
    host_in = {k: pin(env[k].size) for k in names}
    for k in names:
        host_in[k][:] = env[k].data()
    host_A = pin(A.size)
    host_A[:] = A.data()
    host_out = {k: None for k in names}
    e2e_ms = []
    h2d = d2h = 0
    for _ in range(args.steps):
        flush_l2()
        L.xgb_synchronize()
        L.xgb_event_record(2)
        A.set_data(host_A)
        for k in names:
            env[k].set_data(host_in[k])
            ctm.set(k, env[k])
        ctm.grow_all()
        out = ctm.env()
        for k in names:
            host_out[k] = out[k].data()
        L.xgb_event_record(3)
        e2e_ms.append(L.xgb_event_elapsed_ms(2, 3))
        h2d = host_A.nbytes + sum(host_in[k].nbytes for k in names)
        d2h = sum(v.nbytes for v in host_out.values())

    # ---- kernel profile pass over the same steps (CUDA events around every launch)
    L.xgb_profile_reset()
    L.xgb_profile_enable(1)
    for _ in range(args.steps):
        flush_l2()
        ctm.grow_all()
    L.xgb_synchronize()
    L.xgb_profile_enable(0)
    prof = profile_read()
    L.xgb_free(flush)

    t_step = float(np.mean(step_ms))
    t_e2e = float(np.mean(e2e_ms))
    res = dict(step_ms=t_step, e2e_ms=t_e2e, launches=launches, clocks=clocks, prof=prof, h2d=h2d, d2h=d2h)
    return res


def roofline(prof, steps):
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    kinds = {k: v for k, v in prof.items() if v[0] > 0}
    if not kinds:
        return None
    dom = max(kinds, key=lambda k: kinds[k][1])
    n, ms, work = kinds[dom]
    per_launch_ms = ms / n
    per_launch_work = work / n
    if dom in ("gemm_f64", "svd_jacobi", "qr"):
        # FP64 runs on the DFMA pipe; GB300's nominal dense FP64 rate is 1.25 TFLOP/s.
        # SVD work is counted as LAPACK dgesvd-equivalent flops (4m^2n + 8mn^2 + 9n^3, m >= n).
        achieved = per_launch_work / (per_launch_ms * 1e-3) / 1e12
        out = {"bound": "fp64", "kernel": dom, "achieved": achieved, "peak": 1.25, "unit": "TFLOP/s",
               "peak_source": "nominal GB300 FP64 rate (MEASURED_PEAKS.json has no FP64 figure)",
               "work": "LAPACK-equivalent flops" if dom == "svd_jacobi" else "useful flops"}
    else:
        achieved = per_launch_work / (per_launch_ms * 1e-3) / 1e9
        out = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
               "peak_source": "MEASURED_PEAKS.json hbm_gbs" if "hbm_gbs" in peaks else "fallback 6800 GB/s"}
    out["frac"] = out["achieved"] / out["peak"]
    out["traffic"] = None
    out["launches_per_step"] = n / max(steps, 1)
    out["ms_per_launch"] = per_launch_ms
    out["kernel_share"] = {k: round(v[1] / sum(x[1] for x in kinds.values()), 4) for k, v in kinds.items()}
    return out


# ----------------------------------------------------------------------------- CPU oracle
def cpu_ctm_steps(n_steps, warmup, budget_s=None):
    import oracle
    from oracle.basis import Qbasis
    from oracle.ctm import CTM as OCTM
    from oracle.ctm import IPEPS

    s = oracle.make_symmetry("u1")
    aux = Qbasis.from_pairs(s, AUX)
    phys = Qbasis.from_pairs(s, PHYS)
    peps = IPEPS(s, aux, phys)
    data = make_site_tensor_data([b.size for b in peps.A.blocks])
    for i, b in enumerate(peps.A.blocks):
        peps.A.blocks[i] = data[i].reshape(b.shape, order="F")
    peps.update_adag()
    c = OCTM(peps, CHI).init()
    for _ in range(warmup):
        c.grow_all()
    times = []
    t_start = time.perf_counter()
    for _ in range(n_steps):
        t0 = time.perf_counter()
        c.grow_all()
        times.append(time.perf_counter() - t0)
        if budget_s is not None and time.perf_counter() - t_start > budget_s:
            break
    return times


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    rank, world, local = dist_info()

    if args.impl == "reference":
        if rank != 0:
            return
        times = cpu_ctm_steps(args.steps, args.warmup)
        t = float(np.mean(times))
        v = 1.0 / t
        line = {"metric": METRIC, "value": v, "unit": "steps/s", "n_gpus": args.gpus, "steps": len(times),
                "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded N(0,1) site tensor)",
                "config": {"workload": WORKLOAD, "chi": CHI, "D": 4, "phys": 2, "cell": "1x1"},
                "impl": "reference",
                "cpu_baseline": {"value": v, "unit": "steps/s", "cores": os.cpu_count(), "kind": "port",
                                 "sample": f"{len(times)} grow_all steps after {args.warmup} warm-up steps"},
                "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    r = run_gpu(args)
    t_step, t_e2e = r["step_ms"], r["e2e_ms"]
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([t_step, t_e2e], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_step, t_e2e = float(t[0]), float(t[1])
        dist.barrier()
    if rank != 0:
        return
    value = world * 1e3 / t_step
    line = {"metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded N(0,1) site tensor)",
            "config": {"workload": WORKLOAD, "chi": CHI, "D": 4, "phys": 2, "cell": "1x1",
                       "l2": "512 MB buffer written between timed steps (outside the timed events)",
                       "parallelism": f"replicas x{world}"},
            "e2e": {"value": world * 1e3 / t_e2e, "unit": "steps/s", "h2d_bytes_per_step": r["h2d"],
                    "d2h_bytes_per_step": r["d2h"]},
            "gpu_launches": r["launches"], "clocks": r["clocks"],
            "roofline": roofline(r["prof"], args.steps)}
    if not args.no_cpu_baseline:
        times = cpu_ctm_steps(30, 1, budget_s=12.0)
        tc = float(np.mean(times))
        line["cpu_baseline"] = {"value": 1.0 / tc, "unit": "steps/s", "cores": os.cpu_count(), "kind": "port",
                                "sample": f"{len(times)} grow_all steps of the same workload after 1 warm-up step, "
                                          "numpy/OpenBLAS on all host cores"}
    print(json.dumps(line))


if __name__ == "__main__":
    main()
