#!/usr/bin/env python
"""CTMRG-step benchmark of the GB300 backend: chosen form against plain FP64.

Workload (U(1) iPEPS, 1x1 unit cell): physical q in {-1,+1} (dim 2), virtual
D=6 with q in {-1,0,1} and degeneracies [2,2,2], chi=128, site tensor N(0,1)
from a fixed seed, environment initialised FROM_A and grown for `warmup`
steps before timing (chi saturates at 128 after the first step).  One step =
grow_all (left, right, top, bottom moves), all tensor work on the GPU.

Forms, same workload, same GPU:
  chosen   randomized projector SVD (seeded Gaussian sketches, 8 subspace
           iterations, CholeskyQR3 orthonormalisation, widths = the direction's
           last kept counts + max(16, 50 %), exact FP64 tSVD for the first
           decomposition of each direction and as fallback), FP64 SVD core /
           projectors / normalisation;
           block GEMMs (--gemm): f64tc (default: FP64-accurate, exact BF16 slices on
           the tensor cores or the FP64 CUDA cores, per size bucket from the
           autotuner), fp64, 3xtf32 or fp32
  plain    the exact FP64 tSVD in every move (the reference algorithm)
The energy per site (Heisenberg bonds, horizontal + vertical RDM) of both
forms after the same number of steps from the same start is reported with
their difference.

Arms:
  default            this backend on cuda:LOCAL_RANK
  --impl reference   the CPU restatement of the reference algorithm (oracle
                     port; the reference itself cannot be built here) on all
                     host cores, same workload and metric; each timed sample
                     is one CTM move, a step counted as four moves.
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

AUX = [(-1, 2), (0, 2), (1, 2)]
PHYS = [(-1, 1), (1, 1)]
CHI = 128
SEED = 1234
AUX_SMALL = [(-1, 1), (0, 2), (1, 1)]  # D=4, chi=32: the plain FP64 GPU configuration
CHI_SMALL = 32
COMPARE_STEPS = 3
POWER_ITERS = 8  # subspace iterations of the chosen form: energy within ~1e-9 of plain FP64 at this workload
SKETCH_TAIL = 2  # trailing subspace iterations in FP64; the first product and the earlier ones in 3xTF32
METRIC = "CTMRG step throughput, U(1) iPEPS D=6 chi=128, chosen form vs plain FP64"
WORKLOAD = "u1_ipeps_D6_chi128_ctmrg_step"


def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def ranks_barrier():
    """Barrier over the replicas (gloo) when the bench runs under torchrun with N > 1."""
    if dist_info()[1] > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(values):
    """Element-wise maximum of per-rank timings (the slowest replica sets the whole-job time)."""
    if dist_info()[1] <= 1:
        return [float(v) for v in values]
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v) for v in values], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t]


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


def site_tensor(aux_pairs):
    from xped_gb300 import Basis, Tensor
    aux = Basis.from_pairs("U1", aux_pairs)
    phys = Basis.from_pairs("U1", PHYS)
    A = Tensor.zeros([aux, aux], [aux, aux, phys])
    A.set_data(np.random.default_rng(SEED).standard_normal(A.size))
    return A, phys


def make_ctm(A, chi, form, gemm, tail=-1):
    from xped_gb300 import CTM
    c = CTM(A, chi).init()
    if form == "chosen":
        c.set_svd("randomized", power_iters=POWER_ITERS, seed=SEED, oversample=16, growth=0.5)
        c.set_sketch_precision(tail)
    c.set_gemm(gemm)
    return c


# ----------------------------------------------------------------------------- GPU arm
def run_gpu(args):
    import ctypes as C

    from xped_gb300 import ensure_device, lib
    from xped_gb300._lib import profile_read
    from xped_gb300.observables import energy, heisenberg_bond

    rank, world, local = dist_info()
    ensure_device(local)
    L = lib()
    A, phys = site_tensor(AUX)
    H = heisenberg_bond(phys)
    res = {}

    if args.autotune:
        L.xgb_autotune_set(1)  # FP64 GEMM tile / split-K shapes tuned per size bucket during the warm-up
    # ---- chosen form: warm-up (the energy after COMPARE_STEPS steps is kept for the comparison);
    # its projector decompositions are logged to train the width predictor
    t0 = time.perf_counter()
    ctm = make_ctm(A, CHI, "chosen", args.gemm, args.sketch_tail)
    ctm.record(True)
    e_chosen = None
    for i in range(max(args.warmup, COMPARE_STEPS)):
        ctm.grow_all()
        if i + 1 == COMPARE_STEPS:
            e_chosen = energy(ctm, H)
    L.xgb_synchronize()
    records = ctm.records()
    ctm.record(False)
    if args.autotune:
        L.xgb_autotune_set(2)  # frozen: no measurement inside the timed steps
    # one more untimed step in the timed configuration: the first step that runs the move pairs on two
    # streams (not while the autotuner measures) starts the side lane's host thread and its buffers
    ctm.grow_all()
    L.xgb_synchronize()
    res["chosen_setup_s"] = time.perf_counter() - t0
    res["autotune"] = autotune_report(L)

    flush_bytes = 512 << 20  # > 129 MB L2, written between timed steps outside the events
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
    st0 = ctm.stats()
    L.xgb_synchronize()
    ranks_barrier()
    for _ in range(args.steps):
        flush_l2()
        L.xgb_synchronize()
        L.xgb_event_record(0)
        ctm.grow_all()
        L.xgb_event_record(1)
        step_ms.append(L.xgb_event_elapsed_ms(0, 1))
    L.xgb_synchronize()
    ranks_barrier()
    st1 = ctm.stats()
    res["cols_per_step"] = (st1["sketch_cols"] - st0["sketch_cols"]) / args.steps
    res["redo_per_step"] = (st1["redo"] - st0["redo"]) / args.steps
    res["launches"] = int(L.xgb_launch_count() - launches0)  # this library's kernels in the K timed steps
    res["launches_per_step"] = res["launches"] / max(args.steps, 1)
    res["clocks"] = sampler.stop()
    res["step_ms"] = float(np.mean(step_ms))
    res["step_ms_all"] = step_ms

    # ---- end to end: environment and site tensor from pinned host buffers, result back to host
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
    e2e_ms = []
    h2d = d2h = 0
    L.xgb_synchronize()
    ranks_barrier()
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
        host_out = {k: out[k].data() for k in names}
        L.xgb_event_record(3)
        e2e_ms.append(L.xgb_event_elapsed_ms(2, 3))
        h2d = host_A.nbytes + sum(host_in[k].nbytes for k in names)
        d2h = sum(v.nbytes for v in host_out.values())
    L.xgb_synchronize()
    ranks_barrier()
    res["e2e_ms"] = float(np.mean(e2e_ms))
    res["h2d"], res["d2h"] = h2d, d2h

    # ---- kernel profile pass (CUDA events around every launch)
    L.xgb_profile_reset()
    L.xgb_profile_enable(1)
    prof_steps = 2
    for _ in range(prof_steps):
        flush_l2()
        ctm.grow_all()
    L.xgb_synchronize()
    L.xgb_profile_enable(0)
    res["prof"] = profile_read()
    res["prof_steps"] = prof_steps
    res["sketch"] = ctm.stats()
    res["ctm"] = ctm

    # ---- learned widths: the rank predictor trained (device kernels) on the chosen run's own
    # logged spectra, then a fresh run with predicted widths
    if not args.no_learned:
        from xped_gb300.learn import RankModel, dataset
        X, T = dataset(records)
        model = RankModel(seed=SEED)
        t0 = time.perf_counter()
        loss0 = model.gradient(X, T)[0]
        loss = model.train(X, T, steps=2000, lr=2e-3)
        res["learned_train"] = {"samples": int(X.shape[0]), "adam_steps": 2000, "loss_first": loss0,
                                "loss_last": loss, "seconds": time.perf_counter() - t0}
        lc = make_ctm(A, CHI, "plain", args.gemm)
        lc.set_rank_model(model, margin=0.0, min_oversample=2, power_iters=POWER_ITERS, seed=SEED)
        lc.set_sketch_precision(args.sketch_tail)
        for _ in range(COMPARE_STEPS):
            lc.grow_all()
        res["e_learned"] = energy(lc, H)
        if not args.no_converge:
            lc2 = make_ctm(A, CHI, "plain", args.gemm)
            lc2.set_rank_model(model, margin=0.0, min_oversample=2, power_iters=POWER_ITERS, seed=SEED)
            lc2.set_sketch_precision(args.sketch_tail)
            res["solve_learned"] = timed_solve(L, lc2, H, args)
            del lc2
        s0 = lc.stats()
        ms = []
        for _ in range(args.steps):
            flush_l2()
            L.xgb_synchronize()
            L.xgb_event_record(8)
            lc.grow_all()
            L.xgb_event_record(9)
            ms.append(L.xgb_event_elapsed_ms(8, 9))
        s1 = lc.stats()
        res["learned_ms"] = float(np.mean(ms))
        res["learned_cols_per_step"] = (s1["sketch_cols"] - s0["sketch_cols"]) / args.steps
        res["learned_redo_per_step"] = (s1["redo"] - s0["redo"]) / args.steps
        del lc

    # ---- the chosen form run to convergence (CTMSolver::solve) from a fresh FROM_A start
    if not args.no_converge:
        cc = make_ctm(A, CHI, "chosen", args.gemm, args.sketch_tail)
        res["solve_chosen"] = timed_solve(L, cc, H, args)
        del cc

    # ---- plain FP64 form, same workload: COMPARE_STEPS steps (energy compared with the chosen form's),
    # then on to convergence; one more step at saturated chi is timed
    if not args.no_plain:
        t0 = time.perf_counter()
        plain = make_ctm(A, CHI, "plain", "fp64")
        for _ in range(COMPARE_STEPS):
            plain.grow_all()
        res["e_plain"] = energy(plain, H)
        if not args.no_converge:
            res["solve_plain"] = timed_solve(L, plain, H, args, done=COMPARE_STEPS)
        flush_l2()
        L.xgb_synchronize()
        L.xgb_event_record(4)
        plain.grow_all()
        L.xgb_event_record(5)
        res["plain_ms"] = L.xgb_event_elapsed_ms(4, 5)
        res["plain_wall_s"] = time.perf_counter() - t0
        del plain
    res["e_chosen"] = e_chosen

    # ---- plain FP64 at D=4 chi=32 (the reference's GPU configuration), for the record
    A4, _ = site_tensor(AUX_SMALL)
    small = make_ctm(A4, CHI_SMALL, "plain", "fp64")
    for _ in range(3):
        small.grow_all()
    ms = []
    for _ in range(3):
        flush_l2()
        L.xgb_synchronize()
        L.xgb_event_record(6)
        small.grow_all()
        L.xgb_event_record(7)
        ms.append(L.xgb_event_elapsed_ms(6, 7))
    res["small_plain_ms"] = float(np.mean(ms))
    L.xgb_free(flush)
    res["gemm_sweep"] = gemm_sweep()
    res["tensor22_chain"] = tensor22_chain()
    res["fp64_peak"] = fp64_library_peak()
    res["su"] = su_step()
    res["permute_roofline"] = permute_roofline()
    if not args.no_configs:
        res["tsvd_sweep"] = tsvd_sweep(eval_seeds=(0, 1), train_seeds=tuple(range(100, 106)), steps=4)
        res["fz2"] = fz2_compact(args)
    return res


def profile_step(args):
    """One chosen-form step of the headline workload after `warmup` steps, bracketed by the CUDA runtime's
    profiler start / stop so that a profiler started with profiling off captures exactly its launches."""
    import ctypes as C
    from xped_gb300 import ensure_device, lib
    ensure_device(dist_info()[2])
    L = lib()
    # --autotune-cache: the first run measures and saves its choices, a later run (e.g. under a profiler,
    # whose launch interception would skew the measurements) loads them, so both profile the same launches
    cache = args.autotune_cache
    loaded = 0
    if args.autotune:
        if cache and os.path.exists(cache):
            loaded = L.xgb_autotune_load(cache.encode())
            if loaded <= 0:
                raise RuntimeError(f"autotune cache {cache}: no entries for this GPU")
            L.xgb_autotune_set(2)
        else:
            L.xgb_autotune_set(1)
    A, _ = site_tensor(AUX)
    c = make_ctm(A, CHI, "chosen", args.gemm, args.sketch_tail)
    for _ in range(args.warmup):
        c.grow_all()
    L.xgb_synchronize()
    if args.autotune:
        if cache and not loaded and L.xgb_autotune_save(cache.encode()) != 0:
            raise RuntimeError(f"autotune cache {cache} not written")
        L.xgb_autotune_set(2)
    rt = None
    with open("/proc/self/maps") as f:  # the CUDA runtime the library itself loaded
        for line in f:
            if "libcudart.so" in line:
                rt = C.CDLL(line.split()[-1])
                break
    n0 = L.xgb_launch_count()
    rt.cudaProfilerStart()
    L.xgb_event_record(0)
    c.grow_all()
    L.xgb_event_record(1)
    L.xgb_synchronize()
    rt.cudaProfilerStop()
    return {"ms": L.xgb_event_elapsed_ms(0, 1), "launches": L.xgb_launch_count() - n0, "gemm": args.gemm,
            "workload": WORKLOAD, "autotune_cache": cache, "autotune_loaded": int(loaded)}


def dtype_label(args):
    if args.gemm == "f64tc":
        return "f64 (FP64-accurate block GEMMs: exact BF16 slices on the tensor cores or FP64 CUDA cores)"
    return (("f64" if args.gemm == "fp64" else f"f64 ({args.gemm} block GEMMs)")
            + (" + 3xTF32 early sketch products" if args.sketch_tail >= 0 else ""))


def gemm_form_label(args):
    if args.gemm == "f64tc":
        return ("; every block GEMM (corner contractions, renormalisation, T1 T2, projectors, sketch products) "
                "FP64-accurate: exact BF16 slices on the tensor cores, or the FP64 CUDA cores where the autotuner "
                "measures them faster")
    return (f"; sketch products of the first {POWER_ITERS - args.sketch_tail} iterations 3xTF32"
            if args.sketch_tail >= 0 else "")


def autotune_report(L):
    """The FP64 GEMM shapes the autotuner chose (per size bucket) and the time it spent measuring."""
    import ctypes as C
    measured, hits, ms = C.c_int64(), C.c_int64(), C.c_double()
    n = L.xgb_autotune_stats(C.byref(measured), C.byref(hits), C.byref(ms))
    tiles, waves = (C.c_int32 * max(n, 1))(), (C.c_int32 * max(n, 1))()
    L.xgb_autotune_choices(tiles, waves, n)
    hist = {}
    for i in range(n):
        k = "f64tc" if tiles[i] == 0 else f"tile{tiles[i]}_split{waves[i]}"
        hist[k] = hist.get(k, 0) + 1
    return {"enabled": True, "buckets": n, "cache_hits": hits.value, "measure_ms": ms.value, "choices": hist,
            "candidates": "CUDA-core FP64 tile 16/32/64 x split-K target 0/1/2/4 waves; with --gemm f64tc also the "
                          "FP64-accurate tensor-core form"}


def timed_solve(L, c, H, args, done=0):
    """CTMSolver::solve on `c` (tol_E, at most --solve-max-steps grow_all steps); `done` steps were already
    run on it.  Device time of the whole solve (CUDA events) and the energy trajectory."""
    L.xgb_synchronize()
    L.xgb_event_record(12)
    r = c.solve(H, tol_E=args.tol_e, max_steps=args.solve_max_steps)
    L.xgb_event_record(13)
    r["seconds"] = L.xgb_event_elapsed_ms(12, 13) / 1e3
    r["steps_total"] = r["steps"] + done
    r["tol_E"] = args.tol_e
    r["energies"] = [float(e) for e in r["energies"][-4:]]  # the last few are enough to show convergence
    return r


def permute_roofline(degs=(20, 40, 60, 40, 20), reps=5):
    """Tensor::permute<0>(0, 2, 1, 3) of one U(1) Tensor<2,2> with every leg q = -2..2 at degeneracies
    `degs` (1.42 GB of FP64 blocks, far above the 129 MB L2): kernel time per launch from the library's
    per-launch CUDA events, achieved HBM GB/s = algorithmic bytes (every element read once and written
    once, 16 B) / time, against the measured copy rate."""
    from xped_gb300 import Basis, Tensor, lib
    from xped_gb300._lib import profile_read
    L = lib()
    B = Basis.from_pairs("U1", list(zip(range(-2, 3), degs)), sort=True)
    T = Tensor.zeros([B, B], [B, B])
    T.set_data(np.random.default_rng(SEED).standard_normal(T.size))
    out = T.permute(0, [0, 2, 1, 3])  # plan built and cached
    del out
    L.xgb_synchronize()
    L.xgb_profile_reset()
    L.xgb_profile_enable(1)
    for _ in range(reps):
        out = T.permute(0, [0, 2, 1, 3])
        del out
    L.xgb_synchronize()
    L.xgb_profile_enable(0)
    n, ms, work = profile_read()["permute"]
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    per_launch = ms / max(n, 1)
    algorithmic = 16.0 * T.size
    gbs = algorithmic / (per_launch * 1e-3) / 1e9
    del T
    # DRAM read + write of one launch from an ncu capture of the [14, 28, 42, 28, 14] case (42.5 M
    # doubles: 344.7 MB read, 294.2 MB written, the rest of the output still in L2 at the kernel's end),
    # scaled by the element count (the traffic grows in proportion)
    traffic = (344.672e6 + 294.158e6) * (algorithmic / 16.0) / 42526512.0
    return {"kernel": "permute_rows_wide_kernel", "elements": int(algorithmic // 16),
            "gbytes_moved": algorithmic / 1e9, "launches": int(n), "ms_per_launch": per_launch, "achieved": gbs,
            "peak": hbm, "unit": "GB/s", "frac": gbs / hbm, "bound": "hbm", "traffic": traffic,
            "traffic_source": "ncu capture of the deg [14, 28, 42, 28, 14] case scaled by elements",
            "peak_source": "MEASURED_PEAKS.json hbm_gbs" if "hbm_gbs" in peaks else "fallback 6800 GB/s",
            "workload": "U(1) Tensor<2,2>, legs q -2..2 deg " + str(list(degs)) + ", permute<0>(0,2,1,3)"}


FZ2_CHI_SMALL = 48  # the plain form's 20 iterations at chi = 144 take ~17 min; the equal-energy check runs here


def fz2_compact(args):
    """The full chosen form on the fermionic Z2 iPEPS (D=6, q 0,1 with degeneracies [3,3]): FZ2_ITERS CTMRG
    iterations at chi = 144 of the chosen and the learned-width forms (per-step CUDA-event times), and the
    density-density bond after FZ2_ITERS iterations of the chosen and the plain FP64 form at chi = 48
    (the plain form's exact SVDs of ~2600-wide blocks take ~52 s per step at chi = 144)."""
    from xped_gb300 import CTM, Basis, Tensor, lib
    from xped_gb300.learn import RankModel, dataset
    from xped_gb300.observables import density_bond, energy
    L = lib()
    aux = Basis.from_pairs("fZ2", FZ2_AUX)
    phys = Basis.from_pairs("fZ2", FZ2_PHYS)
    A = Tensor.zeros([aux, aux], [aux, aux, phys])
    A.set_data(np.random.default_rng(SEED).standard_normal(A.size))
    H = density_bond(phys)
    out = {"aux": "q 0,1 deg [3,3]", "chi": FZ2_CHI, "iterations": FZ2_ITERS}
    model = None

    def chosen_ctm(chi, form):
        c = CTM(A, chi).init()
        if form == "chosen":
            c.set_svd("randomized", power_iters=POWER_ITERS, seed=SEED, oversample=16, growth=0.5)
        elif form == "learned":
            c.set_rank_model(model, margin=0.0, min_oversample=2, power_iters=POWER_ITERS, seed=SEED)
        if form != "plain":
            c.set_sketch_unseen(True)
            c.set_sketch_precision(args.sketch_tail)
            c.set_gemm(args.gemm)
        return c

    for form in ("chosen", "learned"):
        c = chosen_ctm(FZ2_CHI, form)
        if form == "chosen":
            c.record(True)
        ms = []
        for _ in range(FZ2_ITERS):
            L.xgb_synchronize()
            L.xgb_event_record(12)
            c.grow_all()
            L.xgb_event_record(13)
            ms.append(L.xgb_event_elapsed_ms(12, 13))
        out[form] = {"total_s": sum(ms) / 1e3, "ms_per_step_after_1": float(np.mean(ms[1:])),
                     "nn_bond_last": energy(c, H)}
        if form == "chosen":
            X, T = dataset(c.records())
            model = RankModel(seed=SEED)
            model.train(X, T, steps=2000, lr=2e-3)
            out["learned_train_samples"] = int(X.shape[0])
        del c
    nn = {}
    for form in ("chosen", "plain"):
        c = chosen_ctm(FZ2_CHI_SMALL, form)
        t0 = time.perf_counter()
        for _ in range(FZ2_ITERS):
            c.grow_all()
        L.xgb_synchronize()
        nn[form] = (energy(c, H), time.perf_counter() - t0)
        del c
    out["equal_energy_check"] = {"chi": FZ2_CHI_SMALL, "iterations": FZ2_ITERS, "nn_bond_chosen": nn["chosen"][0],
                                 "nn_bond_plain": nn["plain"][0], "abs_diff": abs(nn["chosen"][0] - nn["plain"][0]),
                                 "wall_s_chosen": nn["chosen"][1], "wall_s_plain": nn["plain"][1]}
    return out


# ----------------------------------------------------------------------------- fermionic Z2 workload
FZ2_AUX = [(0, 3), (1, 3)]   # D = 6
FZ2_PHYS = [(0, 1), (1, 1)]  # spinless fermion: empty / occupied
FZ2_CHI = 144
FZ2_ITERS = 20
FZ2_MARK = 2  # step after which the bond observable is compared with the plain form


def run_fz2(args):
    """Fermionic Z2 iPEPS (ZN<FChargeU1,2>), D=6 with q in {0,1} and degeneracies [3,3], physical
    parity 0/1, chi=144: FZ2_ITERS CTMRG iterations of the chosen form from FROM_A, every step
    timed with CUDA events (the chosen form sketches the first decomposition of each direction too:
    chi + 16 columns); then the same iterations with learned widths (the rank predictor trained on
    the chosen run's own logged decompositions, device Adam); the density-density bond expectation
    after FZ2_MARK steps and after the last one.  The plain FP64 form runs --fz2-plain-steps steps
    from the same start (its exact SVDs of ~2600-wide sector blocks take minutes per step)."""
    from xped_gb300 import CTM, Basis, Tensor, ensure_device, lib
    from xped_gb300.learn import RankModel, dataset
    from xped_gb300.observables import density_bond, energy

    _, _, local = dist_info()
    ensure_device(local)
    L = lib()
    aux = Basis.from_pairs("fZ2", FZ2_AUX)
    phys = Basis.from_pairs("fZ2", FZ2_PHYS)
    A = Tensor.zeros([aux, aux], [aux, aux, phys])
    A.set_data(np.random.default_rng(SEED).standard_normal(A.size))
    H = density_bond(phys)
    npl = args.fz2_plain_steps
    out = {}
    model = None
    for form, iters in (("chosen", FZ2_ITERS), ("learned", FZ2_ITERS), ("plain", npl)):
        if iters <= 0:
            continue
        c = CTM(A, FZ2_CHI).init()
        if form == "chosen":
            c.set_svd("randomized", power_iters=POWER_ITERS, seed=SEED, oversample=16, growth=0.5)
            c.record(True)
        elif form == "learned":
            c.set_rank_model(model, margin=0.0, min_oversample=2, power_iters=POWER_ITERS, seed=SEED)
        if form != "plain":
            c.set_sketch_unseen(True)
            c.set_sketch_precision(args.sketch_tail)
            c.set_gemm(args.gemm)
        ms, marks = [], {}
        for i in range(iters):
            L.xgb_synchronize()
            L.xgb_event_record(12)
            c.grow_all()
            L.xgb_event_record(13)
            ms.append(L.xgb_event_elapsed_ms(12, 13))
            if i + 1 == FZ2_MARK:
                marks["nn_bond_at_mark"] = energy(c, H)
        out[form] = dict(marks, ms_per_step_each=[round(x, 2) for x in ms], total_s=sum(ms) / 1e3,
                         ms_per_step_after_1=float(np.mean(ms[1:])) if len(ms) > 1 else None,
                         nn_bond_last=energy(c, H), stats=c.stats())
        if form == "chosen":
            X, T = dataset(c.records())
            c.record(False)
            model = RankModel(seed=SEED)
            t0 = time.perf_counter()
            loss = model.train(X, T, steps=2000, lr=2e-3)
            out["learned_train"] = {"samples": int(X.shape[0]), "adam_steps": 2000, "loss_last": loss,
                                    "seconds": time.perf_counter() - t0}
        del c
    ch = out["chosen"]
    line = {"metric": f"CTMRG iterations, fermionic Z2 iPEPS D=6 chi={FZ2_CHI}, chosen form",
            "value": 1e3 / float(np.mean(ch["ms_per_step_each"][3:])), "unit": "steps/s", "n_gpus": 1,
            "steps": FZ2_ITERS, "higher_is_better": True, "dtype": "f64", "data": "synthetic (seeded N(0,1))",
            "config": {"workload": f"fz2_ipeps_D6_chi{FZ2_CHI}_{FZ2_ITERS}_iterations", "aux": "q 0,1 deg [3,3]",
                       "phys": "q 0,1", "gemm": args.gemm, "sketch_fp64_tail": args.sketch_tail,
                       "graph_capture": "none: every move synchronises on the host for the truncation result"},
            "forms": out}
    if "plain" in out and out["plain"]["ms_per_step_after_1"]:
        line["chosen_vs_plain_per_step"] = out["plain"]["ms_per_step_after_1"] / ch["ms_per_step_after_1"]
        if "nn_bond_at_mark" in out["plain"]:
            for f in ("chosen", "learned"):
                line[f"nn_bond_abs_diff_{f}_vs_plain_at_step_{FZ2_MARK}"] = abs(out["plain"]["nn_bond_at_mark"] -
                                                                              out[f]["nn_bond_at_mark"])
    print(json.dumps(line))


# ----------------------------------------------------------------------------- block-GEMM sweep
def gemm_sweep(reps=5):
    """Grouped block GEMMs FP64 vs 3xTF32 vs BF16x9 vs FP32 (CUDA cores) vs F64TC (FP64-accurate, exact BF16
    slices on the tensor cores): (i) the sector GEMMs of an SU(2)
    Tensor<2,2> product (irreps q = 2j+1, j = 0..3 integer, multiplicities 1-24);
    (ii) synthetic lists of G blocks, m, n, k log-uniform in [8, 512].  Useful
    TFLOP/s = sum 2mnk / time; error = max over blocks of ||C - C_fp64||_F / ||C_fp64||_F."""
    import ctypes as C

    from xped_gb300 import Basis, Tensor, lib
    from xped_gb300._lib import GemmDesc, check
    from xped_gb300.tensor import set_gemm_precision
    L = lib()
    rng = np.random.default_rng(SEED)
    out = {}

    def timed(fn):
        for _ in range(2):
            fn()
        L.xgb_synchronize()
        L.xgb_event_record(10)
        for _ in range(reps):
            fn()
        L.xgb_event_record(11)
        return L.xgb_event_elapsed_ms(10, 11) / reps

    # (i) SU(2) contraction blocks through the tensor API
    pairs = [(q, int(rng.integers(1, 25))) for q in (1, 3, 5, 7)]
    B = Basis.from_pairs("SU2", pairs)
    T1 = Tensor.zeros([B, B], [B, B])
    T2 = Tensor.zeros([B, B], [B, B])
    T1.set_data(rng.standard_normal(T1.size))
    T2.set_data(rng.standard_normal(T2.size))
    descs = T1.gemm_plan(T2)[0]
    flops = sum(2.0 * d.m * d.n * d.k for d in descs)
    res = {}
    ref = None
    for form in ("fp64", "3xtf32", "bf16x9", "fp32", "f64tc"):
        set_gemm_precision(form)
        ms = timed(lambda: T1.matmul(T2))
        Cm = T1.matmul(T2)
        set_gemm_precision("fp64")
        blocks = Cm.blocks()
        if ref is None:
            ref = blocks
            err = 0.0
        else:
            err = max(np.linalg.norm(blocks[q] - ref[q]) / max(np.linalg.norm(ref[q]), 1e-300) for q in ref)
        res[form] = {"ms": ms, "tflops": flops / (ms * 1e-3) / 1e12, "max_rel_err": err}
    out["su2_tensor22"] = dict(res, blocks=len(descs), gflop=flops / 1e9,
                               multiplicities=[d for _, d in pairs])

    # (ii) synthetic grouped lists
    for G in (40, 100, 200, 400):
        dims = np.exp(rng.uniform(np.log(8), np.log(512), size=(G, 3))).astype(int)
        ds, ao, bo, co = [], 0, 0, 0
        for m, n, k in dims:
            ds.append(GemmDesc(int(m), int(n), int(k), ao, int(m), bo, int(k), co, int(m), 0, 0))
            ao += m * k
            bo += k * n
            co += m * n
        arr = (GemmDesc * G)(*ds)
        flops = float(sum(2.0 * m * n * k for m, n, k in dims))
        bufs = []
        for nel in (ao, bo, co):
            p_ = C.c_void_p()
            check(L.xgb_malloc(C.byref(p_), 8 * int(nel)), "malloc")
            bufs.append(p_)
        for p_, nel in zip(bufs[:2], (ao, bo)):
            h = rng.standard_normal(int(nel))
            L.xgb_memcpy_h2d(p_, h.ctypes.data, h.nbytes)
        res = {}
        ref = None
        for prec, form in ((0, "fp64"), (1, "3xtf32"), (2, "bf16x9"), (3, "fp32"), (4, "f64tc")):
            ms = timed(lambda: L.xgb_grouped_gemm(prec, G, arr, bufs[0], bufs[1], bufs[2], 1.0, 0.0, None))
            check(L.xgb_gemm_tc_status(), "tensor-core gemm")
            h = np.empty(int(co))
            L.xgb_memcpy_d2h(h.ctypes.data, bufs[2], h.nbytes)
            if ref is None:
                ref, err = h, 0.0
            else:
                err, o = 0.0, 0
                for m, n, k in dims:
                    a, b = h[o:o + m * n], ref[o:o + m * n]
                    err = max(err, float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)))
                    o += m * n
            res[form] = {"ms": ms, "tflops": flops / (ms * 1e-3) / 1e12, "max_rel_err": err}
        for p_ in bufs:
            L.xgb_free(p_)
        out[f"synthetic_G{G}"] = dict(res, gflop=flops / 1e9)
    return out


def su_step(steps=3, D=6, tau=0.05):
    """Simple-update imaginary-time steps (TimePropagator::t_step: 8 bond updates, each two full
    tSVDs and one truncated to D) of a U(1) spin-1/2 Heisenberg iPEPS on the checkerboard cell
    [[0, 1], [1, 0]]: virtual q -1,0,1 with degeneracies [2,2,2] (D = 6), N(0,1) site tensors,
    gates exp(-tau H).  Device time per step (CUDA events) beside the numpy oracle on the host
    cores; the largest weight difference between the two after `steps` steps."""
    import oracle
    from oracle.basis import Qbasis
    from oracle.ctm import IPEPS, heisenberg_u1
    from oracle.simple_update import SimpleUpdate as OSU
    from oracle.simple_update import gate
    from xped_gb300 import Basis, SimpleUpdate, Tensor, lib
    L = lib()
    s = oracle.make_symmetry("u1")
    aux_p, phys_p = [(-1, 2), (0, 2), (1, 2)], [(-1, 1), (1, 1)]
    oaux, ophys = Qbasis.from_pairs(s, aux_p), Qbasis.from_pairs(s, phys_p)
    naux, nphys = Basis.from_pairs("U1", aux_p), Basis.from_pairs("U1", phys_p)
    rng = np.random.default_rng(SEED)
    oG = [IPEPS(s, oaux, ophys).set_random(rng).A for _ in range(2)]
    nG = []
    for g in oG:
        t = Tensor.zeros([naux, naux], [naux, naux, nphys])
        t.set_data(g.data())
        nG.append(t)
    U = gate(heisenberg_u1(s, ophys), tau)
    nU = Tensor.zeros([nphys, nphys], [nphys, nphys])
    nU.set_data(U.data())
    pat = [[0, 1], [1, 0]]
    nsu = SimpleUpdate(pat, nG, D)
    nsu.step(nU, nU)  # plans
    ms = []
    for _ in range(steps):
        L.xgb_synchronize()
        L.xgb_event_record(10)
        nsu.step(nU, nU)
        L.xgb_event_record(11)
        ms.append(L.xgb_event_elapsed_ms(10, 11))
    osu = OSU(pat, oG, D)
    t0 = time.perf_counter()
    for _ in range(steps + 1):
        osu.step(U, U)
    cpu_ms = (time.perf_counter() - t0) * 1e3 / (steps + 1)
    err = 0.0
    for i in range(2):
        for name, ow in (("wh", osu.wh[i]), ("wv", osu.wv[i])):
            err = max(err, float(np.abs(nsu.get(name, i).data() - ow.data()).max()))
    return {"gpu_ms_per_step": float(np.median(ms)), "cpu_ms_per_step": cpu_ms, "cores": os.cpu_count(),
            "D": D, "steps": steps + 1, "weights_max_abs_diff": err,
            "workload": "checkerboard U(1) Heisenberg, q -1,0,1 deg [2,2,2], tau 0.05"}


def u1_product(degs, reps=10, form="fp64"):
    """One grouped block GEMM T1*T2 of U(1) Tensor<2,2> operands whose legs carry charges centred on 0
    with degeneracies `degs` (e.g. 6,12,16,12,6: coupled sectors up to 616 wide, as in the CTM
    projector products); N(0,1) entries.  CUDA-event time per product after two warm-up products."""
    from xped_gb300 import Basis, Tensor, lib
    from xped_gb300.tensor import set_gemm_precision
    L = lib()
    qs = list(range(-(len(degs) // 2), len(degs) - len(degs) // 2))
    B = Basis.from_pairs("U1", list(zip(qs, degs)), sort=True)
    rng = np.random.default_rng(SEED)
    T1, T2 = Tensor.zeros([B, B], [B, B]), Tensor.zeros([B, B], [B, B])
    T1.set_data(rng.standard_normal(T1.size))
    T2.set_data(rng.standard_normal(T2.size))
    descs = T1.gemm_plan(T2)[0]
    flops = sum(2.0 * d.m * d.n * d.k for d in descs)
    set_gemm_precision(form)
    try:
        for _ in range(2):
            T1.matmul(T2)
        L.xgb_synchronize()
        L.xgb_event_record(10)
        for _ in range(reps):
            T1.matmul(T2)
        L.xgb_event_record(11)
        ms = L.xgb_event_elapsed_ms(10, 11) / reps
    finally:
        set_gemm_precision("fp64")
    return {"degs": list(degs), "form": form, "blocks": [d.m for d in descs], "gflop": flops / 1e9, "ms": ms,
            "tflops": flops / (ms * 1e-3) / 1e12}


def tensor22_chain(seeds=(0, 1, 2, 3, 4), reps=20):
    """The plain FP64 op chain on a U(1) Tensor<2,2> (every leg q = -2..2, deg [2, 4, 6, 4, 2]; 9 coupled
    sectors, 17,712 doubles): T1*T2 -> permute<0>(0, 2, 1, 3) -> tSVD(16, 1e-10), N(0,1) entries per seed.
    Device time per chain (CUDA events, `reps` chains after warm-up, plans cached) beside the numpy/OpenBLAS
    oracle on the host cores; the largest |sigma| difference between the two."""
    from xped_gb300 import Basis, Tensor, lib
    import oracle
    from oracle.convert import tensor_from_native
    L = lib()
    sym = oracle.make_symmetry("u1")
    B = Basis.from_pairs("U1", [(-2, 2), (-1, 4), (0, 6), (1, 4), (2, 2)], sort=True)
    gpu_ms, cpu_ms, err = [], [], 0.0
    flops = None
    for seed in seeds:
        rng = np.random.default_rng(seed)
        T1, T2 = Tensor.zeros([B, B], [B, B]), Tensor.zeros([B, B], [B, B])
        T1.set_data(rng.standard_normal(T1.size))
        T2.set_data(rng.standard_normal(T2.size))
        if flops is None:
            flops = sum(2.0 * d.m * d.n * d.k for d in T1.gemm_plan(T2)[0])

        def chain():
            return T1.matmul(T2).permute(0, [0, 2, 1, 3]).tSVD(16, 1e-10)
        chain()
        L.xgb_synchronize()
        L.xgb_event_record(10)
        for _ in range(reps):
            out = chain()
        L.xgb_event_record(11)
        gpu_ms.append(L.xgb_event_elapsed_ms(10, 11) / reps)
        o1, o2 = tensor_from_native(sym, T1), tensor_from_native(sym, T2)
        t0 = time.perf_counter()
        for _ in range(reps):
            ref = (o1 * o2).permute(0, [0, 2, 1, 3]).tsvd(16, 1e-10)
        cpu_ms.append((time.perf_counter() - t0) * 1e3 / reps)
        got = np.sort(np.concatenate([np.diag(b) for b in out[1].blocks().values()]))
        exp = np.sort(np.concatenate([np.diag(b) for b in ref[1].blocks]))
        err = max(err, float(np.abs(got - exp).max() / exp.max()))
    return {"gpu_ms_per_chain": float(np.median(gpu_ms)), "cpu_ms_per_chain": float(np.median(cpu_ms)),
            "cpu": {"kind": "port", "cores": os.cpu_count(), "sample": f"{reps} chains per seed, median over seeds"},
            "gemm_flop": flops, "sigma_max_rel_diff": err, "seeds": len(seeds)}


def tsvd_sweep(eval_seeds=(0, 1, 2, 3, 4), train_seeds=tuple(range(100, 112)), steps=6, chi=128, p=3,
               drift=0.02):
    """Learned-width randomized tSVD on U(1) block matrices with power-law spectra (9-15 square sectors,
    n log-uniform in [16, 1024], A_q = U_q diag(c_q (i+1)^-alpha_q s) V_q^T, Haar U_q / V_q, alpha in
    {1, 2, 3}, c_q in [0.1, 1]); every sequence drifts its exponents by s = 1 + drift * t over `steps`
    decompositions, like the projector matrices of consecutive CTM steps.  Step 0 is exact; steps >= 1
    compare, with the previous step's exact result as history:
      exact     the FP64 tSVD (one batched Jacobi launch),
      history   randomized, widths last kept + max(16, 50 %),
      learned   randomized, widths from the MLP trained (device Adam) on the train seeds' sequences
    (p subspace iterations, chi = 128, eps 1e-10).  Reported per form: time (CUDA events), sketch columns,
    sectors whose kept count differs from the exact one, largest kept-value error relative to the largest
    value, saturated sectors; the CPU gesdd + cutoff_matrices time (oracle) of one matrix beside it."""
    from xped_gb300 import Basis, Tensor, lib
    from xped_gb300.learn import (RankModel, history_from_spectra, oversampling_label, sector_features,
                                  widths_from_prediction)
    from xped_gb300.workloads import power_law_sectors, power_law_spectra
    L = lib()

    def exact_keep(spectra):
        vals = np.concatenate(spectra)
        sec = np.concatenate([np.full(len(sp), a) for a, sp in enumerate(spectra)])
        top = np.argsort(-vals, kind="stable")[:chi]
        return np.bincount(sec[top], minlength=len(spectra))

    def sequence(seed):
        for t in range(steps):
            sc = 1.0 + drift * t
            secs = power_law_sectors(seed, exponent_scale=sc)
            yield t, secs, power_law_spectra(secs, sc)

    # training set: features from step t-1, labels from step t (known spectra, no decomposition needed)
    X, T = [], []
    for seed in train_seeds:
        prev = None
        for t, secs, spectra in sequence(seed):
            keep = exact_keep(spectra)
            if prev is not None:
                ns = [n for _q, n, *_ in secs]
                X.append(sector_features(ns, ns, chi, history_from_spectra(*prev)))
                for sp, k, n in zip(spectra, keep, ns):
                    T.append([np.log2(1.0 + k), np.log2(1.0 + oversampling_label(sp, int(k), n))])
            prev = (spectra, keep)
    X = np.concatenate(X).astype(np.float32)
    T = np.asarray(T, np.float32)
    model = RankModel(seed=SEED)
    t0 = time.perf_counter()
    loss0 = model.gradient(X, T)[0]
    loss = model.train(X, T, steps=3000, lr=2e-3)
    train = {"samples": int(X.shape[0]), "adam_steps": 3000, "loss_first": loss0, "loss_last": loss,
             "seconds": time.perf_counter() - t0}

    forms = ("exact", "history", "learned")
    acc = {f: {"ms": 0.0, "sketch_cols": 0, "exact_cols": 0, "keep_mismatch": 0, "max_rel_err": 0.0,
               "saturated": 0} for f in forms}
    n_dec = n_sec = 0
    cpu = None
    vendor = []

    def vendor_svd_ms(blocks):
        """torch.linalg.svd (cuSOLVER, FP64) of every block, same GPU: a library reference point
        for the exact per-sector SVD, not part of this library."""
        import torch
        dev = torch.device("cuda", torch.cuda.current_device())
        tb = [torch.from_numpy(np.ascontiguousarray(b)).to(dev) for b in blocks]
        out = {}
        for drv in ("gesvd", "gesvdj"):
            for b in tb[:2]:
                torch.linalg.svd(b, full_matrices=False, driver=drv)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for b in tb:
                torch.linalg.svd(b, full_matrices=False, driver=drv)
            e1.record()
            torch.cuda.synchronize()
            out[drv] = e0.elapsed_time(e1)
        return out

    for seed in eval_seeds:
        prev = None
        for t, secs, spectra in sequence(seed):
            pairs = [(q, n) for q, n, *_ in secs]
            B = Basis.from_pairs("U1", pairs, sort=True)
            A = Tensor.zeros([B], [B])
            A.set_data(np.concatenate([b.ravel(order="F") for *_r, b in secs]))
            keep_true = exact_keep(spectra)
            if prev is None:
                prev = (spectra, keep_true)
                continue
            ns = [n for _q, n, *_ in secs]
            hist = history_from_spectra(*prev)
            widths = {"history": [h["keep"] + max(16, int(np.ceil(0.5 * h["keep"]))) for h in hist],
                      "learned": widths_from_prediction(model.predict(sector_features(ns, ns, chi, hist)))}
            ref_s = np.concatenate([sp[:k] for sp, k in zip(spectra, keep_true)])
            for f in forms:
                def run():
                    if f == "exact":
                        return A.tSVD(chi, 1e-10)
                    return A.tSVD_randomized(chi, 1e-10, widths[f], p, seed=SEED)
                if t == 1:
                    run()  # build the plans (the structure is fixed along a sequence)
                L.xgb_synchronize()
                L.xgb_event_record(10)
                out = run()
                L.xgb_event_record(11)
                acc[f]["ms"] += L.xgb_event_elapsed_ms(10, 11)
                keep = out[5]
                acc[f]["keep_mismatch"] += int(sum(int(a) != int(b) for a, b in zip(keep, keep_true)))
                got = np.concatenate([np.diag(b) for b in out[1].blocks().values()])
                if got.size == ref_s.size:
                    acc[f]["max_rel_err"] = max(acc[f]["max_rel_err"],
                                                float(np.abs(np.sort(got)[::-1] - np.sort(ref_s)[::-1]).max()
                                                      / ref_s.max()))
                else:
                    acc[f]["max_rel_err"] = float("inf")
                if f == "exact":
                    acc[f]["exact_cols"] += sum(ns)
                else:
                    for w, n in zip(out[6], ns):
                        if 0 < w and 2 * w < n:
                            acc[f]["sketch_cols"] += int(w)
                        else:
                            acc[f]["exact_cols"] += n
                    acc[f]["saturated"] += int(out[7])
            n_dec += 1
            n_sec += len(secs)
            if seed == eval_seeds[0]:
                vendor.append(vendor_svd_ms([b for *_r, b in secs]))
            if cpu is None:
                import oracle
                from oracle.basis import Qbasis
                sym = oracle.make_symmetry("u1")
                oB = Qbasis.from_pairs(sym, pairs, sort=True)
                ot = oracle.Tensor(sym, [oB], [oB], fill=False)
                for q, _n, _a, _c, b in secs:
                    ot.push_back(q, b)
                t0 = time.perf_counter()
                ot.tsvd(chi, 1e-10)
                cpu = {"ms": (time.perf_counter() - t0) * 1e3, "cores": os.cpu_count(), "kind": "port",
                       "sample": f"seed {seed} step {t}: numpy/OpenBLAS gesvd per sector + cutoff_matrices"}
            prev = (spectra, keep_true)
    res = {"decompositions": n_dec, "sectors": n_sec, "chi": chi, "power_iters": p, "drift": drift,
           "train": train, "cpu_one_matrix": cpu}
    if vendor:
        res["torch_linalg_svd_ms_per_decomposition"] = {
            k: float(np.mean([v[k] for v in vendor])) for k in vendor[0]}
        res["torch_linalg_svd_sample"] = (f"seed {eval_seeds[0]}, {len(vendor)} matrices, full thin SVD of every "
                                          "block (cuSOLVER through torch, FP64), no truncation")
    for f in forms:
        a = acc[f]
        a["ms_per_decomposition"] = a.pop("ms") / n_dec
        res[f] = a
    return res


def fp64_library_peak(n=4096, reps=5):
    """cuBLAS DGEMM (torch.matmul, FP64, n x n x n) on this GPU: the measured FP64 rate the FP64
    kernels are compared with (the driver's peak file measures HBM and BF16 only)."""
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())
    g = torch.Generator(device=dev).manual_seed(SEED)
    a = torch.randn(n, n, dtype=torch.float64, device=dev, generator=g)
    b = torch.randn(n, n, dtype=torch.float64, device=dev, generator=g)
    for _ in range(2):
        a @ b
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        a @ b
    e1.record()
    torch.cuda.synchronize()
    return 2.0 * n ** 3 * reps / (e0.elapsed_time(e1) * 1e-3) / 1e12


def roofline(prof, steps, fp64_peak=None):
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
        # SVD work is counted as the thin R-SVD flop count 6mn^2 + 20n^3 (m >= n, Golub & Van Loan).
        achieved = per_launch_work / (per_launch_ms * 1e-3) / 1e12
        out = {"bound": "fp64", "kernel": dom, "achieved": achieved, "peak": fp64_peak or 1.25, "unit": "TFLOP/s",
               "peak_source": ("cuBLAS DGEMM 4096^3 (torch.matmul FP64) measured on this GPU in this run; nominal "
                               "1.25" if fp64_peak else "nominal GB300 FP64 rate (no FP64 figure measured)"),
               "work": "thin R-SVD flops 6mn^2+20n^3" if dom == "svd_jacobi" else "useful flops"}
    elif dom == "gemm_f64tc":
        # FP64-accurate form: each useful FP64 multiply-add is 28 BF16 slice products on the tensor pipe
        bf = peaks.get("bf16_tflops", 1900.0)
        useful = per_launch_work / (per_launch_ms * 1e-3) / 1e12
        out = {"bound": "tensor", "kernel": dom, "achieved": 28.0 * useful, "peak": bf, "unit": "TFLOP/s",
               "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst)" if "bf16_tflops" in peaks else "fallback 1900",
               "work": "BF16 products issued: 28 slice products per useful FP64 flop (slicing launches included)",
               "useful_fp64_equivalent_tflops": useful,
               "useful_vs_fp64_peak": useful / fp64_peak if fp64_peak else None}
    elif dom == "gemm_tc":
        tf = peaks.get("bf16_tflops", 1900.0) / 2.0  # dense TF32 issues at half the BF16 rate
        achieved = per_launch_work / (per_launch_ms * 1e-3) / 1e12
        out = {"bound": "tensor", "kernel": dom, "achieved": achieved, "peak": tf, "unit": "TFLOP/s",
               "peak_source": "half of MEASURED_PEAKS.json bf16_tflops (dense TF32 rate)",
               "work": "useful flops (each taken as three TF32 products)"}
    else:
        achieved = per_launch_work / (per_launch_ms * 1e-3) / 1e9
        out = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
               "peak_source": "MEASURED_PEAKS.json hbm_gbs" if "hbm_gbs" in peaks else "fallback 6800 GB/s"}
    out["frac"] = out["achieved"] / out["peak"]
    # DRAM bytes per launch of the dominant kernel from one ncu capture (profiles/): the chosen
    # step's working sets are L2-resident
    traffic = {"svd_jacobi": (0.355e6, "ncu capture of one svd_cluster_kernel launch of the projected l x l "
                                       "factors, U(1) D=6 chi=128 (dram__bytes_read.sum 322 KB + write 33 KB)"),
               "gemm_tc": (7.025e9, "ncu capture, SU(2) Tensor<2,2> product (6.613 GB read + 0.412 GB written)"),
               "gemm_f64tc": (68.27e6, "ncu one-pass capture of the 76 oz_gemm_kernel launches of one chosen U(1) D=6 "
                                       "chi=128 step (bench.py --profile-step): 67.44 MB read + 0.83 MB written per "
                                       "launch, average (the packed slices of the sector blocks)"),
               "gemm_f64": (14.10e6, "ncu one-pass capture of 348 consecutive gemm_simt_kernel launches of the "
                                     "chosen U(1) D=6 chi=128 run (dram read + write per launch, average; the "
                                     "operands are L2-resident after their first touch)")}
    out["traffic"] = traffic[dom][0] if dom in traffic else None
    if dom in traffic:
        out["traffic_source"] = traffic[dom][1]
    out["launches_per_step"] = n / max(steps, 1)
    out["ms_per_launch"] = per_launch_ms
    out["kernel_share"] = {k: round(v[1] / sum(x[1] for x in kinds.values()), 4) for k, v in kinds.items()}
    out["kernel_ms_per_step"] = {k: round(v[1] / max(steps, 1), 3) for k, v in kinds.items()}
    return out


# ----------------------------------------------------------------------------- CPU oracle
def oracle_ctm(aux_pairs, chi):
    import oracle
    from oracle.basis import Qbasis
    from oracle.ctm import CTM as OCTM
    from oracle.ctm import IPEPS

    s = oracle.make_symmetry("u1")
    aux = Qbasis.from_pairs(s, aux_pairs)
    phys = Qbasis.from_pairs(s, PHYS)
    peps = IPEPS(s, aux, phys)
    data = np.random.default_rng(SEED).standard_normal(sum(b.size for b in peps.A.blocks))
    o = 0
    for i, b in enumerate(peps.A.blocks):
        peps.A.blocks[i] = data[o:o + b.size].reshape(b.shape, order="F")
        o += b.size
    peps.update_adag()
    return OCTM(peps, chi).init()


def time_moves(c, n_moves):
    times = []
    for i in range(n_moves):
        t0 = time.perf_counter()
        c.move("LRTB"[i % 4])
        times.append(time.perf_counter() - t0)
    return times


def cpu_baseline_from_device(ctm):
    """One whole grow_all step (four moves) of the oracle port on a host copy of the device environment
    (saturated chi), all host cores."""
    import oracle
    from oracle.convert import ctm_from_native
    oc = ctm_from_native(oracle.make_symmetry("u1"), ctm, CHI)
    t = float(sum(time_moves(oc, 4)))
    return {"value": 1.0 / t, "unit": "steps/s", "cores": os.cpu_count(), "kind": "port",
            "sample": f"one grow_all step (L, R, T, B moves, {t:.1f} s) of the numpy/OpenBLAS oracle on a host copy "
                      "of the saturated device environment"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--gemm", default="f64tc", choices=["fp64", "3xtf32", "fp32", "f64tc"],
                    help="block GEMM form of the chosen CTM step; f64tc (FP64-accurate tensor-core products from "
                         "exact BF16 slices) also covers the projector and sketch products")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--sketch-tail", type=int, default=SKETCH_TAIL,
                    help="subspace iterations of the chosen form kept in FP64 at the end; the earlier ones "
                         "(and the first sketch product) multiply as 3xTF32 tensor-core GEMMs (< 0: all FP64)")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP64 comparison")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-width run")
    ap.add_argument("--no-converge", action="store_true", help="skip the runs to convergence (CTMSolver::solve)")
    ap.add_argument("--autotune", type=int, default=1, choices=[0, 1],
                    help="1: FP64 GEMM shapes from the library's autotuner (tuned during the warm-up); 0: built-in rule")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the compact learned-tSVD sweep and fermionic Z2 runs folded into the default run")
    ap.add_argument("--tol-e", type=float, default=1e-10, help="energy tolerance of the solver (reference default)")
    ap.add_argument("--solve-max-steps", type=int, default=60, help="grow_all steps the solver may take")
    ap.add_argument("--workload", default="u1", choices=["u1", "fz2"],
                    help="u1: the headline U(1) D=6 chi=128 step; fz2: fermionic Z2 D=6 chi=144, 20 iterations")
    ap.add_argument("--fz2-plain-steps", type=int, default=2,
                    help="steps of the plain FP64 form on the fz2 workload (0: skip)")
    ap.add_argument("--gemm-sweep-only", action="store_true",
                    help="run only the block-GEMM sweep and print it (for kernel profiling)")
    ap.add_argument("--u1-product", default=None, metavar="DEGS",
                    help="time only T1*T2 of U(1) Tensor<2,2> operands with these leg degeneracies (e.g. 6,12,16,12,6)")
    ap.add_argument("--reps", type=int, default=10, help="products timed by --u1-product")
    ap.add_argument("--profile-step", action="store_true",
                    help="warm up the chosen form, then run one step between cudaProfilerStart / Stop (for ncu "
                         "--profile-from-start off) and print its CUDA-event time")
    ap.add_argument("--autotune-cache", default=None, metavar="PATH",
                    help="with --profile-step: load the autotuner's choices from PATH if it exists, else measure "
                         "them during the warm-up and save them there")
    ap.add_argument("--permute-only", action="store_true",
                    help="run only the permute HBM roofline case (1.42 GB U(1) Tensor<2,2>) and print it")
    ap.add_argument("--permute-degs", default="20,40,60,40,20",
                    help="leg degeneracies of the permute case (charges -2..2), e.g. 10,20,30,20,10 for profiling")
    ap.add_argument("--tsvd-sweep-only", action="store_true",
                    help="run only the learned-width randomized tSVD sweep on power-law block matrices")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    rank, world, local = dist_info()
    config = {"workload": WORKLOAD, "chi": CHI, "D": 6, "aux": "q -1,0,1 deg [2,2,2]", "phys": 2, "cell": "1x1",
              "l2": "512 MB buffer written between timed steps (outside the timed events)"}

    if args.impl == "reference":
        if rank != 0:
            return
        # one CPU step of this workload takes ~20 s on the GPU host's cores, so the K requested steps are
        # sampled as ceil(K / 4) whole grow_all steps after min(W, 2) warm-up steps (chi saturates
        # after the first step): ms_per_step x steps is the timed CPU work
        c = oracle_ctm(AUX, CHI)
        warm = min(args.warmup, 2)
        for _ in range(warm):
            c.grow_all()
        n_steps = max(1, (args.steps + 3) // 4)
        times = []
        for _ in range(n_steps):
            t0 = time.perf_counter()
            c.grow_all()
            times.append(time.perf_counter() - t0)
        t = float(np.mean(times))
        v = 1.0 / t
        line = {"metric": METRIC, "value": v, "unit": "steps/s", "n_gpus": args.gpus, "steps": n_steps,
                "warmup": warm, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded N(0,1) site tensor)",
                "config": dict(config, form="reference algorithm (exact FP64 tSVD), numpy/OpenBLAS"),
                "impl": "reference",
                "cpu_baseline": {"value": v, "unit": "steps/s", "cores": os.cpu_count(), "kind": "port",
                                 "sample": f"{n_steps} whole grow_all steps (ceil(K/4) of the K = {args.steps} "
                                           f"requested) after {warm} warm-up steps"},
                "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    if args.workload == "fz2" and args.impl == "ours":
        if rank == 0:
            run_fz2(args)
        return

    if args.u1_product:
        from xped_gb300 import ensure_device
        ensure_device(local)
        print(json.dumps({"u1_product": u1_product([int(x) for x in args.u1_product.split(",")], args.reps,
                                                     args.gemm)}))
        return

    if args.profile_step:
        print(json.dumps({"profiled_step": profile_step(args)}))
        return

    if args.permute_only:
        from xped_gb300 import ensure_device
        ensure_device(local)
        print(json.dumps({"permute_roofline": permute_roofline(tuple(int(x) for x in args.permute_degs.split(",")))}))
        return

    if args.tsvd_sweep_only:
        from xped_gb300 import ensure_device
        ensure_device(local)
        print(json.dumps({"tsvd_sweep": tsvd_sweep()}))
        return

    if args.gemm_sweep_only:
        from xped_gb300 import ensure_device
        ensure_device(local)
        print(json.dumps({"block_gemm_sweep": gemm_sweep()}))
        return

    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    r = run_gpu(args)
    t_step, t_e2e = r["step_ms"], r["e2e_ms"]
    if world > 1:
        t_step, t_e2e = max_over_ranks([t_step, t_e2e])
        ranks_barrier()
    if rank != 0:
        return
    value = world * 1e3 / t_step
    prof = r["prof"]
    gemm_kind = {"3xtf32": "gemm_tc", "fp32": "gemm_f32", "f64tc": "gemm_f64tc"}.get(args.gemm, "gemm_f64")
    g = prof.get(gemm_kind, (0, 0.0, 0.0))
    line = {"metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": dtype_label(args),
            "data": "synthetic (seeded N(0,1) site tensor)",
            "config": dict(config, form=f"chosen: randomized projector SVD ({POWER_ITERS} subspace iterations, "
                                        "CholeskyQR3 bases, widths last kept + max(16, 50%), exact first decomposition "
                                        "per direction and exact FP64 fallback), FP64 SVD core" + gemm_form_label(args),
                           gemm=args.gemm, parallelism=f"replicas x{world}"),
            "e2e": {"value": world * 1e3 / t_e2e, "unit": "steps/s", "h2d_bytes_per_step": r["h2d"],
                    "d2h_bytes_per_step": r["d2h"]},
            "gpu_launches": r["launches"], "gpu_launches_per_step": r["launches_per_step"], "clocks": r["clocks"],
            "roofline": roofline(prof, r["prof_steps"], r.get("fp64_peak")),
            "block_gemm": {"form": args.gemm, "tflops": (g[2] / (g[1] * 1e-3) / 1e12) if g[1] > 0 else None,
                           "ms_per_step": g[1] / r["prof_steps"]},
            "sketch": dict(r["sketch"], cols_per_step=r["cols_per_step"], redo_per_step=r["redo_per_step"]),
            "autotune": r["autotune"] if args.autotune else {"enabled": False},
            "step_ms_each": [round(x, 3) for x in r["step_ms_all"]]}
    if "plain_ms" in r:
        line["plain_fp64"] = {"ms_per_step": r["plain_ms"], "steps_per_s": 1e3 / r["plain_ms"],
                              "timed": f"step {COMPARE_STEPS} of a fresh plain run (one step)"}
        line["chosen_vs_plain"] = r["plain_ms"] / t_step
        line["energy"] = {"after_steps": COMPARE_STEPS, "chosen": r["e_chosen"], "plain": r["e_plain"],
                          "abs_diff": abs(r["e_chosen"] - r["e_plain"]),
                          "observable": "Heisenberg energy per site (rho_h + rho_v bonds)"}
    else:
        line["energy"] = {"after_steps": COMPARE_STEPS, "chosen": r["e_chosen"]}
    conv = {}
    for form in ("chosen", "plain", "learned"):
        if f"solve_{form}" in r:
            conv[form] = r[f"solve_{form}"]
    if conv:
        # this workload's converged CTM energy alternates between two values from step to step (a
        # period-2 environment): each form's last two energies are its two branches, compared branch
        # by branch (the solver may stop on either branch)
        for form, c in conv.items():
            c["branches"] = sorted(c["energies"][-2:])
        line["energy_converged"] = dict(conv, observable="Heisenberg energy per site (rho_h + rho_v bonds)",
                                        rule="CTMSolver::solve: stop when |E - E_prev| < tol_E or |E - E_prevprev| < tol_E",
                                        comparison="largest difference between the sorted last-two-step energies")
        if "plain" in conv:
            for form in ("chosen", "learned"):
                if form in conv:
                    line["energy_converged"][f"abs_diff_{form}_vs_plain"] = max(
                        abs(a - b) for a, b in zip(conv[form]["branches"], conv["plain"]["branches"]))
    if "learned_ms" in r:
        line["learned_widths"] = {"ms_per_step": r["learned_ms"], "steps_per_s": 1e3 / r["learned_ms"],
                                  "sketch_cols_per_step": r["learned_cols_per_step"],
                                  "redo_per_step": r["learned_redo_per_step"], "train": r["learned_train"]}
        if "e_plain" in r:
            line["learned_widths"]["energy_abs_diff_vs_plain"] = abs(r["e_learned"] - r["e_plain"])
    line["plain_fp64_D4_chi32_ms_per_step"] = r["small_plain_ms"]
    line["block_gemm_sweep"] = r["gemm_sweep"]
    line["tensor22_chain"] = r["tensor22_chain"]
    line["simple_update_step"] = r["su"]
    line["permute_roofline"] = r["permute_roofline"]
    if "tsvd_sweep" in r:
        line["learned_tsvd_sweep"] = r["tsvd_sweep"]
    if "fz2" in r:
        line["fermionic_z2_chosen_form"] = r["fz2"]
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_from_device(r["ctm"])
    print(json.dumps(line))


if __name__ == "__main__":
    main()
