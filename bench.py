#!/usr/bin/env python
"""MLSD EM iteration throughput (muon-voxel updates per second) on one scan.

Default workload: the 100^3-voxel, 2 cm, 10M-muon scan (iron / lead /
aluminium blocks and a concrete slab, momentum known per muon), median EM
update (the reference's default), mixed precision, graph-captured iteration.
A step is one EM iteration over all kept muons; value = muon-voxel pairs per
iteration x steps / time.  Inputs are synthetic (seeded generator), resident
in HBM before the timed region; the per-iteration working set (lists, S) is
far larger than L2, so no flush is needed between steps.

--impl reference times the reference's CPU implementation of the same path
(the FP64 restatement in oracle/, serial muon loop + OpenMP voxel loop, all
host cores) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

# --workload choices: grid, voxel size and muon count of each scan
WORKLOADS = {
    "cube100_20mm": lambda W: W.cube100_20mm,  # 100^3 voxels of 20 mm, 10 M muons (default)
    "cube50_40mm": lambda W: W.cube50_40mm,  # the same scene on 50^3 voxels of 40 mm, 2.5 M muons
    "cube20_50mm": lambda W: W.cube20_50mm,  # 20^3 voxels of 50 mm, 100 k muons
    "map128x128x64_15mm": lambda W: W.map128x128x64_15mm,  # 128x128x64 voxels of 15 mm, 20 M muons
    "grid256x256x128_10mm": lambda W: W.grid256x256x128_10mm,  # 256x256x128 voxels of 10 mm, 100 M muons
}

METRIC = "EM-iter muon\u00b7voxel updates/s"  # the headline metric's own wording
UNIT = "muon\u00b7voxel updates/s"


def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        # the timed region starts once sampling has begun (first line, at most 3 s)
        t0 = time.time()
        while time.time() - t0 < 3.0 and self.proc.poll() is None:
            if Path(self.f.name).stat().st_size > 0:
                break
            time.sleep(0.02)

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.flush()
        rows = [r.split(",") for r in Path(self.f.name).read_text().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except ValueError:
                continue
            for n, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    from muontomography_gb300.replicas import env

    return env()


def workload(args, rank: int):
    from muontomography_gb300 import workloads as W
    from muontomography_gb300.replicas import replica_seed

    fn = WORKLOADS[args.workload](W)
    kw = {}
    if args.n_muons:
        kw["n_muons"] = args.n_muons
    wl = fn(**kw)
    wl.seed = replica_seed(wl.seed, rank)  # every rank reconstructs its own scan (weak scaling)
    return wl


# DRAM bytes per pair per launch, measured by ncu (--set full) on the 50^3-voxel
# 2.5 M-muon case of the default scene (median EM, mixed form): muon pass
# 868.4 MB and voxel pass (key pass and all classes) 1378.5 MB for 68 700 086 pairs
TRAFFIC_PER_PAIR = {"muon": 868.4e6 / 68700086, "voxel": 1371.0e6 / 68700086}

# set-up kernels and host phases reported by the library's profiler
SETUP_KERNELS = ["keep_flags", "scan", "compact", "muon_info", "siddon_count", "siddon_fill", "voxel_offset",
                 "voxel_hist", "voxel_major", "voxel_classes", "path_bound", "path_compact"]
SETUP_PHASES = ["gather", "info_count", "offsets", "fill", "voxel_major", "classes", "tiles", "image", "autotune"]


def method_of(args) -> str:
    """MAP for the MAP workload (128x128x64 voxels of 15 mm), MLSD otherwise."""
    return "map" if args.workload.startswith("map") else "mlsd"


def em_config(wl, args, precision: str, n_iter: int) -> dict:
    over = {"precision": precision, "num_iteration": n_iter, "muon_pass": args.muon_pass,
            "muon_layout": args.muon_layout}
    if method_of(args) == "map":  # beta 0.01, p = 1, the 26-neighbour stencil, delta = 0.1 median(lambda) 1e7
        over.update(beta=0.01, p=1.0, all_neighbours=True, delta=0.1 * float(np.median(wl.lam())) * 1e7)
    if getattr(args, "voxel_stream_above", None) is not None:
        over["voxel_stream_above"] = args.voxel_stream_above
    if args.mode == "mean":
        over.update(update_with_mean=True, mean_percentile=100)
    return wl.em_config(**over)


def cpu_port(wl, args, n_sample: int, n_iter: int, threads: int) -> dict:
    """Time the CPU restatement of the reference path on a sample of the workload."""
    os.environ["OMP_NUM_THREADS"] = str(threads)
    import muontomography_gb300 as M
    from oracle import oracle as O

    rays = M.generate(wl.grid, wl.lam(), n_sample, wl.seed)
    cfg = em_config(wl, args, "fp64", n_iter)
    init = np.full(wl.grid.nvox, 1e-7)
    t0 = time.perf_counter()
    ref = O.Mlsd(wl.grid, cfg, rays, init, keep_paths=False, method=method_of(args))
    t_setup = time.perf_counter() - t0
    pairs = ref.counts()["n_pairs"]
    times = []
    for _ in range(n_iter):
        t0 = time.perf_counter()
        ref.iterate(1)
        times.append(time.perf_counter() - t0)
    return {"pairs": pairs, "times": times, "setup_s": t_setup, "n_sample": n_sample}


def run_reference(args) -> int:
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    wl = workload(args, 0)
    threads = os.cpu_count() or 1
    n_sample = args.cpu_sample
    r = cpu_port(wl, args, n_sample, args.warmup + args.steps, threads)
    t = r["times"][args.warmup:]
    value = r["pairs"] * len(t) / sum(t)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000 * sum(t) / len(t), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": wl.name, "method": method_of(args), "grid": list(wl.grid.shape), "mode": args.mode,
                   "sample_muons": n_sample, "sample_pairs": r["pairs"]},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{n_sample} muons of {wl.name}: one EM iteration per step "
                                   f"({r['pairs']} pairs), setup {r['setup_s']:.2f} s untimed"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args) -> int:
    import torch

    from muontomography_gb300.replicas import Replicas

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    rep = Replicas("nccl")
    barrier, allmax, allsum = rep.barrier, rep.max, rep.sum

    import muontomography_gb300 as M
    from muontomography_gb300 import _lib

    lib = M.library()
    wl = workload(args, rank)
    n = wl.n_muons
    lam = torch.tensor(wl.lam(), dtype=torch.float64, device="cuda")
    d_rays = torch.empty((n, 14), dtype=torch.float64, device="cuda")
    prm = _lib.muto_gen_params(wl.seed, np.pi / 3, 1.0, 10.0, 3.0, 500.0, 3, 0, 1.0)
    g = wl.grid.c()
    t0 = time.perf_counter()
    _lib.check(lib.muto_generate_device(C.byref(g), C.c_void_p(lam.data_ptr()), C.byref(prm), 0, n,
                                        C.c_void_p(d_rays.data_ptr()),
                                        C.c_void_p(torch.cuda.current_stream().cuda_stream)), "generate")
    torch.cuda.synchronize()
    t_gen = time.perf_counter() - t0

    # ---- value: EM iterations with the tracks resident in HBM ---------------
    cfg = em_config(wl, args, args.precision, args.warmup + args.steps)
    rec = M.Reconstruction(method_of(args), cfg)
    rec.load_tracks(None, on_device_ptr=d_rays.data_ptr(), n=n)
    rec.set_profiling(True)
    t0 = time.perf_counter()
    rec.prepare()
    t_setup = time.perf_counter() - t0
    setup_ms = {}
    for name in SETUP_KERNELS + ["host:" + p for p in SETUP_PHASES]:
        cnt, tot = rec.kernel_stats(name)
        if cnt:
            setup_ms[name] = round(tot, 3)
    st = rec.status()
    pairs, kept, V = st["n_pairs"], st["n_scat_in_grid"], wl.grid.nvox
    sp = C.c_void_p()
    lib.muto_get_stream(rec._h, C.byref(sp))
    stream = torch.cuda.ExternalStream(sp.value)
    for _ in range(args.warmup):
        rec.iterate(1)
    cnt, tot = rec.kernel_stats("host:graph_capture")
    if cnt:
        setup_ms["host:graph_capture"] = round(tot, 3)
    rec.reset_kernel_stats()
    l0 = rec.launch_count()
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        rec.iterate(1)
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    barrier()
    ms_local = e0.elapsed_time(e1)
    clk = clocks.stop()
    launches = rec.launch_count() - l0
    ms = allmax(ms_local)
    total_pairs = allsum(float(pairs))
    value = total_pairs * args.steps / (ms / 1000.0)
    nm_, tm_ = rec.kernel_stats("em_muon")
    nv_, tv = rec.kernel_stats("em_voxel")
    rec.set_profiling(False)
    rec.close()

    # algorithmic bytes per launch (mixed: 4-byte index, L, T; fp64: 8-byte L, T)
    rb = 4 if args.precision == "mixed" else 8
    muon_bytes = (4 + 2 * rb) * pairs + (4 * rb + rb + 8 + 4 * rb) * kept + rb * V  # lists, S/D/pr2/off, k out, lambda
    voxel_bytes = (4 + 2 * rb) * pairs + (16 + 6 * rb) * V  # voxel-major lists; descriptor, lambda in/out, window in/out
    pk = peaks()
    muon_ms = tm_ / max(nm_, 1)
    voxel_ms = tv / max(nv_, 1)  # the voxel pass: all class launches of one iteration
    achieved = muon_bytes / (muon_ms / 1000.0) / 1e9 if nm_ else None
    v_ach = voxel_bytes / (voxel_ms / 1000.0) / 1e9 if nv_ else None
    # DRAM traffic (read + write) per launch: ncu's bytes per pair on the 50^3-voxel
    # case of the same scene, scaled by this run's pairs
    measured = args.precision == "mixed" and args.mode == "median" and args.workload in ("cube100_20mm", "cube50_40mm")
    t_voxel = (args.ncu_traffic if args.ncu_traffic is not None
               else (TRAFFIC_PER_PAIR["voxel"] * pairs if measured else None))
    t_muon = TRAFFIC_PER_PAIR["muon"] * pairs if measured else None
    # the voxel pass takes about two thirds of an iteration: it is the dominant kernel
    roofline = {"bound": "hbm", "achieved": v_ach, "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": (v_ach / pk["hbm_gbs"]) if v_ach else None, "traffic": t_voxel,
                "kernel": "k_pair_keys + k_em_voxel (one launch per segment-length class)", "kernel_ms": voxel_ms,
                "algorithmic_bytes": voxel_bytes, "peak_source": pk["source"],
                "muon_pass": {"kernel": "k_em_muon", "kernel_ms": muon_ms, "algorithmic_bytes": muon_bytes,
                              "achieved": achieved, "frac": (achieved / pk["hbm_gbs"]) if achieved else None,
                              "traffic": t_muon}}

    # ---- e2e: full reconstruct through the C ABI from pinned host tracks ------
    e2e = None
    if args.e2e_steps > 0:
        host = torch.empty((n, 14), dtype=torch.float64, pin_memory=True)
        host.copy_(d_rays)
        del d_rays
        torch.cuda.empty_cache()
        e_iters = args.e2e_iters if args.e2e_iters > 0 else wl.n_iter  # the workload's reconstruct call
        ecfg = em_config(wl, args, args.precision, e_iters)
        out = np.empty(V, np.float64)
        times = []
        for k in range(args.e2e_steps + 1):  # the first call is a warm-up
            r2 = M.Reconstruction(method_of(args), ecfg)
            lib.muto_get_stream(r2._h, C.byref(sp))
            s2 = torch.cuda.ExternalStream(sp.value)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            barrier()
            torch.cuda.synchronize()
            a.record(s2)
            rc = lib.muto_reconstruct(r2._h, C.c_void_p(host.data_ptr()), n, _lib.dptr(out), V)
            b.record(s2)
            b.synchronize()
            _lib.check(rc, "muto_reconstruct")
            if k > 0:
                times.append(a.elapsed_time(b))
            r2.close()
        # the set-up of one more reconstruct, untimed, by phase (modules loaded)
        r2 = M.Reconstruction(method_of(args), ecfg)
        r2.set_profiling(True)
        t0 = time.perf_counter()
        r2.load_tracks(host.numpy())
        setup_warm = {"load_tracks_h2d": round((time.perf_counter() - t0) * 1e3, 3)}
        t0 = time.perf_counter()
        r2.prepare()
        setup_warm["prepare"] = round((time.perf_counter() - t0) * 1e3, 3)
        for name in SETUP_KERNELS + ["host:" + p for p in SETUP_PHASES]:
            cnt, tot = r2.kernel_stats(name)
            if cnt:
                setup_warm[name] = round(tot, 3)
        r2.close()
        e_ms = allmax(statistics.mean(times))
        e2e = {"value": total_pairs * e_iters / (e_ms / 1000.0), "unit": UNIT,
               "h2d_bytes_per_step": int(n * 14 * 8), "d2h_bytes_per_step": int(V * rb),
               "ms_per_step": e_ms, "em_iterations_per_step": e_iters, "setup_ms": setup_warm,
               "what": "muto_reconstruct: H2D of pinned tracks, setup (gather, Siddon lists), "
                       f"{e_iters} EM iterations (the workload's num_iteration), D2H of the image"}
    else:
        host = None

    # ---- time to lambda: mixed vs the plain FP64 form, same iteration count ---
    ttl = None
    if args.ttl_iters > 0 and rank == 0:
        if host is None:
            host = torch.empty((n, 14), dtype=torch.float64, pin_memory=True)
            host.copy_(d_rays)
            del d_rays
        res = {}
        for prec in ("fp64", "mixed"):
            d = torch.empty((n, 14), dtype=torch.float64, device="cuda")
            d.copy_(host)
            r3 = M.Reconstruction(method_of(args), em_config(wl, args, prec, args.ttl_iters))
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r3.load_tracks(None, on_device_ptr=d.data_ptr(), n=n)
            r3.prepare()
            r3.iterate(args.ttl_iters)
            im = r3.image()
            res[prec] = (time.perf_counter() - t0, im)
            r3.close()
            del d
            torch.cuda.empty_cache()
        a64, b32 = res["fp64"][1].ravel(), res["mixed"][1].ravel()
        rel = float(np.linalg.norm(b32 - a64) / np.linalg.norm(a64))
        ttl = {"iterations": args.ttl_iters, "fp64_s": res["fp64"][0], "mixed_s": res["mixed"][0],
               "rel_l2_mixed_vs_fp64": rel, "speedup": res["fp64"][0] / res["mixed"][0],
               "within_1e-4": rel < 1e-4}

    # ---- CPU baseline on this machine's host cores (rank 0 only) ----------------
    cpu = None
    if rank == 0 and args.cpu_sample > 0:
        threads = os.cpu_count() or 1
        r = cpu_port(wl, args, args.cpu_sample, 2, threads)
        cval = r["pairs"] * len(r["times"]) / sum(r["times"])
        cpu = {"value": cval, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{args.cpu_sample} muons of the same workload, 2 EM iterations "
                         f"({r['pairs']} pairs each), setup untimed"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32" if args.precision == "mixed" else "f64",
            "data": "synthetic",
            "config": {"workload": wl.name, "method": method_of(args), "grid": list(wl.grid.shape),
                       "voxel_mm": wl.grid.dx, "muons": n,
                       "kept_muons": kept, "pairs_per_iteration": pairs, "mode": args.mode,
                       "precision": args.precision, "per_muon_2x2": "f64", "graph": True,
                       "parallelism": f"replicas x{world} (one scan per GPU)",
                       "l2": "inputs larger than L2: pair lists and s_ij far exceed 126 MB, no flush",
                                  "setup_s": t_setup, "setup_ms": setup_ms, "generate_s": t_gen, "muon_pass": {1: "tma_tiles", 2: "warp_batched"}.get(st["muon_pass"]),
            "muon_group": st["muon_group"], "tile_pairs": st["tile_pairs"]},
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": int(launches),
            "clocks": clk,
            "time_to_lambda": ttl,
        }
        print(json.dumps(line), flush=True)
    rep.close()
    return 0


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="cube100_20mm", choices=list(WORKLOADS))
    ap.add_argument("--n-muons", type=int, default=0)
    ap.add_argument("--mode", choices=["median", "mean"], default="median")
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--e2e-iters", type=int, default=0, help="EM iterations per e2e call (0: the workload's)")
    ap.add_argument("--ttl-iters", type=int, default=50)
    ap.add_argument("--cpu-sample", type=int, default=150_000)
    ap.add_argument("--muon-pass", choices=["auto", "tile", "warp"], default="auto")
    ap.add_argument("--muon-layout", choices=["auto", "columns", "index"], default="auto")
    ap.add_argument("--voxel-stream-above", type=int, default=None,
                    help="segments longer than this are selected without holding their keys (-1: never)")
    ap.add_argument("--ncu-traffic", type=float, default=None,
                    help="DRAM bytes per voxel-pass iteration from an ncu capture of this workload")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    return run_reference(args) if args.impl == "reference" else run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
