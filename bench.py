#!/usr/bin/env python
"""MLSD EM iteration throughput (muon-voxel updates per second) on one scan.

Default workload: the largest single scan -- 256x256x128 voxels of 10 mm
(8.4 M voxels) with 100 M muons through 12 mixed iron / lead / aluminium /
concrete blocks, momentum known per muon -- reconstructed with the mean EM
update over stored muon-major lists (int32 voxel index, FP32 L and T), mixed
precision, graph-captured iteration.  A step is one EM iteration over all
kept muons; value = muon-voxel pairs per iteration x steps / time.  Inputs
are synthetic (seeded generator), resident in HBM before the timed region;
the lists read every iteration (118 GB) are far larger than L2, so no flush
is needed between steps.  Beside it, the same line carries: the recomputed-
paths variant, PoCA on the same tracks, an end-to-end reconstruct from
pinned host tracks, time to lambda (mixed vs the FP64 GPU form) and the CPU
port of the reference on a sample.

--workload cube100_20mm runs the 100^3 scan with the median update (the
reference's default) over the voxel-major lists.

--impl reference times the reference's CPU implementation of the same path
(the FP64 restatement in oracle/, serial muon loop + OpenMP voxel loop, all
host cores) on a bounded sample of the same workload, with tracks made by
the oracle's own build of the generator (the product library is not loaded).
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
    "grid256x256x128_10mm": lambda W: W.grid256x256x128_10mm,  # 256x256x128 voxels of 10 mm, 100 M muons (default)
    "cube100_20mm": lambda W: W.cube100_20mm,  # 100^3 voxels of 20 mm, 10 M muons
    "cube50_40mm": lambda W: W.cube50_40mm,  # the same scene on 50^3 voxels of 40 mm, 2.5 M muons
    "cube20_50mm": lambda W: W.cube20_50mm,  # 20^3 voxels of 50 mm, 100 k muons
    "map128x128x64_15mm": lambda W: W.map128x128x64_15mm,  # 128x128x64 voxels of 15 mm, 20 M muons
    "batch64": None,  # 64 scans of 32^3..128^3 voxels of 20 mm, 50 k..5 M muons each, in one batch handle
}
# the EM update each workload is benchmarked with: the throughput workloads
# (the largest scan, whose per-voxel lists do not fit next to the muon-major
# ones, and the 64-scan batch) with the mean update, the others with the
# reference's default median
DEFAULT_MODE = {"grid256x256x128_10mm": "mean", "batch64": "mean"}

METRIC = "EM-iter muon·voxel updates/s"  # the headline metric's own wording
UNIT = "muon·voxel updates/s"

# DRAM bytes (read + write) per pair per launch from ncu captures of each
# kernel (mixed form), scaled by a run's pairs: the full workloads are above
# the capture size the profiler is run at.  Captures:
# profiles/em_split_grid256x256x128_10mm_2M.md (the 256x256x128 grid with 2 M
# muons, mean update, 195 962 860 pairs) and
# profiles/em_passes_cube50_40mm_2.5M.md (the 100^3 scene on 50^3 voxels,
# median update, 68 700 086 pairs).
TRAFFIC_PER_PAIR = {
    ("grid256", "em_muon"): (2.461541e9 + 8.514816e6) / 195962860,
    ("grid256", "em_scatter"): (2.511995e9 + 9.667328e6) / 195962860,  # the 8-deep scatter
    ("cube", "em_muon"): 868.4e6 / 68700086,
    ("cube", "em_voxel"): 1371.0e6 / 68700086,
}

# set-up kernels and host phases reported by the library's profiler
SETUP_KERNELS = ["keep_flags", "scan", "compact", "muon_info", "siddon_count", "siddon_fill", "voxel_offset",
                 "voxel_hist", "voxel_major", "voxel_classes", "path_bound", "path_compact", "path_stats"]
SETUP_PHASES = ["load_alloc", "load_copy", "gather", "info_count", "fill", "path_stats", "voxel_major", "classes",
                "tiles", "image", "autotune"]
ITER_KERNELS = ["em_muon", "em_scatter", "em_fused", "em_walk", "em_voxel", "em_update", "brick_lambda", "map_voxel",
                "map_copy", "cost"]


def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def host_cores() -> int:
    """Cores this process may run on (affinity / cgroup cpuset), not the machine's count."""
    try:
        return len(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        return os.cpu_count() or 1


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

    if args.workload == "batch64":  # the CPU legs sample the batch's first scan
        wl = W.batch64(seed=replica_seed(4, rank))[0]
        return wl
    fn = WORKLOADS[args.workload](W)
    kw = {}
    if args.n_muons:
        kw["n_muons"] = args.n_muons
    wl = fn(**kw)
    wl.seed = replica_seed(wl.seed, rank)  # every rank reconstructs its own scan (weak scaling)
    return wl


def method_of(args) -> str:
    """MAP for the MAP workload (128x128x64 voxels of 15 mm), MLSD otherwise."""
    return "map" if args.workload.startswith("map") else "mlsd"


def wl_lambda(wl) -> np.ndarray:
    """The workload's phantom, rasterised without the product library."""
    from muontomography_gb300 import X0_MM
    from oracle import synthetic as S

    return S.phantom(wl.grid, wl.blocks, X0_MM["air"], 3.0)


def em_config(wl, args, precision: str, n_iter: int, lists: str | None = None) -> dict:
    over = {"precision": precision, "num_iteration": n_iter, "muon_pass": args.muon_pass,
            "muon_layout": args.muon_layout, "path_lists": lists or args.lists, "fused_variant": args.fused_variant}
    if method_of(args) == "map":  # beta 0.01, p = 1, the 26-neighbour stencil, delta = 0.1 median(lambda) 1e7
        over.update(beta=0.01, p=1.0, all_neighbours=True, delta=0.1 * float(np.median(wl_lambda(wl))) * 1e7)
    if getattr(args, "voxel_stream_above", None) is not None:
        over["voxel_stream_above"] = args.voxel_stream_above
    if args.mode == "mean":
        over.update(update_with_mean=True, mean_percentile=100)
    return wl.em_config(**over)


def map_conditioning(wl, args, d_rays, n: int, img64: np.ndarray, img32: np.ndarray) -> dict:
    """How far the MAP EM moves under a rounding-sized change of its input.

    With p = 1 the prior's surrogate picks among up to three roots per voxel,
    and a change at the level of one rounding can switch the pick; the
    iteration then amplifies it.  The FP64 form run again from an initial
    image perturbed by 1e-7 (relative, uniform) shows that spread; the mixed
    form is judged against it and by the objective F (NLL + prior, evaluated
    in FP64) that each image reaches."""
    import muontomography_gb300 as M

    cfg = em_config(wl, args, "fp64", args.ttl_iters)
    r = M.Reconstruction(method_of(args), cfg)
    r.load_tracks(None, on_device_ptr=d_rays.data_ptr(), n=n)
    r.prepare()
    init = np.full(wl.grid.nvox, cfg["initialize_value"])
    r.set_image(init * (1.0 + 1e-7 * np.random.default_rng(12345).uniform(-1.0, 1.0, init.size)))
    r.iterate(args.ttl_iters)
    imgp = r.image()
    mult = r.multiplicity()
    r.close()
    rf = M.Reconstruction(method_of(args), dict(cfg, num_iteration=0))
    rf.load_tracks(None, on_device_ptr=d_rays.data_ptr(), n=n)
    rf.prepare()

    def objective(img):
        flat = img.reshape(-1, order="F")
        return rf.nll(np.log(np.where(mult > 0, np.maximum(flat, 1e-300), 1.0)))

    def rel(x, y):
        return float(np.linalg.norm(x - y) / np.linalg.norm(y))

    spread = rel(imgp, img64)
    out = {"rel_l2_fp64_perturbed_vs_fp64": spread, "perturbation": "initial image x (1 + 1e-7 u), u ~ U(-1, 1)",
           "F_fp64": objective(img64), "F_fp64_perturbed": objective(imgp), "F_mixed": objective(img32),
           "within_fp64_spread": bool(rel(img32, img64) <= 2.0 * spread)}
    rf.close()
    return out


def run_next_rows(wl, rays: np.ndarray) -> dict:
    """PoCut (src/MutoPoCut.cpp:19-121), SLR (src/MutoSLR.cpp:47-103), SLRIter
    (src/MutoSLRIter.cpp:15-83) and the reader's line fit
    (src/MutoFile.cpp:248-304) on the same tracks: GPU time per call
    (`reconstruct` from host tracks, copies included; the library's profiler
    for the kernels), and the oracle on the host cores for the same call."""
    import muontomography_gb300 as M
    from oracle import oracle as O

    n = rays.shape[0]
    out = {"tracks": n, "what": "wall clock of one reconstruct call from host tracks (copies and set-up included), "
                                "the best of three; the oracle on the same tracks, one call"}

    def gpu_call(make):
        best = None
        for _ in range(3):
            with make() as r:
                t0 = time.perf_counter()
                img = r.reconstruct(rays)
                dt = time.perf_counter() - t0
                st = r.status()
            best = dt if best is None or dt < best else best
        return best, img, st

    def cpu_call(f):
        t0 = time.perf_counter()
        v = f()
        return time.perf_counter() - t0, v

    cfg = wl.poca_config(cut_percentile=0.5)
    g_s, img, _ = gpu_call(lambda: M.MutoPoCut(cfg))
    c_s, (ref, _, _) = cpu_call(lambda: O.pocut(wl.grid, cfg, rays))
    out["pocut_cut_0.5"] = {"gpu_s": g_s, "cpu_s": c_s, "tracks_per_s": n / g_s,
                            "rel_l2_vs_oracle": rel_l2(img.reshape(-1, order="F"), ref)}
    cfg = wl.poca_config(length_weighted=True)
    g_s, img, _ = gpu_call(lambda: M.MutoSLR(cfg))
    c_s, ref = cpu_call(lambda: O.slr(wl.grid, cfg, rays))
    out["slr"] = {"gpu_s": g_s, "cpu_s": c_s, "tracks_per_s": n / g_s,
                  "rel_l2_vs_oracle": rel_l2(img.reshape(-1, order="F"), ref)}
    for sch in ("levels", "sequential"):
        cfg = dict(wl.poca_config(length_weighted=True), num_iteration=4, slr_iter_schedule=sch)
        g_s, img, st = gpu_call(lambda: M.MutoSLRIter(cfg))
        row = {"gpu_s": g_s, "levels": st["slr_levels"]}
        if sch == "levels":
            c_s, ref = cpu_call(lambda: O.slr(wl.grid, cfg, rays, iterative=True))
            row.update(cpu_s=c_s, rel_l2_vs_oracle=rel_l2(img.reshape(-1, order="F"), ref))
        out[f"slr_iter_4_passes_{sch}"] = row
    # detector records of the same tracks: 3 + 3 planes 500 mm apart around the
    # grid, hits on the fitted lines (input/example_mlsd.json:3-4 spacing)
    zt, zb = wl.grid.z_min + wl.grid.nz * wl.grid.dz, wl.grid.z_min
    z = np.array([zt + 1000.0, zt + 500.0, zt, zb, zb - 500.0, zb - 1000.0])
    rec = np.empty((n, 14))
    rec[:, 0], rec[:, -1] = rays[:, 0], rays[:, 1]
    for k, zk in enumerate(z):
        p, d = (rays[:, 2:5], rays[:, 8:11]) if k < 3 else (rays[:, 5:8], rays[:, 11:14])
        t = (zk - p[:, 2]) / d[:, 2]
        rec[:, 1 + 2 * k] = p[:, 0] + t * d[:, 0]
        rec[:, 2 + 2 * k] = p[:, 1] + t * d[:, 1]
    best = None
    for _ in range(3):
        t0 = time.perf_counter()
        fit = M.fit_tracks(rec, z, 3)
        dt = time.perf_counter() - t0
        best = dt if best is None or dt < best else best
    c_s, ref = cpu_call(lambda: O.fit_records(rec, z, 3))
    out["line_fit"] = {"gpu_s": best, "cpu_s": c_s, "records_per_s": n / best,
                       "max_abs_diff_vs_oracle": float(np.nanmax(np.abs(fit - ref))) if len(fit) == len(ref) else None}
    return out


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def cpu_port(wl, args, rays: np.ndarray, n_iter: int, threads: int) -> dict:
    """Time the CPU restatement of the reference path on a sample of the workload's tracks."""
    os.environ["OMP_NUM_THREADS"] = str(threads)
    from oracle import oracle as O

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
    return {"pairs": pairs, "times": times, "setup_s": t_setup, "n_sample": rays.shape[0]}


def reference_sample(steps: int, warmup: int, cap: int) -> int:
    """Muons of the reference leg's sample: about 150 s of EM iterations at the
    port's ~1.5e7 pairs/s with ~100 pairs per sampled muon, at most `cap`."""
    per_step_s = 150.0 / max(steps + warmup, 1)
    return int(min(cap, max(20_000, per_step_s * 1.5e7 / 100.0)))


def run_reference(args) -> int:
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    from oracle import synthetic as S

    wl = workload(args, 0)
    threads = host_cores()
    n_sample = args.cpu_sample if args.cpu_sample_fixed else reference_sample(args.steps, args.warmup, args.cpu_sample)
    t0 = time.perf_counter()
    rays = S.generate(wl.grid, wl_lambda(wl), n_sample, wl.seed)  # the first n_sample muons of the workload's stream
    t_gen = time.perf_counter() - t0
    r = cpu_port(wl, args, rays, args.warmup + args.steps, threads)
    t = r["times"][args.warmup:]
    value = r["pairs"] * len(t) / sum(t)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000 * sum(t) / len(t), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": wl.name, "method": method_of(args), "grid": list(wl.grid.shape), "mode": args.mode,
                   "muons": wl.n_muons, "sample_muons": n_sample, "sample_pairs": r["pairs"]},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"the first {n_sample} of the {wl.n_muons} muons of {wl.name} "
                                   f"({r['pairs']} pairs per EM iteration): one EM iteration per step; "
                                   f"set-up {r['setup_s']:.1f} s and track generation {t_gen:.1f} s untimed"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def algorithmic_bytes(kernel: str, rb: int, P: int, N: int, V: int) -> int:
    """Bytes a kernel must move per launch (rb: bytes of the storage precision)."""
    lists = (4 + 2 * rb) * P  # voxel index, L, T of every pair, read once
    return {
        "em_muon": lists + (8 + 9 * rb) * N + rb * V,      # + offsets, (S, D), pr^2, k out; lambda gathered
        "em_scatter": lists + (8 + 4 * rb) * N + rb * V,   # + offsets, k in; G reduced
        "em_fused": lists + (8 + 5 * rb) * N + 2 * rb * V,  # + offsets, (S, D), pr^2; lambda in, G reduced
        "em_voxel": lists + (16 + 6 * rb) * V,             # voxel-major lists; descriptor, lambda, window
        "em_update": (4 + 4 * rb) * V,                     # lambda, M, G in, G cleared, lambda out
    }.get(kernel, 0)


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
    del lam
    sp = C.c_void_p()

    def stream_of(rec):
        lib.muto_get_stream(rec._h, C.byref(sp))
        return torch.cuda.ExternalStream(sp.value)

    def setup_stats(rec) -> dict:
        out = {}
        for name in SETUP_KERNELS + ["host:" + p for p in SETUP_PHASES]:
            cnt, tot = rec.kernel_stats(name)
            if cnt:
                out[name] = round(tot, 3)
        return out

    # ---- value: EM iterations with the tracks resident in HBM ---------------
    cfg = em_config(wl, args, args.precision, args.warmup + args.steps)
    rec = M.Reconstruction(method_of(args), cfg)
    rec.load_tracks(None, on_device_ptr=d_rays.data_ptr(), n=n)
    rec.set_profiling(True)
    t0 = time.perf_counter()
    rec.prepare()
    t_setup = time.perf_counter() - t0
    setup_ms = setup_stats(rec)
    st = rec.status()
    pairs, kept, V = st["n_pairs"], st["n_scat_in_grid"], wl.grid.nvox
    stream = stream_of(rec)
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
    kern = {}
    for k in ITER_KERNELS:
        c, t = rec.kernel_stats(k)
        if c:
            kern[k] = t / args.steps  # ms per iteration (all launches of that name in one iteration)
    rec.set_profiling(False)
    rec.close()

    # ---- rooflines: every iteration kernel by its algorithmic bytes ----------
    rb = 4 if args.precision == "mixed" else 8
    pk = peaks()
    fam = "grid256" if args.workload.startswith("grid256") else "cube"
    per_kernel = {}
    for k, kms in kern.items():
        b = algorithmic_bytes(k, rb, pairs, kept, V)
        if not b:
            continue
        ach = b / (kms / 1000.0) / 1e9
        tpp = TRAFFIC_PER_PAIR.get((fam, k)) if args.precision == "mixed" else None
        per_kernel[k] = {"kernel_ms": kms, "algorithmic_bytes": b, "achieved": ach, "frac": ach / pk["hbm_gbs"],
                         "traffic": tpp * pairs if tpp else None}
    dom = max(per_kernel, key=lambda k: per_kernel[k]["kernel_ms"]) if per_kernel else None
    # one iteration's algorithmic bytes: the lists once, per-muon inputs and cost, lambda in, G, lambda out
    b_iter = (4 + 2 * rb) * pairs + 24 * kept + 12 * V
    roofline = {"bound": "hbm", "peak": pk["hbm_gbs"], "unit": "GB/s", "peak_source": pk["source"]}
    if dom:
        d = per_kernel[dom]
        roofline.update(kernel=dom, achieved=d["achieved"], frac=d["frac"], traffic=d["traffic"],
                        kernel_ms=d["kernel_ms"], algorithmic_bytes=d["algorithmic_bytes"])
    roofline["kernels"] = per_kernel
    if st["muon_pass"] == 5 and st["tile_muons"]:
        roofline["kernels_note"] = ("each kernel timed alone in profiled iterations; the timed iterations run the "
                                    f"scatter of one of {st['tile_muons']} chunks of muons beside the muon pass of the "
                                    "next, so the kernel times add up to more than ms_per_step")
    roofline["iteration"] = {"algorithmic_bytes": b_iter, "ms": ms / args.steps,
                             "achieved": b_iter / (ms / args.steps / 1000.0) / 1e9,
                             "frac": b_iter / (ms / args.steps / 1000.0) / 1e9 / pk["hbm_gbs"],
                             "what": f"{4 + 2 * rb} B per pair (index, L, T) + 24 B per kept muon + 12 B per voxel"}

    # ---- e2e: full reconstruct through the C ABI from pinned host tracks ------
    e2e = None
    if args.e2e_steps > 0:
        hst = torch.empty((n, 14), dtype=torch.float64, pin_memory=True)
        hst.copy_(d_rays)
        e_iters = args.e2e_iters if args.e2e_iters > 0 else wl.n_iter  # the workload's reconstruct call
        ecfg = em_config(wl, args, args.precision, e_iters)
        out = np.empty(V, np.float64)
        times = []
        for k in range(args.e2e_steps + 1):  # the first call is a warm-up
            r2 = M.Reconstruction(method_of(args), ecfg)
            s2 = stream_of(r2)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            barrier()
            torch.cuda.synchronize()
            a.record(s2)
            rc = lib.muto_reconstruct(r2._h, C.c_void_p(hst.data_ptr()), n, _lib.dptr(out), V)
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
        r2.load_tracks(hst.numpy())
        setup_warm = {"load_tracks_h2d": round((time.perf_counter() - t0) * 1e3, 3)}
        t0 = time.perf_counter()
        r2.prepare()
        setup_warm["prepare"] = round((time.perf_counter() - t0) * 1e3, 3)
        setup_warm.update(setup_stats(r2))
        r2.close()
        del hst
        e_ms = allmax(statistics.mean(times))
        e2e = {"value": total_pairs * e_iters / (e_ms / 1000.0), "unit": UNIT,
               "h2d_bytes_per_step": int(n * 14 * 8), "d2h_bytes_per_step": int(V * 8),
               "ms_per_step": e_ms, "em_iterations_per_step": e_iters, "setup_ms": setup_warm,
               "what": "muto_reconstruct: H2D of pinned tracks, setup (gather, Siddon lists), "
                       f"{e_iters} EM iterations (the workload's num_iteration), D2H of the image"}

    # ---- stored lists against paths recomputed every iteration ----------------
    recompute = None
    if args.recompute_iters > 0 and args.mode == "mean" and rank == 0:
        r4 = M.Reconstruction(method_of(args), em_config(wl, args, args.precision, 1 + args.recompute_iters,
                                                         lists="recompute"))
        r4.load_tracks(None, on_device_ptr=d_rays.data_ptr(), n=n)
        t0 = time.perf_counter()
        r4.prepare()
        r_setup = time.perf_counter() - t0
        s4 = stream_of(r4)
        r4.iterate(1)  # graph capture and a first pass
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(s4)
        for _ in range(args.recompute_iters):
            r4.iterate(1)
        b.record(s4)
        b.synchronize()
        r_ms = a.elapsed_time(b) / args.recompute_iters
        r4st = r4.status()
        r4.close()
        recompute = {"ms_per_iteration": r_ms, "value": r4st["n_pairs"] / (r_ms / 1000.0), "unit": UNIT,
                     "setup_s": r_setup, "iterations_timed": args.recompute_iters,
                     "device_bytes": r4st["device_bytes"], "stored_ms_per_iteration": ms / args.steps,
                     "stored_device_bytes": st["device_bytes"],
                     "recompute_over_stored_time": r_ms / (ms / args.steps),
                     "what": "no stored lists: every path walked in FP64 twice per iteration (sum, scatter)"}

    # ---- PoCA on the same tracks (src/MutoPoCA.cpp:51-134) --------------------
    poca = None
    if args.poca and rank == 0:
        pcfg = wl.poca_config()
        times = []
        for k in range(3):  # one warm-up
            r5 = M.Reconstruction("poca", pcfg)
            r5.load_tracks(None, on_device_ptr=d_rays.data_ptr(), n=n)
            r5.set_profiling(True)
            torch.cuda.synchronize()
            r5.prepare()
            c1, t1 = r5.kernel_stats("poca")
            c2, t2 = r5.kernel_stats("poca_normalize")
            pst = r5.status()
            r5.close()
            if k > 0:
                times.append((t1, t2))
        t_poca = statistics.mean(t for t, _ in times)
        t_norm = statistics.mean(t for _, t in times)
        pb = n * 112 + 2 * 8 * V  # every track read once; image and weight sums
        poca = {"rays_per_s": n / ((t_poca + t_norm) / 1000.0), "kernel_ms": t_poca, "normalize_ms": t_norm,
                "algorithmic_bytes": pb, "achieved": pb / (t_poca / 1000.0) / 1e9,
                "frac": pb / (t_poca / 1000.0) / 1e9 / pk["hbm_gbs"], "peak": pk["hbm_gbs"],
                "in_grid": pst["n_scat_in_grid"],
                "bound": "the FP64 pipe, not HBM: the frac above is by bytes only (ncu: "
                         "profiles/poca_walk_grid256x256x128_10mm_2M.md)",
                "what": "k_poca: FP64 closest approach, binning and the length-weighted Siddon weights of every "
                        "track (FP64 atomics, a thread per kept track), then the normalisation"}

    # ---- the rows either side of the path: PoCut, SLR, SLRIter, the line fit ----
    next_rows = None
    if args.next_rows > 0 and rank == 0:
        next_rows = run_next_rows(wl, d_rays[:min(args.next_rows, n)].cpu().numpy())

    # ---- time to lambda: mixed vs the plain FP64 form, same iteration count ---
    ttl = None
    if args.ttl_iters > 0 and rank == 0:
        res = {}
        for prec in ("fp64", "mixed"):
            r3 = M.Reconstruction(method_of(args), em_config(wl, args, prec, args.ttl_iters))
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r3.load_tracks(None, on_device_ptr=d_rays.data_ptr(), n=n)
            r3.prepare()
            r3.iterate(args.ttl_iters)
            im = r3.image()
            res[prec] = (time.perf_counter() - t0, im, r3.status()["device_bytes"])
            r3.close()
        a64, b32 = res["fp64"][1].ravel(), res["mixed"][1].ravel()
        rel = float(np.linalg.norm(b32 - a64) / np.linalg.norm(a64))
        ttl = {"iterations": args.ttl_iters, "fp64_s": res["fp64"][0], "mixed_s": res["mixed"][0],
               "rel_l2_mixed_vs_fp64": rel, "speedup": res["fp64"][0] / res["mixed"][0],
               "within_1e-4": rel < 1e-4, "fp64_device_bytes": res["fp64"][2],
               "what": "set-up and iterations from device-resident tracks, wall clock; the FP64 GPU form stands "
                       "in for the FP64 oracle at this size"}
        if method_of(args) == "map":
            ttl.update(map_conditioning(wl, args, d_rays, n, res["fp64"][1], res["mixed"][1]))
    # ---- the gradient MAP solver against the MAP EM, to the same objective ---
    grad_vs_em = None
    if method_of(args) == "map" and args.grad_vs_em > 0 and rank == 0:
        K = args.grad_vs_em
        delta = 0.1 * float(np.median(wl_lambda(wl))) * 1e7
        grad_vs_em = []
        for beta in (1e-3, 1e-2):
            for p in (2.0, 1.0):
                gcfg = em_config(wl, args, args.precision, K)
                gcfg.update(update_with_mean=True, mean_percentile=100, beta=beta, p=p, all_neighbours=True,
                            delta=delta)
                ra = M.Reconstruction("map", gcfg)
                ra.load_tracks(None, on_device_ptr=d_rays.data_ptr(), n=n)
                ra.prepare()
                sa = stream_of(ra)
                a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                torch.cuda.synchronize()
                a.record(sa)
                ra.iterate(K)
                z.record(sa)
                z.synchronize()
                mult = ra.multiplicity()
                img = ra.image().reshape(-1, order="F")
                f_em = ra.nll(np.log(np.where(mult > 0, np.maximum(img, 1e-300), 1.0)))
                ra.close()
                rg = M.Reconstruction("map", dict(gcfg, num_iteration=0))
                rg.load_tracks(None, on_device_ptr=d_rays.data_ptr(), n=n)
                rg.prepare()
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                f_g, it = rg.gradient_solve_until(f_em, 200)
                t_g = time.perf_counter() - t0
                rg.close()
                grad_vs_em.append({"beta": beta, "p": p, "em_iterations": K, "em_s": a.elapsed_time(z) / 1000.0,
                                   "F_em": f_em, "gradient_iterations": it, "gradient_s": t_g, "F_gradient": f_g,
                                   "reached": bool(f_g <= f_em)})

    # ---- CPU baseline on this machine's host cores (rank 0 only) ----------------
    cpu = None
    if rank == 0 and args.cpu_sample > 0:
        threads = host_cores()
        ns = min(args.cpu_sample, n)
        sample = d_rays[:ns].cpu().numpy()  # the first muons of the workload's stream
        r = cpu_port(wl, args, sample, 2, threads)
        cval = r["pairs"] * len(r["times"]) / sum(r["times"])
        cpu = {"value": cval, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"the first {ns} of the {n} muons of the same workload, 2 EM iterations "
                         f"({r['pairs']} pairs each), set-up untimed"}
    del d_rays

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
                       "path_lists": {1: "voxel_major", 2: "muon_major", 3: "recompute"}.get(st["path_lists"]),
                       "parallelism": f"replicas x{world} (one scan per GPU)",
                       "l2": "inputs larger than L2: the pair lists read every iteration far exceed 126 MB, no flush",
                       "device_bytes": st["device_bytes"], "setup_s": t_setup, "setup_ms": setup_ms,
                       "generate_s": t_gen,
                       "muon_pass": {1: "tma_tiles", 2: "warp_batched", 3: "one_pass_lists", 4: "recompute_walk",
                                     5: "split_muon_pass_and_scatter",
                                     6: "one_pass_staged_in_shared_memory"}.get(st["muon_pass"]),
                       "muon_group": st["muon_group"], "tile_pairs": st["tile_pairs"],
                       "overlap_chunks": st["tile_muons"] if st["muon_pass"] == 5 else 0},
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": int(launches),
            "clocks": clk,
            "time_to_lambda": ttl,
            "recompute": recompute,
            "poca": poca,
            "next_rows": next_rows,
        }
        if grad_vs_em is not None:
            line["gradient_vs_em"] = {"runs": grad_vs_em, "what": (
                "F = NLL + MAP prior (26 neighbours, delta 0.1 median lambda); the MAP EM with the mean ML step "
                "(a scaled gradient step) for em_iterations, graph-captured, timed on the device; then the "
                "gradient solver (preconditioned descent in log lambda with backtracking) from the same start "
                "until F <= F_em, wall clock, its F and gradient from the same passes")}
        print(json.dumps(line), flush=True)
    rep.close()
    return 0


def run_batch(args) -> int:
    """The 64-scan batch: every pass of an EM iteration is one launch over all scans."""
    import torch

    from muontomography_gb300.replicas import Replicas, replica_seed

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    rep = Replicas("nccl")
    import muontomography_gb300 as M
    from muontomography_gb300 import _lib
    from muontomography_gb300 import workloads as W

    lib = M.library()
    wls = W.batch64(scale=args.batch_scale, seed=replica_seed(4, rank))
    grids = [w.grid for w in wls]
    t0 = time.perf_counter()
    tracks = []
    for w in wls:
        lam = torch.tensor(w.lam(), dtype=torch.float64, device="cuda")
        d = torch.empty((w.n_muons, 14), dtype=torch.float64, device="cuda")
        prm = _lib.muto_gen_params(w.seed, np.pi / 3, 1.0, 10.0, 3.0, 500.0, 3, 0, 1.0)
        g = w.grid.c()
        _lib.check(lib.muto_generate_device(C.byref(g), C.c_void_p(lam.data_ptr()), C.byref(prm), 0, w.n_muons,
                                            C.c_void_p(d.data_ptr()),
                                            C.c_void_p(torch.cuda.current_stream().cuda_stream)), "generate")
        tracks.append(d)
    torch.cuda.synchronize()
    t_gen = time.perf_counter() - t0
    n_all = sum(w.n_muons for w in wls)
    sp = C.c_void_p()

    def batch_cfg(precision, n_iter):
        cfg = em_config(wls[0], args, precision, n_iter)
        cfg.pop("grid")
        cfg.update(initialize_method=2, voxel_stream_above="auto")
        return cfg

    def loaded(precision, n_iter):
        b = M.Batch(batch_cfg(precision, n_iter), grids)
        for k, d in enumerate(tracks):
            b.load_scan(k, on_device_ptr=d.data_ptr(), n=d.shape[0])
        return b

    b = loaded(args.precision, args.warmup + args.steps)
    b.set_profiling(True)
    t0 = time.perf_counter()
    b.prepare()
    t_setup = time.perf_counter() - t0
    st = b.status()
    pairs, kept, V = st["n_pairs"], st["n_scat_in_grid"], sum(g.nvox for g in grids)
    lib.muto_get_stream(b._h, C.byref(sp))
    stream = torch.cuda.ExternalStream(sp.value)
    for _ in range(args.warmup):
        b.iterate(1)
    b.reset_kernel_stats()
    l0 = b.launch_count()
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    rep.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        b.iterate(1)
    e1.record(stream)
    e1.synchronize()
    rep.barrier()
    ms = rep.max(e0.elapsed_time(e1))
    clk = clocks.stop()
    launches = b.launch_count() - l0
    value = rep.sum(float(pairs)) * args.steps / (ms / 1000.0)
    kern = {}
    for k in ITER_KERNELS:
        c, t = b.kernel_stats(k)
        if c:
            kern[k] = t / args.steps
    b.set_profiling(False)
    img_mixed = [b.scan_image(k) for k in range(len(wls))] if args.precision == "mixed" else None
    b.close()

    rb = 4 if args.precision == "mixed" else 8
    pk = peaks()
    per_kernel = {}
    for k, kms in kern.items():
        nb = algorithmic_bytes(k, rb, pairs, kept, V)
        if nb:
            ach = nb / (kms / 1000.0) / 1e9
            per_kernel[k] = {"kernel_ms": kms, "algorithmic_bytes": nb, "achieved": ach, "frac": ach / pk["hbm_gbs"],
                             "traffic": None}
    dom = max(per_kernel, key=lambda k: per_kernel[k]["kernel_ms"]) if per_kernel else None
    roofline = {"bound": "hbm", "peak": pk["hbm_gbs"], "unit": "GB/s", "peak_source": pk["source"],
                "kernels": per_kernel}
    if dom:
        d = per_kernel[dom]
        roofline.update(kernel=dom, achieved=d["achieved"], frac=d["frac"], traffic=None, kernel_ms=d["kernel_ms"],
                        algorithmic_bytes=d["algorithmic_bytes"])

    # per-scan lambda of the mixed form against the plain FP64 form after the same iterations
    errors = None
    if img_mixed is not None and args.ttl_iters > 0:
        b64 = loaded("fp64", args.warmup + args.steps)
        t0 = time.perf_counter()
        b64.prepare()
        b64.iterate(args.warmup + args.steps)
        ref = [b64.scan_image(k) for k in range(len(wls))]
        t64 = time.perf_counter() - t0
        b64.close()
        rel = [float(np.linalg.norm(a.ravel() - r.ravel()) / max(np.linalg.norm(r.ravel()), 1e-300))
               for a, r in zip(img_mixed, ref)]
        errors = {"iterations": args.warmup + args.steps, "max_rel_l2": max(rel), "median_rel_l2": statistics.median(rel),
                  "all_within_1e-4": max(rel) < 1e-4, "per_scan_rel_l2": [round(x, 10) for x in rel],
                  "fp64_form_s": t64, "what": "per scan, the mixed form's lambda against the plain FP64 GPU form "
                                             "after the same iterations (set-up and iterations of the FP64 form timed)"}

    # e2e: load every scan from pinned host memory, set up, iterate, read every image
    e2e = None
    if args.e2e_steps > 0:
        hosts = []
        for d in tracks:
            h = torch.empty(tuple(d.shape), dtype=torch.float64, pin_memory=True)
            h.copy_(d)
            hosts.append(h)
        e_iters = args.e2e_iters if args.e2e_iters > 0 else wls[0].n_iter
        times = []
        for rnd in range(args.e2e_steps + 1):  # the first round is a warm-up
            bb = M.Batch(batch_cfg(args.precision, e_iters), grids)
            lib.muto_get_stream(bb._h, C.byref(sp))
            s2 = torch.cuda.ExternalStream(sp.value)
            a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            a.record(s2)
            for k, h in enumerate(hosts):
                _lib.check(lib.muto_batch_load_tracks(bb._h, k, C.c_void_p(h.data_ptr()), h.shape[0], 0), "load")
            bb.prepare()
            bb.iterate(e_iters)
            out = [bb.scan_image(k) for k in range(len(wls))]
            z.record(s2)
            z.synchronize()
            if rnd > 0:
                times.append(a.elapsed_time(z))
            bb.close()
        e_ms = rep.max(statistics.mean(times))
        e2e = {"value": rep.sum(float(pairs)) * e_iters / (e_ms / 1000.0), "unit": UNIT,
               "h2d_bytes_per_step": int(n_all * 14 * 8), "d2h_bytes_per_step": int(V * 8), "ms_per_step": e_ms,
               "em_iterations_per_step": e_iters,
               "what": f"64 scans: H2D of pinned tracks, set-up, {e_iters} EM iterations, D2H of every image"}
        del hosts, out

    cpu = None
    if rank == 0 and args.cpu_sample > 0:
        ns = min(args.cpu_sample, tracks[0].shape[0])
        sample = tracks[0][:ns].cpu().numpy()
        r = cpu_port(wls[0], args, sample, 2, host_cores())
        cval = r["pairs"] * len(r["times"]) / sum(r["times"])
        cpu = {"value": cval, "unit": UNIT, "cores": host_cores(), "kind": "port",
               "sample": f"the first {ns} muons of scan 0 ({wls[0].grid.nx}^3 voxels), 2 EM iterations "
                         f"({r['pairs']} pairs each), set-up untimed"}
    del tracks
    if rank == 0:
        sides = [g.nx for g in grids]
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32" if args.precision == "mixed" else "f64", "data": "synthetic",
            "config": {"workload": "batch64", "scans": len(wls), "muons": n_all, "kept_muons": kept,
                       "pairs_per_iteration": pairs, "voxels": V, "mode": args.mode, "precision": args.precision,
                       "grids": {str(n): sides.count(n) for n in (32, 64, 96, 128)},
                       "muons_per_scan": [min(w.n_muons for w in wls), max(w.n_muons for w in wls)],
                       "graph": True, "one_launch_per_pass": True, "setup_s": t_setup, "generate_s": t_gen,
                       "device_bytes": st["device_bytes"],
                       "path_lists": {1: "voxel_major", 2: "muon_major", 3: "recompute"}.get(st["path_lists"]),
                       "autotuner": {"pass": {1: "tma_tiles", 2: "warp_batched", 3: "one_pass_lists",
                                              5: "split_muon_pass_and_scatter",
                                              6: "one_pass_staged_in_shared_memory"}.get(st["muon_pass"]),
                                     "lanes_per_muon": st["muon_group"], "tile_pairs": st["tile_pairs"],
                                     "voxel_stream_above": st["voxel_stream_above"]},
                       "parallelism": f"replicas x{world} (one batch per GPU)",
                       "l2": "inputs larger than L2: the batch's pair lists far exceed 126 MB, no flush"},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches), "clocks": clk,
            "lambda_errors": errors,
        }
        print(json.dumps(line), flush=True)
    rep.close()
    return 0


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="grid256x256x128_10mm", choices=list(WORKLOADS))
    ap.add_argument("--n-muons", type=int, default=0)
    ap.add_argument("--mode", choices=["median", "mean"], default=None,
                    help="EM update (default: mean for the 256x256x128 scan, median otherwise)")
    ap.add_argument("--lists", choices=["auto", "voxel_major", "muon_major", "recompute"], default="auto")
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--e2e-iters", type=int, default=0, help="EM iterations per e2e call (0: the workload's)")
    ap.add_argument("--ttl-iters", type=int, default=-1,
                    help="iterations of the time-to-lambda runs (-1: the workload's)")
    ap.add_argument("--recompute-iters", type=int, default=2)
    ap.add_argument("--poca", type=int, default=1)
    ap.add_argument("--next-rows", type=int, default=0,
                    help="time PoCut, SLR, SLRIter and the line fit on the first N tracks (0: off)")
    ap.add_argument("--cpu-sample", type=int, default=1_000_000)
    ap.add_argument("--batch-scale", type=float, default=1.0, help="batch64: muons per scan times this")
    ap.add_argument("--grad-vs-em", type=int, default=20,
                    help="MAP workload: EM iterations the gradient solver is run to match (0: skip)")
    ap.add_argument("--cpu-sample-fixed", action="store_true",
                    help="reference leg: use --cpu-sample as it is instead of sizing it to the step count")
    ap.add_argument("--muon-pass", choices=["auto", "tile", "warp"], default="auto")
    ap.add_argument("--fused-variant", choices=["auto", "4x8", "8x4", "8x8", "8x16", "16x8", "16x16", "staged", "split", "split8",
                             "split8_overlap"],
                    default="auto", help="the mean update's pass over muon-major lists (auto: timed at set-up)")
    ap.add_argument("--muon-layout", choices=["auto", "columns", "index"], default="auto")
    ap.add_argument("--voxel-stream-above", type=int, default=None,
                    help="segments longer than this are selected without holding their keys (-1: never)")
    args = ap.parse_args()
    if args.mode is None:
        args.mode = DEFAULT_MODE.get(args.workload, "median")
    if args.ttl_iters < 0:
        from muontomography_gb300 import workloads as W

        args.ttl_iters = 20 if args.workload == "batch64" else WORKLOADS[args.workload](W)().n_iter
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_batch(args) if args.workload == "batch64" else run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
