"""Seeded synthetic workloads with the shapes of the benchmark configurations.

The reference measures on detector data that is not available here; each
workload below stands in for it with muons from ``generate`` (cos^2 zenith
below 60 degrees, log-uniform 1-10 GeV/c, entry uniform on the grid top,
per-voxel Gaussian scattering, 1 mm hit smearing) through a block phantom
whose lambda follows the Highland-type scaling (13.6 MeV / p0)^2 / X0.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import X0_MM, Block, Grid, generate, phantom


@dataclass
class Workload:
    name: str
    grid: Grid
    blocks: list[Block]
    n_muons: int
    seed: int
    has_energy: bool
    n_iter: int
    extra: dict = field(default_factory=dict)

    def lam(self) -> np.ndarray:
        return phantom(self.grid, self.blocks, X0_MM["air"], 3.0)

    def tracks(self, n: int | None = None, first: int = 0) -> np.ndarray:
        return generate(self.grid, self.lam(), self.n_muons if n is None else n, self.seed, first=first)

    def em_config(self, **over) -> dict:
        cfg = {"grid": self.grid.json(), "has_energy": self.has_energy, "num_iteration": self.n_iter,
               "initialize_method": 2, "initialize_value": 1.0e-7, "update_with_mean": False,
               "mean_percentile": 100, "straight_line": False, "early_stop": False, "eps": 1.0e-8}
        cfg.update(over)
        return cfg

    def poca_config(self, **over) -> dict:
        cfg = {"grid": self.grid.json(), "length_weighted": True, "straight_line": False,
               "has_energy": False, "angle_unit_mag": 1.0, "eps": 1.0e-8}
        cfg.update(over)
        return cfg


def _random_blocks(rng, grid: Grid, materials, edge_lo, edge_hi, margin=0.1):
    lo = np.array([grid.x_min, grid.y_min, grid.z_min])
    ext = np.array([grid.nx * grid.dx, grid.ny * grid.dy, grid.nz * grid.dz])
    out = []
    for m in materials:
        e = rng.uniform(edge_lo, edge_hi, size=3)
        c = lo + ext * margin + e / 2 + rng.uniform(0, 1, size=3) * np.maximum(ext * (1 - 2 * margin) - e, 0)
        out.append(Block(tuple(c - e / 2), tuple(c + e / 2), X0_MM[m]))
    return out


def cube20_50mm(n_muons: int = 100_000, seed: int = 1) -> Workload:
    """20^3 voxels of 50 mm (1 m cube), iron 200 mm cube at the centre, lead 100 mm cube 250 mm along x."""
    g = Grid(20, 20, 20, -500.0, -500.0, -500.0, 50.0, 50.0, 50.0)
    blocks = [Block((-100.0, -100.0, -100.0), (100.0, 100.0, 100.0), X0_MM["iron"]),
              Block((200.0, -50.0, -50.0), (300.0, 50.0, 50.0), X0_MM["lead"])]
    return Workload("cube20_50mm_100k", g, blocks, n_muons, seed, False, 20)


def cube100_20mm(n_muons: int = 10_000_000, seed: int = 2) -> Workload:
    """100^3 voxels of 20 mm (2 m cube): iron, lead, aluminium blocks (150-300 mm) and a 50 mm concrete slab."""
    g = Grid(100, 100, 100, -1000.0, -1000.0, -1000.0, 20.0, 20.0, 20.0)
    rng = np.random.default_rng(seed)
    blocks = _random_blocks(rng, g, ["iron", "lead", "aluminium"], 150.0, 300.0)
    z0 = float(rng.uniform(-800.0, -500.0))
    blocks.insert(0, Block((-800.0, -800.0, z0), (800.0, 800.0, z0 + 50.0), X0_MM["concrete"]))
    return Workload("cube100_20mm_10M", g, blocks, n_muons, seed, True, 50)


def cube50_40mm(n_muons: int = 2_500_000, seed: int = 2) -> Workload:
    """cube100_20mm's scene on 50^3 voxels of 40 mm with a quarter of the muons: the same
    pairs per voxel (about 550) in a quarter of the memory, for profiler captures."""
    full = cube100_20mm(seed=seed)
    g = Grid(50, 50, 50, -1000.0, -1000.0, -1000.0, 40.0, 40.0, 40.0)
    return Workload("cube50_40mm_2.5M", g, full.blocks, n_muons, seed, True, 50)


def map128x128x64_15mm(n_muons: int = 20_000_000, seed: int = 3) -> Workload:
    """128x128x64 voxels of 15 mm, MAP with the 26-neighbour prior."""
    g = Grid(128, 128, 64, -960.0, -960.0, -480.0, 15.0, 15.0, 15.0)
    rng = np.random.default_rng(seed)
    blocks = _random_blocks(rng, g, ["iron", "lead", "aluminium", "concrete"], 100.0, 300.0)
    return Workload("map128x128x64_15mm_20M", g, blocks, n_muons, seed, True, 20)


def grid256x256x128_10mm(n_muons: int = 100_000_000, seed: int = 5) -> Workload:
    """256x256x128 voxels of 10 mm, 12 mixed blocks."""
    g = Grid(256, 256, 128, -1280.0, -1280.0, -640.0, 10.0, 10.0, 10.0)
    rng = np.random.default_rng(seed)
    mats = ["iron", "lead", "aluminium", "concrete"] * 3
    blocks = _random_blocks(rng, g, mats, 100.0, 400.0)
    return Workload("grid256x256x128_10mm_100M", g, blocks, n_muons, seed, True, 30)


def small(n_muons: int = 4000, seed: int = 11, n: int = 12) -> Workload:
    """A few-thousand-muon case for quick parity tests."""
    g = Grid(n, n, n, -300.0, -300.0, -300.0, 600.0 / n, 600.0 / n, 600.0 / n)
    blocks = [Block((-100.0, -100.0, -100.0), (100.0, 100.0, 100.0), X0_MM["iron"]),
              Block((120.0, -60.0, -60.0), (240.0, 60.0, 60.0), X0_MM["lead"])]
    return Workload(f"small_{n}cube_{n_muons}", g, blocks, n_muons, seed, True, 5)


def batch64(scale: float = 1.0, seed: int = 4) -> list[Workload]:
    """64 independent scans of uneven sizes: cubic grids of 32, 64, 96 or 128
    voxels a side at 20 mm, muon counts log-uniform between 50 k and 5 M (times
    `scale`), each scan with its own seeded random phantom of three blocks of
    iron, lead, aluminium or concrete."""
    rng = np.random.default_rng(seed)
    sides = rng.choice([32, 64, 96, 128], size=64)
    muons = np.exp(rng.uniform(np.log(50_000), np.log(5_000_000), size=64))
    mats = ["iron", "lead", "aluminium", "concrete"]
    out = []
    for k, (nside, nm) in enumerate(zip(sides, muons)):
        half = float(nside) * 20.0 / 2
        g = Grid(int(nside), int(nside), int(nside), -half, -half, -half, 20.0, 20.0, 20.0)
        ext = float(nside) * 20.0
        blocks = _random_blocks(rng, g, list(rng.choice(mats, size=3)), 0.1 * ext, 0.3 * ext)
        out.append(Workload(f"batch64_scan{k:02d}", g, blocks, max(1000, int(nm * scale)), 400 + k, True, 20))
    return out
