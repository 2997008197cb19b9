"""Batched sweep of many independent cores (moc_batch_* in the C ABI).

`batched_specs` draws the batched workload: independent small cores of uneven
sizes, each with its own seeded cross sections as in the small problem.
`Batch` sweeps their tracks in one persistent launch and replays their power
iteration as a CUDA graph.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .problem import ProblemSpec, pins
from .solver import Solver


def batched_specs(n_cores: int = 64, seed: int = 20260103, z_stacked: int = 24,
                  height: float = 200.0) -> list[ProblemSpec]:
    """Cores of 1x1 to 4x4 assemblies of 17x17 pins (4 coarse x 5 fine axial
    regions per pin), 8 to 32 azimuthal angles (even) x 32 tracks per assembly
    width, 2 to 6 polar angles (even), 20 to 100 groups, 20 to 80 segments per
    track; core c is seeded seed + c."""
    rng = np.random.default_rng(seed)
    specs = []
    for c in range(n_cores):
        ax, ay = (int(v) for v in rng.integers(1, 5, size=2))
        n_az = 2 * int(rng.integers(4, 17))
        n_polar = 2 * int(rng.integers(1, 4))
        groups = int(rng.integers(20, 101))
        segs = int(rng.integers(20, 81))
        specs.append(ProblemSpec(
            n_groups=groups, fai=5, cai=4, height=height, n_sources=pins(ax, ay) * 4,
            n_tracks_2d=n_az * 32 * max(ax, ay), n_polar=n_polar, z_stacked=z_stacked,
            n_seg=segs, seed=seed + c))
    return specs


class Batch:
    """One persistent sweep launch over the tracks of several Solvers."""

    def __init__(self, solvers: list[Solver]):
        self._lib = L._lib()
        self.solvers = list(solvers)
        arr = (C.c_void_p * len(solvers))(*[s.handle.value for s in solvers])
        h = C.c_void_p()
        L.check(self._lib.moc_batch_create(len(solvers), arr, C.byref(h)), "moc_batch_create")
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.moc_batch_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def autotune(self) -> list[int]:
        L.check(self._lib.moc_batch_autotune(self._h), "moc_batch_autotune")
        return self.widths()

    def widths(self) -> list[int]:
        w = (C.c_int * len(self.solvers))()
        L.check(self._lib.moc_batch_widths(self._h, w), "moc_batch_widths")
        return list(w)

    def set_width(self, core: int, threads_per_track: int) -> None:
        L.check(self._lib.moc_batch_set_width(self._h, core, threads_per_track),
                "moc_batch_set_width")

    def sweep(self) -> None:
        L.check(self._lib.moc_batch_sweep(self._h), "moc_batch_sweep")

    def power_iterations(self, iters: int, graph: bool = True) -> float:
        """Runs `iters` power iterations of every core; returns device ms."""
        ms = C.c_double()
        L.check(self._lib.moc_batch_power_iterations(self._h, iters, 1 if graph else 0,
                                                     C.byref(ms)), "moc_batch_power_iterations")
        return ms.value

    def results(self) -> tuple[np.ndarray, np.ndarray]:
        n = len(self.solvers)
        k = np.empty(n, np.float64)
        r = np.empty(n, np.float64)
        L.check(self._lib.moc_batch_results(self._h, L.ptr(k, C.c_double), L.ptr(r, C.c_double)),
                "moc_batch_results")
        return k, r

    def launch_count(self) -> int:
        return int(self._lib.moc_batch_launch_count(self._h))
