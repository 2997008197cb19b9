"""The solver interface of SimpleMOC (src/solver.c) over the GPU library.

Method names and meanings follow the reference's four entry points
(src/SimpleMOC_header.h:225,235-237, called from src/main.c:61,75,81,87):

    transport_sweep()        -> segments processed (Input.segments_processed)
    renormalize_flux()
    update_sources(keff)     -> source residual
    compute_keff(leakage=0)  -> k_eff

State lives on the device between calls; `download()` copies it back.
Errors raise MocError (the library never exits the process).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .problem import HostProblem

MODES = {"plain": L.MOC_MODE_PLAIN, "mixed": L.MOC_MODE_MIXED, "fp64": L.MOC_MODE_FP64}


class Solver:
    def __init__(self, problem: HostProblem, device: int = 0, mode: str = "plain",
                 compensated: bool = False, simt_update: bool = False,
                 deterministic: bool = False, fp32_state: bool = False):
        self._lib = L._lib()
        self.problem = problem
        self.spec = problem.spec
        self._dims = problem.dims()
        self._host = problem.host()
        h = C.c_void_p()
        L.check(self._lib.moc_create(C.byref(self._dims), C.byref(self._host), device,
                                     C.byref(h)), "moc_create")
        self._h = h
        self.mode = "plain"
        self.set_mode(mode, compensated, simt_update, deterministic, fp32_state)

    # ---- lifecycle ---------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.moc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def set_mode(self, mode: str, compensated: bool = False, simt_update: bool = False,
                 deterministic: bool = False, fp32_state: bool = False) -> None:
        """mode: "plain", "mixed" or "fp64".  compensated: MIXED tallies with
        compensation.  simt_update: MIXED update_sources on the CUDA cores
        instead of the tensor cores.  deterministic: tallies added in the
        serial order of tracks and segments (PLAIN, MIXED).  fp32_state: FP64
        arithmetic on state rounded to FP32 values (the FP32-storage floor)."""
        flags = (L.MOC_FLAG_COMPENSATED if compensated else 0) | \
            (L.MOC_FLAG_SIMT_UPDATE if simt_update else 0) | \
            (L.MOC_FLAG_DETERMINISTIC if deterministic else 0) | \
            (L.MOC_FLAG_FP32_STATE if fp32_state else 0)
        L.check(self._lib.moc_set_mode(self._h, MODES[mode], flags), "moc_set_mode")
        self.mode = mode

    def set_launch(self, threads_per_track: int, chunks_per_thread: int) -> None:
        L.check(self._lib.moc_set_launch(self._h, threads_per_track, chunks_per_thread),
                "moc_set_launch")

    def set_pipeline(self, stages: int) -> None:
        """0: register prefetch of the next segment's rows; 4: a 4-stage
        shared-memory ring filled by the bulk-copy engine; -1: automatic."""
        L.check(self._lib.moc_set_pipeline(self._h, stages), "moc_set_pipeline")

    def pipeline(self) -> int:
        v = C.c_int()
        L.check(self._lib.moc_get_pipeline(self._h, C.byref(v)), "moc_get_pipeline")
        return int(v.value)

    def launch_shape(self) -> tuple[int, int]:
        a, b = C.c_int(), C.c_int()
        L.check(self._lib.moc_get_launch(self._h, C.byref(a), C.byref(b)), "moc_get_launch")
        return a.value, b.value

    def autotune(self, n_tracks: int = 0, measure: bool = True) -> tuple[int, int, float]:
        """Picks the fastest launch shape for the current mode (moc_autotune)."""
        a, b, ms = C.c_int(), C.c_int(), C.c_double()
        L.check(self._lib.moc_autotune(self._h, n_tracks, C.byref(a), C.byref(b),
                                       C.byref(ms) if measure else None), "moc_autotune")
        return a.value, b.value, ms.value

    def upload(self, problem: HostProblem | None = None) -> None:
        """Copies `problem` (default: the problem the solver was made with) to
        the device.  The per-track copies may still be in flight when this
        returns.  The arrays of this upload and of the one before it stay
        referenced: an upload joins the copies of the one before on the device
        only, and its own staging wait is what retires the copies of the upload
        two back."""
        p = problem or self.problem
        self._host_prev = getattr(self, "_host_problem", None)
        self._host = p.host()
        self._host_problem = p
        L.check(self._lib.moc_upload(self._h, C.byref(self._host)), "moc_upload")

    # ---- the four reference entry points ------------------------------------
    def transport_sweep(self) -> int:
        n = C.c_int64()
        L.check(self._lib.moc_transport_sweep(self._h, C.byref(n)), "transport_sweep")
        return int(n.value)

    def renormalize_flux(self) -> None:
        L.check(self._lib.moc_renormalize_flux(self._h), "renormalize_flux")

    def update_sources(self, keff: float) -> float:
        r = C.c_double()
        L.check(self._lib.moc_update_sources(self._h, keff, C.byref(r)), "update_sources")
        return float(r.value)

    def compute_keff(self, leakage: float = 0.0) -> float:
        k = C.c_double()
        L.check(self._lib.moc_compute_keff(self._h, leakage, C.byref(k)), "compute_keff")
        return float(k.value)

    def power_iteration(self, keff: float) -> tuple[float, float]:
        """One pass of src/main.c:57-92; returns (keff, residual)."""
        k, r = C.c_double(), C.c_double()
        L.check(self._lib.moc_power_iteration(self._h, keff, C.byref(k), C.byref(r)),
                "power_iteration")
        return float(k.value), float(r.value)

    def run(self, n_iters: int, keff: float = 1.0) -> list[tuple[float, float]]:
        out = []
        for _ in range(n_iters):
            keff, res = self.power_iteration(keff)
            out.append((keff, res))
        return out

    # ---- utilities ----------------------------------------------------------
    def synchronize(self) -> None:
        L.check(self._lib.moc_synchronize(self._h), "synchronize")

    def time_sweep(self, iters: int = 1) -> float:
        ms = C.c_double()
        L.check(self._lib.moc_time_sweep(self._h, iters, C.byref(ms)), "time_sweep")
        return float(ms.value)

    def time_power_iterations(self, iters: int) -> dict:
        """Device-timed power iterations (k_eff chained on the device)."""
        tot, sw, k, r = C.c_double(), C.c_double(), C.c_double(), C.c_double()
        L.check(self._lib.moc_time_power_iterations(self._h, iters, C.byref(tot), C.byref(sw),
                                                    C.byref(k), C.byref(r)),
                "time_power_iterations")
        return {"ms_total": tot.value, "ms_sweeps": sw.value, "keff": k.value,
                "residual": r.value}

    def time_phases(self, iters: int) -> dict:
        """Device time of each phase of `iters` power iterations, under the
        reference's phase names (src/main.c:103-113), in milliseconds summed
        over the iterations, plus the final k_eff and residual."""
        ms = (C.c_double * len(L.PHASE_NAMES))()
        k, r = C.c_double(), C.c_double()
        L.check(self._lib.moc_time_phases(self._h, iters, ms, C.byref(k), C.byref(r)),
                "moc_time_phases")
        return {"phases_ms": dict(zip(L.PHASE_NAMES, (float(x) for x in ms))),
                "keff": k.value, "residual": r.value}

    def launch_count(self) -> int:
        return int(self._lib.moc_launch_count(self._h))

    def zero_state(self, flux: bool = True, psi: bool = False) -> None:
        """Zeroes the scalar flux and/or the angular flux (moc_zero_state)."""
        L.check(self._lib.moc_zero_state(self._h, int(flux), int(psi)), "moc_zero_state")

    def flux_storage(self) -> dict:
        """The handle's scalar-flux storage on the device (moc_fine_flux_storage):
        pointer, element count, row stride and element size.  Access it only
        after synchronize() and before the handle's next call."""
        ptr, n, ldg, eb = C.c_void_p(), C.c_int64(), C.c_int32(), C.c_int32()
        L.check(self._lib.moc_fine_flux_storage(self._h, C.byref(ptr), C.byref(n), C.byref(ldg),
                                                C.byref(eb)), "moc_fine_flux_storage")
        return {"ptr": int(ptr.value or 0), "n": int(n.value), "ldg": int(ldg.value),
                "elem_bytes": int(eb.value)}

    def device_bytes(self) -> int:
        return int(self._lib.moc_device_bytes(self._h))

    def download(self, fine_flux=True, fine_source=True, psi_f=True, psi_b=False,
                 out: dict | None = None) -> dict:
        s = self.spec
        nf, nt = s.n_fsr * s.n_groups, s.n_tracks_3d * s.n_groups
        res = {} if out is None else out
        want = {"fine_flux": (fine_flux, nf), "fine_source": (fine_source, nf),
                "psi_f": (psi_f, nt), "psi_b": (psi_b, nt)}
        for k, (w, n) in want.items():
            if w and k not in res:
                res[k] = np.empty(n, dtype=np.float32)
        f = C.c_float
        L.check(self._lib.moc_download(self._h, L.ptr(res.get("fine_flux"), f),
                                       L.ptr(res.get("fine_source"), f),
                                       L.ptr(res.get("psi_f"), f), L.ptr(res.get("psi_b"), f)),
                "moc_download")
        return res

    def download64(self, fine_flux=True, fine_source=False, psi_f=False, psi_b=False) -> dict:
        s = self.spec
        nf, nt = s.n_fsr * s.n_groups, s.n_tracks_3d * s.n_groups
        res = {}
        if fine_flux:
            res["fine_flux"] = np.empty(nf, dtype=np.float64)
        if fine_source:
            res["fine_source"] = np.empty(nf, dtype=np.float64)
        if psi_f:
            res["psi_f"] = np.empty(nt, dtype=np.float64)
        if psi_b:
            res["psi_b"] = np.empty(nt, dtype=np.float64)
        d = C.c_double
        L.check(self._lib.moc_download64(self._h, L.ptr(res.get("fine_flux"), d),
                                         L.ptr(res.get("fine_source"), d),
                                         L.ptr(res.get("psi_f"), d), L.ptr(res.get("psi_b"), d)),
                "moc_download64")
        return res
