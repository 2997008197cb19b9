"""Benchmark: segment-group integrations/s of the SimpleMOC transport sweep.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--config CONFIG] [--launch T,C]
    python bench.py --impl reference ...     # the CPU reference arm

CONFIG: default (the headline), batched (64 independent cores in one launch,
CUDA-graph power iteration), adjoint (adjoint / forward sweep time), dropin
(power iterations through the reference's own entry points), flat (the default
problem with the flat source, axial_exp = 0), small and default_1k (parity and
profiling sizes).

A step is one power iteration of src/main.c:57-92 (transport sweep,
renormalize_flux, update_sources, compute_keff) over the whole problem; the
value counts N3D * S * G integrations per step.  The default workload is the
default strawman problem (17x17 assemblies of 17x17 pins, 400 cm, 30 axial
regions per pin, 64 azimuthal x 256 tracks, 10 polar angles, 80 stacked rays,
50 segments per 3D track, 100 groups; ~15 GB on the device).  Inputs are
synthetic and seeded, larger than L2 (no flush needed).

`value` is the chosen mode (MIXED: the fastest mode whose FSR flux stays
within 1e-5 of the FP64 mode); the PLAIN (reference-arithmetic) rate is
reported beside it.  `e2e` repeats the measurement through the public C ABI
with pinned host buffers: every step uploads all inputs (streamed: the sweep
starts on the first chunks of tracks while the rest copy), runs one power
iteration and downloads the FSR fluxes and k_eff.  Its value is the median
step (the metric's statistic; the host link of a shared machine has slow
phases), with the per-step times and the mean beside it.

With --gpus N > 1 (torchrun) every rank sweeps an independent replica of the
problem: the sweep has no data-path collective on one problem per GPU
("replicas only"), so scaling is weak.
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


def _args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--config", choices=["default", "small", "default_1k", "flat", "batched",
                                         "adjoint", "dropin"],
                    default="default")
    ap.add_argument("--cores", type=int, default=64, help="cores of the batched workload")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0,
                    help="target CPU time of one reference-arm sample")
    ap.add_argument("--accuracy-iters", type=int, default=20,
                    help="power iterations of the accuracy comparison against the FP64 mode "
                         "(on the whole workload)")
    ap.add_argument("--floor", action="store_true",
                    help="accuracy: also FP64 arithmetic on FP32-rounded state")
    ap.add_argument("--no-compensated", action="store_true",
                    help="skip timing MIXED with compensated tallies")
    ap.add_argument("--launch", default=None, metavar="TPW,CPL",
                    help="fixed sweep launch shape (threads per track, chunks per thread) "
                         "instead of the autotuner's")
    a = ap.parse_args()
    a.launch = tuple(int(v) for v in a.launch.split(",")) if a.launch else None
    return a


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def _job_value(ms_local: float, units_per_step: float, steps: int, world: int, pg,
               device: str = "cuda") -> tuple[float, float]:
    """The whole job's time and throughput: every rank runs its own replica
    (weak scaling), the job takes as long as the slowest rank, and the value
    counts the units of all ranks.  pg is torch.distributed (any backend) or
    None for one process."""
    ms = ms_local
    if pg is not None:
        import torch
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        ms = float(t.item())
    return ms, world * units_per_step * steps / (ms / 1e3)


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def _pinned_alloc():
    import torch

    def alloc(shape, dtype):
        t = torch.empty(int(np.prod(shape)), dtype=getattr(torch, np.dtype(dtype).name),
                        pin_memory=True)
        return t.numpy().reshape(shape)
    return alloc


def _timing_port():
    """The oracle's restatement built with the reference's own timing flags
    (-Ofast -ffast-math -ftree-vectorize -fopenmp, src/Makefile:77,102-113),
    and those flags."""
    import oracle
    return oracle.Port(fast=True), oracle.timing_flags()


def _cpu_sample_spec(spec, target_s: float, port, threads: int):
    """A sample of the workload for the CPU: the same sources, groups, polar
    angles, stacked rays and segments, over fewer 2D tracks, sized to take about
    target_s seconds of OpenMP sweep."""
    import oracle
    import simplemoc_gb300 as sm
    n2d = 4
    while True:
        s = spec.with_(n_tracks_2d=n2d)
        hp = sm.generate(s)
        st = oracle.fresh_state(hp)
        op = oracle.make_problem(hp)
        t0 = time.perf_counter()
        port.sweep_omp(op, st["fine_source"], st["fine_flux"], st["psi_f"], threads)
        dt = time.perf_counter() - t0
        if dt > 0.5 or n2d >= spec.n_tracks_2d:
            n = int(min(spec.n_tracks_2d, max(1, n2d * target_s / max(dt, 1e-3))))
            return spec.with_(n_tracks_2d=n)
        n2d *= 4


def cpu_rate(spec, target_s: float, steps: int = 1):
    """Integrations/s of the oracle's OpenMP sweep (lock per fine region, as the
    reference's OpenMP build) on a bounded sample of the workload."""
    import oracle
    import simplemoc_gb300 as sm
    port, flags = _timing_port()
    threads = port.lib.oracle_omp_max_threads()
    sspec = _cpu_sample_spec(spec, target_s, port, threads)
    hp = sm.generate(sspec)
    st = oracle.fresh_state(hp)
    op = oracle.make_problem(hp)
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        port.sweep_omp(op, st["fine_source"], st["fine_flux"], st["psi_f"], threads)
        times.append(time.perf_counter() - t0)
    rate = sspec.integrations_per_sweep / float(np.median(times))
    sample = (f"OpenMP sweep of {sspec.n_tracks_2d} of {spec.n_tracks_2d} 2D tracks (all "
              f"{spec.n_polar} polar x {spec.z_stacked} stacked 3D tracks each, "
              f"{sspec.integrations_per_sweep:.3e} integrations) over the full source storage; "
              f"compiled {flags}")
    return rate, threads, sample, times, flags


METRIC = ("segment-group integrations/s per sweep, chosen vs plain @ FSR flux rel "
          "err <=1e-5")


def _workload(name: str, spec) -> str:
    """The workload as both arms name it in config.workload."""
    return (f"{name} problem: {spec.n_tracks_3d} 3D tracks x {spec.n_seg} segments x "
            f"{spec.n_groups} groups, {spec.n_fsr} FSRs")


CONTRACT = 1e-5          # FSR flux relative error against the FP64 mode
KEFF_CONTRACT = 1e-6


def flux_errors(a, ref, G: int) -> dict:
    """Relative errors of a scalar flux against the FP64 one: normwise
    (max |a - ref| / max |ref|), per FSR (each FSR's group vector in the max
    norm: max_g |a - ref| / max_g |ref|), and per element (FSR x group)."""
    a = np.asarray(a, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    d = np.abs(a - ref)
    r = np.abs(ref)
    fsr_den = r.reshape(-1, G).max(1)
    per_fsr = d.reshape(-1, G).max(1)[fsr_den > 0] / fsr_den[fsr_den > 0]
    nz = r > 0
    per_el = d[nz] / r[nz]
    qs = (0.5, 0.99, 0.999, 0.9999)
    return {
        "normwise": float(d.max() / r.max()),
        "per_fsr_max": float(per_fsr.max()),
        "per_fsr_quantiles": {str(q): float(np.quantile(per_fsr, q)) for q in qs},
        "per_fsr_frac_within_contract": float((per_fsr <= CONTRACT).mean()),
        "per_element_max": float(per_el.max()),
        "per_element_quantiles": {str(q): float(np.quantile(per_el, q)) for q in qs},
    }


def accuracy_block(spec, device: int, iters: int, floor: bool = False) -> dict:
    """Every mode against the FP64 mode (the same formulas in double with an
    exact 1 - exp(-tau)) on the whole workload over `iters` power iterations:
    FSR flux errors normwise, per FSR and per element, and the k_eff error.
    floor: also FP64 arithmetic on state rounded to FP32 after every step
    (MOC_FLAG_FP32_STATE), the error that FP32 storage alone sets."""
    import simplemoc_gb300 as sm
    hp = sm.generate(spec, with_state=False)
    t0 = time.perf_counter()
    with sm.Solver(hp, device=device, mode="fp64") as s64:
        h64 = s64.run(iters)
        p64 = s64.download64(fine_flux=True)["fine_flux"]
    out = {"workload": f"all {spec.n_tracks_3d} 3D tracks, {iters} power iterations",
           "reference": "FP64 mode", "fp64_seconds": time.perf_counter() - t0,
           "contract": {"fsr_flux_rel_err": CONTRACT, "keff_rel_err": KEFF_CONTRACT}}
    k64 = h64[-1][0]
    for name, mode, comp in (("mixed", "mixed", False), ("mixed_compensated", "mixed", True),
                             ("plain", "plain", False)):
        with sm.Solver(hp, device=device, mode=mode, compensated=comp) as s:
            h = s.run(iters)
            ph = s.download(fine_flux=True, fine_source=False, psi_f=False)["fine_flux"]
        e = flux_errors(ph, p64, spec.n_groups)
        e["keff_rel_err"] = abs(h[-1][0] - k64) / abs(k64)
        e["normwise_within_contract"] = (e["normwise"] <= CONTRACT
                                         and e["keff_rel_err"] <= KEFF_CONTRACT)
        out[name] = e
    if floor:
        with sm.Solver(hp, device=device, mode="fp64", fp32_state=True) as s:
            h = s.run(iters)
            ph = s.download64(fine_flux=True)["fine_flux"]
        e = flux_errors(ph, p64, spec.n_groups)
        e["keff_rel_err"] = abs(h[-1][0] - k64) / abs(k64)
        out["fp64_on_fp32_state"] = e
    return out


def run_reference(args, spec):
    rank, world, _ = _dist()
    if rank != 0:
        return
    import oracle
    kind = "reference" if oracle.Reference.available() else "port"
    # warm-up + timed steps, each one bounded sample sweep
    rate, threads, sample, times, flags = cpu_rate(
        spec, args.cpu_seconds / 2, steps=max(1, args.steps) + max(0, args.warmup))
    timed = times[max(0, args.warmup):] or times
    sample_ints = rate * float(np.median(times))
    value = sample_ints / float(np.mean(timed))
    line = {
        "impl": "reference", "metric": METRIC,
        "value": value, "unit": "integrations/s", "n_gpus": args.gpus, "steps": len(timed),
        "warmup": args.warmup, "ms_per_step": 1e3 * float(np.mean(timed)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": {"workload": _workload(args.config, spec),
                   "mode": "the reference's CPU sweep (PLAIN arithmetic), host cores",
                   "step": "one sweep of a bounded sample of the workload",
                   "sample": sample, "compiler_flags": flags},
        "cpu_baseline": {"value": value, "unit": "integrations/s", "cores": threads,
                         "kind": "port", "sample": sample, "compiler_flags": flags},
        "e2e": {"value": value, "unit": "integrations/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": ("the reference's own sweep code is C with a time-seeded RNG; the timed CPU "
                 "path is the oracle's restatement of attenuate_fluxes with the reference's "
                 "per-region OpenMP locks (pinned bit-for-bit to the reference objects in "
                 "this repository's tests when built with the results flags), built here "
                 "with the reference's own timing flags"),
    }
    if kind == "reference":
        line["note"] += "; reference objects available but the sweep is timed on the port"
    print(json.dumps(line), flush=True)


def _traffic_from_profiles(shape):
    """Per-launch DRAM bytes of the sweep kernel of launch shape (tpw, cpl) from the
    committed ncu summary, None if that shape was not captured."""
    p = ROOT / "profiles" / "sweep_default_traffic.txt"
    if not p.exists() or shape is None:
        return None
    key = f"dram_bytes_per_launch_full_size[{shape[0]}x{shape[1]}]"
    for ln in p.read_text().splitlines():
        if ln.startswith(key):
            try:
                return float(ln.split("=")[1].split()[0])
            except (IndexError, ValueError):
                return None
    return None


def run_batched(args):
    """The batched workload: independent small cores of uneven sizes swept in
    one persistent launch per iteration, the power iteration replayed as a CUDA
    graph.  value = integrations of all cores per second (MIXED, graph); the
    same cores run one after the other through the single-problem path, and
    the PLAIN batch, are reported beside it."""
    import torch

    import simplemoc_gb300 as sm
    from simplemoc_gb300.batch import Batch, batched_specs
    torch.cuda.set_device(0)
    specs = batched_specs(args.cores)
    hps = [sm.generate(s, with_state=False) for s in specs]
    ints = sum(s.integrations_per_sweep for s in specs)
    K, W = max(1, args.steps), max(0, args.warmup)
    out = {}
    for mode in ("mixed", "plain"):
        solvers = [sm.Solver(h, mode=mode) for h in hps]
        with Batch(solvers) as b:
            widths = b.autotune()
            b.power_iterations(max(1, W), graph=True)
            with ClockSampler(0) as clk:
                ms = b.power_iterations(K, graph=True)
            keff, _ = b.results()
        out[mode] = {"value": ints * K / (ms / 1e3), "ms_per_step": ms / K, "widths": widths,
                     "clocks": clk.summary(), "keff_mean": float(np.mean(keff))}
        # the same cores one after the other through the single-problem path
        for s_ in solvers:
            s_.power_iteration(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        tot = 0.0
        for s_ in solvers:
            r = s_.time_power_iterations(K)
            tot += r["ms_total"]
        out[mode]["sequential_value"] = ints * K / (tot / 1e3)
        for s_ in solvers:
            s_.close()
    line = {
        "metric": "segment-group integrations/s per sweep, chosen vs plain @ FSR flux rel err "
                  "<=1e-5",
        "value": out["mixed"]["value"], "unit": "integrations/s", "n_gpus": 1, "steps": K,
        "warmup": W, "ms_per_step": out["mixed"]["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": f"batched: {len(specs)} independent cores, "
                               f"{sum(s.n_tracks_3d for s in specs)} 3D tracks, "
                               f"{ints:.3e} integrations per iteration",
                   "mode": "mixed", "step": "one power iteration of every core (CUDA graph)",
                   "l2": "inputs larger than L2 (no flush)"},
        "plain": {"value": out["plain"]["value"], "unit": "integrations/s"},
        "chosen_vs_plain": out["mixed"]["value"] / out["plain"]["value"],
        "sequential": {"mixed": out["mixed"]["sequential_value"],
                       "plain": out["plain"]["sequential_value"]},
        "batched_vs_sequential": out["mixed"]["value"] / out["mixed"]["sequential_value"],
        "widths": out["mixed"]["widths"], "clocks": out["mixed"]["clocks"],
    }
    print(json.dumps(line), flush=True)


def run_adjoint(args):
    """The adjoint workload: the small problem's geometry with 40 groups, one
    fixed-source sweep and its reverse sweep (psi checkpoints every 8
    segments).  Reports forward, forward-with-checkpoints and reverse times
    (events on the library stream, via the C ABI).  value = reverse / forward:
    the checkpointed forward replaces the plain forward at the same cost, so the
    gradient costs the reverse sweep; (checkpointed forward + reverse) / forward
    is reported beside it."""
    import ctypes as C

    import torch

    import simplemoc_gb300 as sm
    from simplemoc_gb300 import _lib as L
    torch.cuda.set_device(0)
    spec = sm.CONFIG_SMALL.with_(n_groups=40, seed=20260104)
    hp = sm.generate(spec, with_state=False)
    dev = torch.device("cuda", 0)
    K, W = max(1, args.steps), max(0, args.warmup)
    with sm.Solver(hp, mode="mixed") as s:
        lib, h = s._lib, s.handle
        shape = s.autotune()[:2]
        s.time_sweep(max(1, W))
        t_fwd = s.time_sweep(K)
        dphi = torch.rand(spec.n_fsr * spec.n_groups, device=dev)
        torch.cuda.synchronize()
        fms, rms = C.c_double(), C.c_double()
        fw, rv = [], []
        for it in range(W + K):
            L.check(lib.moc_time_adjoint(h, 8, dphi.data_ptr(), C.byref(fms), C.byref(rms)),
                    "moc_time_adjoint")
            if it >= W:
                fw.append(fms.value)
                rv.append(rms.value)
    f, r = float(np.median(fw)), float(np.median(rv))
    line = {
        "metric": "adjoint (reverse) sweep time / forward sweep time", "value": r / t_fwd,
        "checkpointed_forward_plus_reverse_over_forward": (f + r) / t_fwd,
        "unit": "ratio", "n_gpus": 1, "steps": K, "warmup": W, "higher_is_better": False,
        "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": f"adjoint: {spec.n_tracks_3d} tracks x {spec.n_seg} segments x "
                               f"{spec.n_groups} groups, checkpoints every 8 segments"},
        "forward_ms": t_fwd, "forward_with_checkpoints_ms": f, "reverse_ms": r,
        "launch_shape": list(shape),
        "integrations_per_s_forward": spec.integrations_per_sweep / (t_fwd / 1e3),
    }
    print(json.dumps(line), flush=True)


def run_dropin(args):
    """The drop-in: the reference's own entry points (transport_sweep,
    renormalize_flux, update_sources, compute_keff with the reference's structs,
    include/simplemoc_refabi.h) on a reference-layout problem of the small
    problem's size: 1024 2D tracks of ~50 segments, 4 polar angles, 300 stacked
    rays over 200 cm, 100 groups.  The traversal is the reference's (axial
    splitting, stacked-ray retirement) in PLAIN arithmetic.  A step is one power
    iteration through the four symbols (each returns on the host, as the
    reference's do); integrations = the traversal's 3D sub-segments x groups.
    The value is the library's default source-id mode, libc rand() drawn on the
    host in the serial reference's order (what an unchanged src/main.c gets);
    the counter-hash mode, whose ids are drawn on the device, is reported
    beside it."""
    import ctypes as C

    import simplemoc_gb300 as sm
    from simplemoc_gb300 import refabi
    spec = sm.CONFIG_SMALL
    hp = sm.generate(spec, with_state=False)
    Z = spec.z_stacked
    geo = refabi.make_geometry(spec.seed + 1, spec.n_tracks_2d, spec.n_polar, Z, 50.0,
                               spec.height / Z)
    G = spec.n_groups
    K, W = max(1, args.steps), max(1, args.warmup)
    lb = refabi.lib()
    out = {}
    for mode_name, mode in (("hash", refabi.RNG_HASH), ("libc", refabi.RNG_LIBC)):
        rp = refabi.build(hp, geo)
        lb.moc_ref_finalize()
        lb.moc_ref_set_rng(mode, 1234)
        grid = refabi.CommGrid()
        keff = [1.0]
        rng_ms = []

        def step():
            lb.transport_sweep(C.byref(rp.params), C.byref(rp.input))
            rng_ms.append(float(lb.moc_ref_last_rng_ms()))
            lb.renormalize_flux(rp.params, rp.input, grid)
            lb.update_sources(rp.params, rp.input, keff[0])
            keff[0] = lb.compute_keff(rp.params, rp.input, grid)
            if lb.moc_ref_status() != 0:
                raise RuntimeError(f"drop-in status {lb.moc_ref_status()}")
            return int(lb.moc_ref_last_segments())

        for _ in range(W):
            step()
        rng_ms.clear()
        t0 = time.perf_counter()
        segs = sum(step() for _ in range(K))
        dt = time.perf_counter() - t0
        lb.moc_ref_finalize()
        out[mode_name] = {"value": segs * G / dt, "ms_per_step": 1e3 * dt / K,
                          "rng_ms_per_step": float(np.mean(rng_ms)),
                          "sub_segments_per_sweep": segs // K, "keff": keff[0]}
    line = {
        "metric": "segment-group integrations/s per power iteration through the reference's "
                  "entry points", "value": out["libc"]["value"], "unit": "integrations/s",
        "n_gpus": 1, "steps": K, "warmup": W, "ms_per_step": out["libc"]["ms_per_step"],
        "higher_is_better": True, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": f"drop-in: {spec.n_tracks_2d} 2D tracks x {spec.n_polar} polar x "
                               f"{Z} stacked rays, {G} groups, reference traversal, PLAIN",
                   "source_ids": "libc rand() on the host, the serial reference's sequence",
                   "sub_segments_per_sweep": out["libc"]["sub_segments_per_sweep"]},
        "libc_rand_ms_per_step": out["libc"]["rng_ms_per_step"],
        "hash": {k: out["hash"][k] for k in ("value", "ms_per_step", "sub_segments_per_sweep")},
        "keff": out["libc"]["keff"],
    }
    print(json.dumps(line), flush=True)


def main():
    args = _args()
    import simplemoc_gb300 as sm
    if args.config == "dropin":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable":
                              "the drop-in line times this library through the reference's "
                              "symbols; the reference arm is the default config's"}))
            return
        run_dropin(args)
        return
    if args.config == "adjoint":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable":
                              "the reference has no adjoint sweep"}))
            return
        run_adjoint(args)
        return
    if args.config == "batched":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable":
                              "the CPU arm times the default problem"}))
            return
        run_batched(args)
        return
    spec = sm.CONFIGS[args.config]
    if args.impl == "reference":
        run_reference(args, spec)
        return
    rank, world, local = _dist()
    import torch
    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        pg = dist

    def barrier():
        if pg:
            pg.barrier()
        torch.cuda.synchronize()

    e2e_on = not args.no_e2e
    alloc = _pinned_alloc() if e2e_on else None
    hp = sm.generate(spec, with_state=e2e_on, alloc=alloc)
    solver = sm.Solver(hp, device=local, mode="mixed")
    K, W = max(1, args.steps), max(0, args.warmup)
    ints = spec.integrations_per_sweep

    # ---- chosen (MIXED) ------------------------------------------------------
    def tune():
        if args.launch:
            solver.set_launch(*args.launch)
            return list(args.launch)
        return list(solver.autotune()[:2])

    shapes = {"mixed": tune()}
    if W:
        solver.time_power_iterations(W)
    barrier()
    l0 = solver.launch_count()
    with ClockSampler(local) as clk:
        r = solver.time_power_iterations(K)
    launches = solver.launch_count() - l0
    barrier()
    ms, value = _job_value(r["ms_total"], ints, K, world, pg)
    sweep_ms = r["ms_sweeps"] / K

    # ---- plain (reference arithmetic) ------------------------------------------
    solver.set_mode("plain")
    shapes["plain"] = tune()
    solver.time_power_iterations(1)
    rp = solver.time_power_iterations(K)
    plain_value = ints * K / (rp["ms_total"] / 1e3)
    plain_sweep_ms = rp["ms_sweeps"] / K

    # ---- MIXED with compensated tallies ------------------------------------------
    comp = None
    if not args.no_compensated:
        solver.set_mode("mixed", compensated=True)
        shapes["mixed_compensated"] = tune()
        solver.time_power_iterations(1)
        rc_ = solver.time_power_iterations(K)
        comp = {"value": ints * K / (rc_["ms_total"] / 1e3), "unit": "integrations/s",
                "sweep_ms": rc_["ms_sweeps"] / K}
    solver.set_mode("mixed")
    if args.launch:
        solver.set_launch(*args.launch)
    else:
        solver.autotune(measure=False)
    phases = solver.time_phases(3)["phases_ms"]

    # ---- end to end through the C ABI with host buffers ------------------------
    e2e = None
    if e2e_on:
        out = {"fine_flux": alloc((spec.n_fsr * spec.n_groups,), np.float32)}
        steps = K
        # the backward angular flux goes as NULL (zeros): the reference never
        # sweeps it (only f_psi, src/solver.c:489) and only rescales it, so in
        # its power iteration it stays the zeros it starts as (src/tracks.c:143)
        from dataclasses import replace as _replace
        hp_step = _replace(hp, psi_b=None)
        solver.upload(hp_step)
        solver.power_iteration(1.0)
        solver.download(fine_flux=True, fine_source=False, psi_f=False, out=out)
        barrier()
        t0 = time.perf_counter()
        marks = [t0]
        for _ in range(steps):
            solver.upload(hp_step)
            solver.power_iteration(1.0)
            solver.download(fine_flux=True, fine_source=False, psi_f=False, out=out)
            marks.append(time.perf_counter())
        dt = marks[-1] - t0
        barrier()
        step_s = [b - a for a, b in zip(marks, marks[1:])]
        # the median step, as the metric takes the median of its timed sweeps:
        # the host link of a shared machine has phases several times slower,
        # which the mean over all steps keeps too (value_mean)
        med = float(np.median(step_s))
        if pg:
            t = torch.tensor([med], dtype=torch.float64, device="cuda")
            pg.all_reduce(t, op=pg.ReduceOp.MAX)
            med = float(t.item())
        e2e = {"value": world * ints / med, "unit": "integrations/s",
               "statistic": f"median of {steps} steps",
               "value_mean": world * ints * steps / dt,
               "h2d_bytes_per_step": hp_step.input_nbytes(),
               "inputs": "every input array of the problem from pinned host memory; psi_b "
                         "as NULL (zeros: never swept, only rescaled)",
               "d2h_bytes_per_step": int(out["fine_flux"].nbytes + 16),
               "ms_steps": [round(1e3 * x, 2) for x in step_s]}

    # ---- accuracy of every mode against the FP64 mode, on the whole workload ---
    accuracy = None
    if not args.no_accuracy and rank == 0:
        solver.close()                  # room for the FP64 state
        accuracy = accuracy_block(spec, local, max(1, args.accuracy_iters), args.floor)

    # ---- CPU baseline (rank 0, N = 1 only) -------------------------------------
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        rate, threads, sample, _, flags = cpu_rate(spec, args.cpu_seconds)
        cpu = {"value": rate, "unit": "integrations/s", "cores": threads, "kind": "port",
               "sample": sample, "compiler_flags": flags}

    peak, peak_kind = _peaks()
    alg_bytes = spec.algorithmic_bytes()
    achieved = alg_bytes / (sweep_ms / 1e3) / 1e9
    traffic = (_traffic_from_profiles(tuple(shapes["mixed"])) if args.config == "default"
               else None)
    if rank == 0:
        line = {
            "metric": METRIC,
            "value": value, "unit": "integrations/s", "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": _workload(args.config, spec),
                       "mode": "mixed", "tallies": "FP32 reductions, uncompensated",
                       "step": "one power iteration",
                       "l2": "inputs larger than L2 (no flush)",
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "accuracy_criterion": "FSR flux normwise <= 1e-5 and k_eff <= 1e-6 "
                                             "against the FP64 mode, whole problem, 20 "
                                             "iterations; per-FSR figures in accuracy"},
            "plain": {"value": plain_value, "unit": "integrations/s",
                      "sweep_ms": plain_sweep_ms},
            "chosen_vs_plain": value / world / plain_value,
            "compensated": comp,
            "phases_ms": {k: v / 3 for k, v in phases.items()},
            "sweep_ms": sweep_ms, "keff": r["keff"], "launch_shape": shapes,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "traffic_source": "ncu of the chosen launch shape on 1024 of the 2D "
                                           "tracks, scaled to the full launch",
                         "peak_source": peak_kind,
                         "algorithmic_bytes_per_launch": alg_bytes},
            "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
            "clocks": clk.summary(), "accuracy": accuracy,
        }
        print(json.dumps(line), flush=True)
    solver.close()
    if pg:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
