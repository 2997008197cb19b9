"""The track-partitioned power iteration on the GPU library, on one device.

Two track ranges of one problem run as two handles driven from two host
threads, each through TrackPartitioned with SolverBackend; their all-reduce is
a host-side stand-in (a barrier and a sum on the device, no kernel waiting on
another).  The result equals one handle sweeping every track.  The collective
itself (NCCL across GPUs, gloo on CPU) is covered by the CPU ranks of
test_tracks_parallel.py."""
import threading

import numpy as np
import pytest

from tests._util import rel_err

pytestmark = pytest.mark.gpu
TOL = 1e-5


class _ThreadAllReduce:
    """all_reduce(SUM) between host threads: every thread's tensor is replaced
    by the sum of all of them (in rank order)."""

    class ReduceOp:
        SUM = "sum"

    def __init__(self, world):
        self.world = world
        self.bar = threading.Barrier(world)
        self.slots = [None] * world
        self.lock = threading.Lock()
        self.calls = 0

    def all_reduce(self, t, op=None, group=None):
        import torch
        assert op == self.ReduceOp.SUM
        rank = threading.current_thread().rank
        self.slots[rank] = t
        self.bar.wait()
        if rank == 0:
            acc = self.slots[0].clone()
            for x in self.slots[1:]:
                acc += x
            for x in self.slots:
                x.copy_(acc)
            torch.cuda.synchronize()
            with self.lock:
                self.calls += 1
        self.bar.wait()


@pytest.mark.parametrize("mode", ["plain", "mixed"])
def test_two_track_ranges_equal_one_problem(gpu_available, mode):
    import simplemoc_gb300 as sm
    from simplemoc_gb300.tracks_parallel import (SolverBackend, TrackPartitioned, partition,
                                                 rank_problem)
    spec = sm.ProblemSpec(n_groups=40, fai=5, cai=4, height=200.0, n_sources=400,
                          n_tracks_2d=33, n_polar=4, z_stacked=20, n_seg=50, seed=9090)
    hp = sm.generate(spec)
    iters = 3
    with sm.Solver(hp, mode=mode) as full:
        ref_hist = full.run(iters)
        ref = full.download(fine_flux=True, fine_source=True, psi_f=True)
    world = 2
    dist = _ThreadAllReduce(world)
    results = [None] * world
    errors = []

    def rank_main(rank):
        threading.current_thread().rank = rank
        try:
            lo, hi = partition(spec.n_tracks_2d, world, rank)
            with sm.Solver(rank_problem(hp, lo, hi), mode=mode) as s:
                hist = TrackPartitioned(SolverBackend(s, 0), rank, world, dist).run(iters)
                results[rank] = (lo, hi, hist, s.download(fine_flux=True, fine_source=True,
                                                          psi_f=True))
        except Exception as e:          # reported by the main thread
            errors.append(e)
            dist.bar.abort()

    threads = [threading.Thread(target=rank_main, args=(r,)) for r in range(world)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=300)
    assert not errors, errors
    assert dist.calls == iters
    G = spec.n_groups
    PZG = spec.n_polar * spec.z_stacked * G
    for lo, hi, hist, out in results:
        np.testing.assert_allclose(np.asarray(hist)[:, 0], np.asarray(ref_hist)[:, 0], rtol=TOL)
        assert rel_err(out["fine_flux"], ref["fine_flux"]) <= TOL
        assert rel_err(out["fine_source"], ref["fine_source"]) <= TOL
        assert rel_err(out["psi_f"], ref["psi_f"][lo * PZG:hi * PZG]) <= TOL
    # the replicated state is the same on both ranks, to the bit
    assert np.array_equal(results[0][3]["fine_flux"], results[1][3]["fine_flux"])
    assert results[0][2] == results[1][2]


def test_flux_storage_is_the_handles_flux(gpu_available):
    """moc_fine_flux_storage: the padded [NS*F][ldg] storage of the scalar flux;
    writing through it changes what the handle downloads."""
    import torch

    import simplemoc_gb300 as sm
    from simplemoc_gb300.tracks_parallel import SolverBackend
    spec = sm.ProblemSpec(n_groups=7, fai=3, cai=2, height=60.0, n_sources=30, n_tracks_2d=4,
                          n_polar=2, z_stacked=4, n_seg=10, seed=77)
    hp = sm.generate(spec)
    with sm.Solver(hp) as s:
        s.transport_sweep()
        s.synchronize()
        st = s.flux_storage()
        assert st["ldg"] == 8 and st["elem_bytes"] == 4
        assert st["n"] == spec.n_fsr * st["ldg"]
        t = SolverBackend(s, 0).flux_tensor()
        view = t.view(spec.n_fsr, st["ldg"])
        got = s.download(fine_flux=True, fine_source=False, psi_f=False)["fine_flux"]
        assert np.array_equal(view[:, :7].cpu().numpy().ravel(), got)
        assert not view[:, 7:].any()                    # padding stays zero
        view.mul_(2.0)
        torch.cuda.synchronize()
        twice = s.download(fine_flux=True, fine_source=False, psi_f=False)["fine_flux"]
        assert np.array_equal(twice, 2 * got)


def test_phase_times_under_the_reference_names(gpu_available):
    """moc_time_phases: the five phases of the reference's summary; the sweep
    dominates, there is no exchange on one device, and the state it leaves is
    that of the same number of power iterations."""
    import simplemoc_gb300 as sm
    from simplemoc_gb300 import _lib as L
    spec = sm.ProblemSpec(n_groups=40, fai=5, cai=4, height=200.0, n_sources=300,
                          n_tracks_2d=1024, n_polar=4, z_stacked=64, n_seg=50, seed=31)
    hp = sm.generate(spec)
    with sm.Solver(hp) as a, sm.Solver(hp) as b:
        r = a.time_phases(3)
        hist = b.run(3)
        oa = a.download(fine_flux=True, fine_source=True, psi_f=True)
        ob = b.download(fine_flux=True, fine_source=True, psi_f=True)
    ph = r["phases_ms"]
    assert tuple(ph) == L.PHASE_NAMES
    assert ph["Domain Flux Exchange"] == 0.0
    assert all(ph[k] > 0 for k in L.PHASE_NAMES if k != "Domain Flux Exchange")
    assert ph["Transport Sweep"] == max(ph.values())
    assert abs(r["keff"] - hist[-1][0]) <= 1e-6 * abs(hist[-1][0])
    for k in ("fine_flux", "fine_source", "psi_f"):   # tally order only
        assert rel_err(oa[k], ob[k]) <= TOL, k
