"""Failure handling without a GPU fault.  Nothing here traps, faults or hangs
the GPU: out-of-memory comes from a capped allocation budget, the failing calls
are injected on the host, and the one device wait that runs out waits on an
mbarrier that nothing completes, bounded by a cycle limit.  Each failure must
give its status, make its handle refuse further work (MOC_ERR_STATE), and
leave other handles and the CUDA context usable."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MOC_ERR_ARG, MOC_ERR_CUDA, MOC_ERR_OOM, MOC_ERR_STATE, MOC_ERR_TIMEOUT = 1, 2, 3, 4, 5


def _problem():
    import simplemoc_gb300 as sm
    spec = sm.ProblemSpec(n_groups=16, fai=5, cai=4, height=200.0, n_sources=80, n_tracks_2d=8,
                          n_polar=4, z_stacked=10, n_seg=20, seed=61)
    return sm.generate(spec)


def _usable(hp):
    import simplemoc_gb300 as sm
    with sm.Solver(hp) as s:
        s.transport_sweep()
        out = s.download(psi_f=True, fine_flux=False, fine_source=False)
    assert np.isfinite(out["psi_f"]).all() and out["psi_f"].any()


def test_memory_limit_gives_out_of_memory(gpu_available):
    import simplemoc_gb300 as sm
    from simplemoc_gb300 import _lib as L
    lib = L._lib()
    hp = _problem()
    try:
        L.check(lib.moc_set_memory_limit(4096), "limit")         # below this problem's needs
        with pytest.raises(sm.MocError) as e:
            sm.Solver(hp)
        assert e.value.status == MOC_ERR_OOM
    finally:
        L.check(lib.moc_set_memory_limit(0), "limit")
    _usable(hp)


@pytest.mark.parametrize("kind,status", [(0, MOC_ERR_CUDA), (1, MOC_ERR_ARG),
                                         (2, MOC_ERR_TIMEOUT)])
def test_injected_failures_stop_only_their_handle(gpu_available, kind, status):
    import simplemoc_gb300 as sm
    from simplemoc_gb300 import _lib as L
    hp = _problem()
    a, b = sm.Solver(hp), sm.Solver(hp)
    try:
        L.check(a._lib.moc_inject_fault(a.handle, kind), "inject")
        if kind != 0:                      # reported by the next call that waits
            with pytest.raises(sm.MocError) as e:
                a.synchronize()
            assert e.value.status == status
        assert a._lib.moc_status(a.handle) == status
        with pytest.raises(sm.MocError) as e:
            a.transport_sweep()
        assert e.value.status == MOC_ERR_STATE
        b.transport_sweep()
        b.synchronize()
    finally:
        a.close()
        b.close()
    _usable(hp)


def test_device_wait_that_nothing_completes_times_out(gpu_available):
    import simplemoc_gb300 as sm
    hp = _problem()
    with sm.Solver(hp) as s:
        t0 = time.perf_counter()
        rc = s._lib.moc_selftest_wait(s.handle, 20_000_000)      # ~10 ms of SM clocks
        dt = time.perf_counter() - t0
        assert rc == MOC_ERR_TIMEOUT
        assert dt < 5.0
        assert s._lib.moc_status(s.handle) == MOC_ERR_TIMEOUT
    _usable(hp)
