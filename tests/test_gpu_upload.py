"""GPU tests of the streamed upload (moc_upload): the per-track arrays go to
the device on a second stream in chunks of whole 2D tracks, and the next sweep
starts on each chunk once it has landed.  Every call sequence must give what
the synchronous upload at creation gives:

* psi after one sweep: bit-identical (each track's arithmetic is unchanged);
* fine_flux: FP32 atomic tallies in another order, normwise <= 1e-5;
* k_eff and the renormalised psi_b: <= 1e-5 relative.

13 2D tracks make three chunks of 1, 4 and 8 2D tracks (the chunks grow 4x).
"""
import ctypes as C

import numpy as np
import pytest

from tests._util import rel_err

pytestmark = pytest.mark.gpu


def _problem(seed=5, state_seed=11, n_tracks_2d=13):
    import simplemoc_gb300 as sm
    spec = sm.ProblemSpec(n_groups=22, fai=5, cai=4, height=200.0, n_sources=300,
                          n_tracks_2d=n_tracks_2d, n_polar=4, z_stacked=10, n_seg=30, seed=seed)
    hp = sm.generate(spec)
    rng = np.random.default_rng(state_seed)
    hp.fine_flux[:] = rng.random(hp.fine_flux.size, dtype=np.float32)
    hp.psi_f[:] = rng.random(hp.psi_f.size, dtype=np.float32)
    hp.psi_b[:] = rng.random(hp.psi_b.size, dtype=np.float32)
    return hp


def _other_state(hp):
    """Same dims and inputs, a different state to be overwritten by the upload."""
    c = hp.copy_state()
    c.fine_flux[:] = 7.0
    c.psi_f[:] = 3.0
    c.psi_b[:] = 0.0
    return c


@pytest.mark.parametrize("mode,n2d", [("plain", 13), ("mixed", 13), ("plain", 1),
                                      ("mixed", 300)])
def test_streamed_upload_then_sweep_matches_synchronous(gpu_available, mode, n2d):
    """1, 13 and 300 2D tracks: one chunk, three (1, 4, 8 tracks) and five
    (1, 4, 16, 64, 215 tracks)."""
    import simplemoc_gb300 as sm
    hp = _problem(n_tracks_2d=n2d)
    with sm.Solver(hp, mode=mode) as a:
        a.transport_sweep()
        ra = a.download(psi_f=True, fine_flux=True, fine_source=False)
    with sm.Solver(_other_state(hp), mode=mode) as b:
        b.upload(hp)
        b.transport_sweep()
        rb = b.download(psi_f=True, fine_flux=True, fine_source=False)
    assert np.array_equal(ra["psi_f"], rb["psi_f"])
    assert rel_err(rb["fine_flux"], ra["fine_flux"]) <= 1e-5


def test_streamed_upload_power_iterations_match(gpu_available):
    import simplemoc_gb300 as sm
    hp = _problem(seed=8)
    with sm.Solver(hp, mode="plain") as a:
        ha = a.run(2)
        ra = a.download(psi_f=True, psi_b=True, fine_flux=True, fine_source=True)
    with sm.Solver(_other_state(hp), mode="plain") as b:
        b.upload(hp)
        hb = b.run(2)
        rb = b.download(psi_f=True, psi_b=True, fine_flux=True, fine_source=True)
    assert abs(hb[-1][0] - ha[-1][0]) <= 1e-5 * abs(ha[-1][0])
    # psi_b is only rescaled: its nonzero flag is set once its copy has landed
    for k in ("psi_b", "psi_f", "fine_flux", "fine_source"):
        assert rel_err(rb[k], ra[k]) <= 1e-5, k


def test_upload_round_trip_and_ordering(gpu_available):
    import simplemoc_gb300 as sm
    hp = _problem(seed=9)
    with sm.Solver(_other_state(hp), mode="plain") as b:
        # download straight after the upload waits for the copies
        b.upload(hp)
        r = b.download(psi_f=True, psi_b=True, fine_flux=True, fine_source=True)
        for k in ("psi_f", "psi_b", "fine_flux", "fine_source"):
            assert np.array_equal(r[k], getattr(hp, k)), k
        # zeroing after an upload is not overtaken by the copies
        b.upload(hp)
        from simplemoc_gb300 import _lib as L
        L.check(b._lib.moc_zero_state(b.handle, 1, 1), "moc_zero_state")
        r = b.download(psi_f=True, psi_b=True, fine_flux=True, fine_source=False)
        assert not r["psi_f"].any() and not r["psi_b"].any() and not r["fine_flux"].any()
        # two uploads in a row: the second one wins
        b.upload(_other_state(hp))
        b.upload(hp)
        b.transport_sweep()
        rb = b.download(psi_f=True, fine_flux=False, fine_source=False)
    with sm.Solver(hp, mode="plain") as a:
        a.transport_sweep()
        ra = a.download(psi_f=True, fine_flux=False, fine_source=False)
    assert np.array_equal(ra["psi_f"], rb["psi_f"])


def _bad_ids(hp, track_2d):
    """A copy of the state whose first segment of 2D track `track_2d` has a
    source id out of range."""
    bad = hp.copy_state()
    bad.seg_src = hp.seg_src.copy()
    spec = hp.spec
    bad.seg_src[track_2d * spec.n_polar * spec.z_stacked * spec.n_seg] = spec.n_sources
    return bad


def _fresh_sweep_matches(b, hp):
    """After a valid upload the handle sweeps as a fresh one."""
    import simplemoc_gb300 as sm
    b.upload(hp)
    b.transport_sweep()
    out = b.download(psi_f=True, fine_flux=False, fine_source=False)
    with sm.Solver(hp, mode="plain") as a:
        a.transport_sweep()
        ref = a.download(psi_f=True, fine_flux=False, fine_source=False)
    assert np.array_equal(out["psi_f"], ref["psi_f"])


MOC_ERR_ARG, MOC_ERR_STATE = 1, 4


@pytest.mark.parametrize("track_2d", [0, 12])          # the first and the last chunk
@pytest.mark.parametrize("then", ["sweep_download", "power_iteration", "upload"])
def test_bad_source_ids_are_reported_by_the_next_waiting_call(gpu_available, track_2d, then):
    """A streamed upload leaves the source ids to the sweep, which reads each
    one through a bounds check: an id out of range makes the next call that
    waits for the device return MOC_ERR_ARG, then work is refused until a valid
    upload (a second upload before any sweep simply replaces the first)."""
    import simplemoc_gb300 as sm
    hp = _problem(seed=10)
    with sm.Solver(hp, mode="plain") as b:
        b.upload(_bad_ids(hp, track_2d))
        if then == "upload":
            _fresh_sweep_matches(b, hp)
            return
        with pytest.raises(sm.MocError) as e:
            if then == "sweep_download":
                b.transport_sweep()
                b.download(psi_f=True, fine_flux=False, fine_source=False)
            else:
                b.power_iteration(1.0)
        assert e.value.status == MOC_ERR_ARG
        with pytest.raises(sm.MocError) as e:
            b.transport_sweep()
        assert e.value.status == MOC_ERR_STATE
        assert b._lib.moc_status(b.handle) == 0          # refused, not failed
        _fresh_sweep_matches(b, hp)


def test_create_rejects_bad_source_ids(gpu_available):
    """Creation uploads synchronously and checks every id on the host."""
    import simplemoc_gb300 as sm
    hp = _problem(seed=10)
    bad = _bad_ids(hp, 12)
    with pytest.raises(sm.MocError) as e:
        sm.Solver(bad, mode="plain")
    assert e.value.status == MOC_ERR_ARG


def test_streamed_upload_without_room_for_the_flux_side_buffer(gpu_available):
    """A streamed upload copies the scalar flux into a side buffer and adds it
    after the sweep; when the handle may not allocate that buffer (a capped
    device budget) the flux is copied into place instead, with the same result."""
    import simplemoc_gb300 as sm
    from simplemoc_gb300 import _lib as L
    hp = _problem(seed=12)
    with sm.Solver(hp, mode="plain") as a:
        a.transport_sweep()
        ra = a.download(psi_f=True, fine_flux=True, fine_source=False)
    lib = L._lib()
    with sm.Solver(_other_state(hp), mode="plain") as b:
        held = int(lib.moc_device_bytes(b.handle))
        try:
            L.check(lib.moc_set_memory_limit(held + 4096), "limit")   # no room for 1 flux copy
            b.upload(hp)
            b.transport_sweep()
            rb = b.download(psi_f=True, fine_flux=True, fine_source=False)
            assert int(lib.moc_device_bytes(b.handle)) == held
        finally:
            L.check(lib.moc_set_memory_limit(0), "limit")
    assert np.array_equal(ra["psi_f"], rb["psi_f"])
    assert rel_err(rb["fine_flux"], ra["fine_flux"]) <= 1e-5


def test_streamed_upload_of_null_backward_flux_gives_zeros(gpu_available):
    """psi_b passed as NULL to a streamed upload means zeros: it replaces a
    non-zero psi_b on the device, and two power iterations then equal those of
    an upload with a zero array."""
    from dataclasses import replace

    import simplemoc_gb300 as sm
    hp = _problem()                                      # psi_b non-zero
    zero_b = hp.copy_state()
    zero_b.psi_b[:] = 0.0
    null_b = replace(hp.copy_state(), psi_b=None)
    with sm.Solver(hp) as a, sm.Solver(hp) as b:
        a.upload(null_b)
        b.upload(zero_b)
        ha, hb = a.run(2), b.run(2)
        oa = a.download(fine_flux=True, fine_source=True, psi_f=True, psi_b=True)
        ob = b.download(fine_flux=True, fine_source=True, psi_f=True, psi_b=True)
    assert not oa["psi_b"].any()
    assert abs(ha[-1][0] - hb[-1][0]) <= 1e-5 * abs(hb[-1][0])
    for k in ("fine_flux", "fine_source", "psi_f"):
        assert rel_err(oa[k], ob[k]) <= 1e-5, k
