"""GPU tests of the streamed upload (moc_upload): the per-track arrays go to
the device on a second stream in chunks of whole 2D tracks, and the next sweep
starts on each chunk once it has landed.  Every call sequence must give what
the synchronous upload at creation gives:

* psi after one sweep: bit-identical (each track's arithmetic is unchanged);
* fine_flux: FP32 atomic tallies in another order, normwise <= 1e-5;
* k_eff and the renormalised psi_b: <= 1e-5 relative.

13 2D tracks make eight uneven chunks (one or two 2D tracks each).
"""
import ctypes as C

import numpy as np
import pytest

from tests._util import rel_err

pytestmark = pytest.mark.gpu


def _problem(seed=5, state_seed=11):
    import simplemoc_gb300 as sm
    spec = sm.ProblemSpec(n_groups=22, fai=5, cai=4, height=200.0, n_sources=300,
                          n_tracks_2d=13, n_polar=4, z_stacked=10, n_seg=30, seed=seed)
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


@pytest.mark.parametrize("mode", ["plain", "mixed"])
def test_streamed_upload_then_sweep_matches_synchronous(gpu_available, mode):
    import simplemoc_gb300 as sm
    hp = _problem()
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


def test_upload_rejects_bad_source_ids(gpu_available):
    import simplemoc_gb300 as sm
    hp = _problem(seed=10)
    bad = hp.copy_state()
    bad.seg_src = hp.seg_src.copy()
    bad.seg_src[hp.seg_src.size // 2] = hp.spec.n_sources
    with sm.Solver(hp, mode="plain") as b:
        with pytest.raises(sm.MocError):
            b.upload(bad)
        # the rejected upload overwrote part of the state: work is refused ...
        with pytest.raises(sm.MocError):
            b.transport_sweep()
        # ... until a valid upload, after which the handle sweeps as a fresh one
        b.upload(hp)
        b.transport_sweep()
        out = b.download(psi_f=True, fine_flux=False, fine_source=False)
    with sm.Solver(hp, mode="plain") as a:
        a.transport_sweep()
        ref = a.download(psi_f=True, fine_flux=False, fine_source=False)
    assert np.array_equal(out["psi_f"], ref["psi_f"])
