"""GPU tests of the reference-ABI drop-in: transport_sweep / renormalize_flux /
update_sources / compute_keff with the reference's own structs (Params,
Input, CommGrid) against the oracle's restatement of the reference traversal,
which the CPU tests pin to the reference's own transport_sweep.

Tolerances as in test_gpu_sweep: psi, stacked-ray heights and sub-segment
counts bit-identical; fluxes normwise <= 1e-5 (tally order); k_eff <= 1e-5.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from tests._util import rel_err

pytestmark = pytest.mark.gpu

LIBC = C.CDLL(None)


def _problem(axial_exp=2, seed=11, n2d=8, n_polar=4, sep=0.5, height=40.0, groups=24, spt=30):
    import simplemoc_gb300 as sm
    from simplemoc_gb300 import refabi
    z = int(height / sep)
    spec = sm.ProblemSpec(n_groups=groups, fai=5, cai=4, height=height, n_sources=80,
                          n_tracks_2d=n2d, n_polar=n_polar, z_stacked=z, n_seg=10,
                          axial_exp=axial_exp, seed=seed)
    hp = sm.generate(spec)
    geo = refabi.make_geometry(seed + 1, n2d, n_polar, z, spt, sep)
    return hp, geo


@pytest.fixture()
def ref_lib(gpu_available):
    from simplemoc_gb300 import refabi
    lb = refabi.lib()
    lb.moc_ref_finalize()
    lb.moc_ref_set_rng(refabi.RNG_LIBC, 0)
    yield lb
    lb.moc_ref_finalize()


@pytest.mark.parametrize("axial_exp,n_polar,sep", [(2, 4, 0.5), (0, 4, 0.5), (2, 6, 0.25)])
def test_dropin_transport_sweep_matches_reference_traversal(ref_lib, port, axial_exp, n_polar,
                                                            sep):
    from simplemoc_gb300 import refabi
    hp, geo = _problem(axial_exp=axial_exp, n_polar=n_polar, sep=sep)
    rp = refabi.build(hp, geo)
    rg = oracle.make_refgeo(geo)
    op = oracle.make_problem(hp)
    st = oracle.fresh_state(hp)
    z = geo.z_height.copy()
    for sweep in range(3):
        LIBC.srand(500 + sweep)
        ref_lib.transport_sweep(C.byref(rp.params), C.byref(rp.input))
        assert ref_lib.moc_ref_status() == 0
        LIBC.srand(500 + sweep)
        n = port.ref_sweep(op, rg, st["fine_source"], st["fine_flux"], st["psi_f"], z)
        assert rp.input.segments_processed == n == ref_lib.moc_ref_last_segments()
        assert ref_lib.moc_ref_sync_to_host(C.byref(rp.params), C.byref(rp.input)) == 0
        assert np.array_equal(rp.z_heights(), z)
        assert np.array_equal(rp.psi_f, st["psi_f"])
        assert rel_err(rp.fine_flux, st["fine_flux"]) <= 1e-5


def test_dropin_power_iterations_match_oracle(ref_lib, port):
    """src/main.c:57-92 through the four reference symbols."""
    from simplemoc_gb300 import refabi
    hp, geo = _problem(seed=21)
    rp = refabi.build(hp, geo)
    rg = oracle.make_refgeo(geo)
    op = oracle.make_problem(hp)
    st = oracle.fresh_state(hp)
    z = geo.z_height.copy()
    grid = refabi.CommGrid()
    keff_d = keff_o = 1.0
    for it in range(3):
        LIBC.srand(900 + it)
        ref_lib.transport_sweep(C.byref(rp.params), C.byref(rp.input))
        ref_lib.renormalize_flux(rp.params, rp.input, grid)
        res_d = ref_lib.update_sources(rp.params, rp.input, keff_d)
        keff_d = ref_lib.compute_keff(rp.params, rp.input, grid)
        assert ref_lib.moc_ref_status() == 0
        LIBC.srand(900 + it)
        port.ref_sweep(op, rg, st["fine_source"], st["fine_flux"], st["psi_f"], z)
        port.renormalize(op, st["fine_flux"], st["psi_f"], st["psi_b"])
        res_o = port.update_sources(op, st["fine_flux"], st["fine_source"], keff_o)
        keff_o = port.compute_keff(op, st["fine_flux"], 0.0)
        assert abs(keff_d - keff_o) <= 1e-5 * abs(keff_o)
        # the residual divides by old^2 and is dominated by near-zero sources, so
        # tally-order noise is amplified; it is a diagnostic (src/main.c:81 drops it)
        if np.isfinite(res_o):
            assert abs(res_d - res_o) <= 1e-3 * abs(res_o)
    assert ref_lib.moc_ref_sync_to_host(C.byref(rp.params), C.byref(rp.input)) == 0
    for k in ("fine_flux", "fine_source", "psi_f"):
        assert rel_err(getattr(rp, k), st[k]) <= 1e-5, k


def test_dropin_hash_rng_keeps_the_geometry(ref_lib, port):
    """The counter-hash source picks change only which regions are hit: the
    sub-segment count and the stacked-ray heights equal the libc run's."""
    from simplemoc_gb300 import refabi
    hp, geo = _problem(seed=31)
    rp = refabi.build(hp, geo)
    rg = oracle.make_refgeo(geo)
    op = oracle.make_problem(hp)
    st = oracle.fresh_state(hp)
    z = geo.z_height.copy()
    ref_lib.moc_ref_set_rng(refabi.RNG_HASH, 1234)
    ref_lib.transport_sweep(C.byref(rp.params), C.byref(rp.input))
    assert ref_lib.moc_ref_status() == 0
    LIBC.srand(1)
    n = port.ref_sweep(op, rg, st["fine_source"], st["fine_flux"], st["psi_f"], z)
    assert rp.input.segments_processed == n
    assert ref_lib.moc_ref_sync_to_host(C.byref(rp.params), C.byref(rp.input)) == 0
    assert np.array_equal(rp.z_heights(), z)
    assert np.isfinite(rp.fine_flux).all() and np.abs(rp.fine_flux).max() > 0


def test_dropin_reports_bad_axial_order_without_exiting(ref_lib):
    """The reference exits on axial_exp not in {0, 2} (src/solver.c:506-511);
    the library reports MOC_ERR_ARG and leaves the inputs alone."""
    from simplemoc_gb300 import refabi
    hp, geo = _problem(seed=41)
    rp = refabi.build(hp, geo)
    rp.input.axial_exp = 1
    rp.input.segments_processed = -7
    ref_lib.transport_sweep(C.byref(rp.params), C.byref(rp.input))
    assert ref_lib.moc_ref_status() == 1
    assert rp.input.segments_processed == -7


def test_dropin_sweep_of_an_openmoc_track_file(ref_lib, port, tmp_path):
    """A track file (src/tracks.c:170-323) read by the library's reader and
    swept by the drop-in traversal equals the oracle's traversal of the same
    2D tracks: psi, heights and sub-segment counts bit for bit."""
    import simplemoc_gb300 as sm
    from simplemoc_gb300 import openmoc, refabi
    t, len64 = openmoc.synthetic(12, n_azimuthal=4, tracks_per_angle=2, segments_per_track=30)
    path = tmp_path / "tracks.bin"
    openmoc.write(path, t, seg_len64=len64)
    tr = openmoc.read(path)
    height, sep, n_polar = 40.0, 0.5, 4
    z_stacked = int(height / sep)
    spec = sm.ProblemSpec(n_groups=24, fai=5, cai=4, height=height, n_sources=80,
                          n_tracks_2d=tr.n_tracks_2d, n_polar=n_polar, z_stacked=z_stacked,
                          n_seg=10, seed=41)
    hp = sm.generate(spec)
    geo = openmoc.to_geometry(tr, n_polar, z_stacked, sep, seed=5)
    rp = refabi.build(hp, geo)
    rg = oracle.make_refgeo(geo)
    op = oracle.make_problem(hp)
    st = oracle.fresh_state(hp)
    z = geo.z_height.copy()
    for sweep in range(2):
        LIBC.srand(70 + sweep)
        ref_lib.transport_sweep(C.byref(rp.params), C.byref(rp.input))
        assert ref_lib.moc_ref_status() == 0
        LIBC.srand(70 + sweep)
        n = port.ref_sweep(op, rg, st["fine_source"], st["fine_flux"], st["psi_f"], z)
        assert rp.input.segments_processed == n
        assert ref_lib.moc_ref_sync_to_host(C.byref(rp.params), C.byref(rp.input)) == 0
        assert np.array_equal(rp.z_heights(), z)
        assert np.array_equal(rp.psi_f, st["psi_f"])
        assert rel_err(rp.fine_flux, st["fine_flux"]) <= 1e-5
