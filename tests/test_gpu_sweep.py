"""GPU parity tests: the CUDA path (through the C ABI) against the oracle and
the reference's golden fixtures.

Tolerances:
  * psi after one sweep from identical inputs: bit-identical (PLAIN mode
    reproduces every float operation of the reference's attenuate_fluxes).
  * fine_flux: FP32 atomic tallies add in a different order than the serial
    reference, so they agree to rounding: normwise relative error <= 1e-5.
  * k_eff: the device sums in FP64, the reference in FP32 pairwise:
    relative error <= 1e-5.
  * FP64 mode vs the FP64 oracle: <= 1e-11 (order of additions only).
  * MIXED vs FP64 (the accuracy contract of the fast mode): FSR flux
    normwise relative error <= 1e-5, k_eff relative error <= 1e-6.
"""
import numpy as np
import pytest

import oracle
from tests._util import GOLDEN_CASES, elem_rel_err, load_golden, rel_err

pytestmark = pytest.mark.gpu

PHI_TOL = 1e-5
KEFF_TOL = 1e-5


def _solver(hp, mode="plain", **kw):
    import simplemoc_gb300 as sm
    return sm.Solver(hp, mode=mode, **kw)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_plain_sweep_matches_reference_golden(gpu_available, name):
    hp, z = load_golden(name)
    with _solver(hp) as s:
        n = s.transport_sweep()
        out = s.download(psi_f=True, fine_flux=True)
    assert n == hp.spec.n_tracks_3d * hp.spec.n_seg
    assert np.array_equal(out["psi_f"], z["sweep1_psi_f"])
    assert rel_err(out["fine_flux"], z["sweep1_fine_flux"]) <= PHI_TOL


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_plain_power_iterations_match_reference_golden(gpu_available, name):
    hp, z = load_golden(name)
    iters = int(z["iters"])
    with _solver(hp) as s:
        keff = 1.0
        hist = []
        for _ in range(iters):
            s.transport_sweep()
            s.renormalize_flux()
            res = s.update_sources(keff)
            keff = s.compute_keff(0.0)
            hist.append((keff, res))
        out = s.download(psi_f=True, psi_b=True)
    h = np.asarray(hist)
    np.testing.assert_allclose(h[:, 0], z["hist"][:, 0], rtol=KEFF_TOL)
    for k in ("fine_flux", "fine_source", "psi_f"):
        assert rel_err(out[k], z[f"final_{k}"]) <= PHI_TOL, k


def _spec(**kw):
    import simplemoc_gb300 as sm
    base = dict(n_groups=100, fai=5, cai=4, height=200.0, n_sources=400, n_tracks_2d=64,
                n_polar=4, z_stacked=30, n_seg=50, seed=77)
    base.update(kw)
    return sm.ProblemSpec(**base)


# (10, 5): chunks of two groups, 10 lanes x 5 chunks = 100 groups, three tracks a warp;
# (10, 1): one chunk of four groups, 10 lanes = 40 groups, three tracks a warp
SHAPES = [(32, 1), (32, 2), (32, 4), (16, 1), (16, 2), (8, 1), (8, 4), (4, 2), (10, 5), (10, 1)]


@pytest.mark.parametrize("groups,axial_exp", [(100, 2), (7, 2), (32, 2), (20, 2), (98, 2),
                                              (40, 2), (37, 2), (1, 2), (2, 2), (3, 2),
                                              (100, 0), (37, 0), (3, 0)])
def test_plain_every_launch_shape_bit_exact(gpu_available, port, groups, axial_exp):
    """PLAIN psi equals the oracle's to the bit at every launch shape that covers
    G, quadratic and flat source, G from 1 to 100 (pairs of groups, half-padded
    where G is odd)."""
    import simplemoc_gb300 as sm
    spec = _spec(n_groups=groups, n_tracks_2d=16, z_stacked=10, axial_exp=axial_exp)
    hp = sm.generate(spec)
    st = oracle.fresh_state(hp)
    op = oracle.make_problem(hp)
    port.sweep(op, st["fine_source"], st["fine_flux"], st["psi_f"])
    ldg = (groups + 3) // 4 * 4
    ran = 0
    for tpw, cpl in SHAPES:
        vw = 2 if (tpw, cpl) == (10, 5) else 4         # chunk width: groups per lane chunk
        if tpw * cpl * vw < ldg:
            continue
        with _solver(hp) as s:
            s.set_launch(tpw, cpl)
            s.transport_sweep()
            out = s.download(psi_f=True, fine_flux=True)
        assert np.array_equal(out["psi_f"], st["psi_f"]), (tpw, cpl)
        assert rel_err(out["fine_flux"], st["fine_flux"]) <= PHI_TOL, (tpw, cpl)
        ran += 1
    assert ran >= 1


@pytest.mark.parametrize("groups,axial_exp", [(100, 2), (7, 2), (3, 2), (40, 2), (10, 0)])
def test_mixed_every_launch_shape_identical(gpu_available, groups, axial_exp):
    """MIXED runs the same operations per group at every launch shape (groups in
    packed pairs, a pair half-padded where G is odd), so psi is the same to the
    bit at every shape that covers G."""
    import simplemoc_gb300 as sm
    spec = _spec(n_groups=groups, n_tracks_2d=16, z_stacked=10, axial_exp=axial_exp)
    hp = sm.generate(spec)
    ldg = (groups + 3) // 4 * 4
    first = None
    ran = 0
    for tpw, cpl in SHAPES:
        vw = 2 if (tpw, cpl) == (10, 5) else 4
        if tpw * cpl * vw < ldg:
            continue
        with _solver(hp, mode="mixed") as s:
            s.set_launch(tpw, cpl)
            s.transport_sweep()
            out = s.download(psi_f=True, fine_flux=True)
        if first is None:
            first = out
        else:
            assert np.array_equal(out["psi_f"], first["psi_f"]), (tpw, cpl)
            assert rel_err(out["fine_flux"], first["fine_flux"]) <= PHI_TOL, (tpw, cpl)
        ran += 1
    assert ran >= 2


STAGED_SHAPES = [(32, 1), (32, 2), (16, 1), (16, 2), (8, 1)]


@pytest.mark.parametrize("groups,axial_exp", [(100, 2), (7, 2), (32, 0), (20, 2), (64, 0)])
def test_staged_pipeline_bit_exact(gpu_available, port, groups, axial_exp):
    """The 4-stage shared-memory ring (bulk copies): PLAIN psi equals the
    oracle's bit for bit in every shape; MIXED psi equals the register
    pipeline's (the same arithmetic on the same rows)."""
    import simplemoc_gb300 as sm
    spec = _spec(n_groups=groups, n_tracks_2d=16, z_stacked=10, axial_exp=axial_exp)
    hp = sm.generate(spec)
    st = oracle.fresh_state(hp)
    op = oracle.make_problem(hp)
    port.sweep(op, st["fine_source"], st["fine_flux"], st["psi_f"])
    ldg = (groups + 3) // 4 * 4
    ran = 0
    for tpw, cpl in STAGED_SHAPES:
        if tpw * cpl * 4 < ldg:
            continue
        with _solver(hp) as s:
            s.set_launch(tpw, cpl)
            s.set_pipeline(4)
            s.transport_sweep()
            out = s.download(psi_f=True, fine_flux=True)
        assert np.array_equal(out["psi_f"], st["psi_f"]), (tpw, cpl)
        assert rel_err(out["fine_flux"], st["fine_flux"]) <= PHI_TOL, (tpw, cpl)
        psis = []
        for stages in (0, 4):
            with _solver(hp, mode="mixed") as s:
                s.set_launch(tpw, cpl)
                s.set_pipeline(stages)
                s.transport_sweep()
                psis.append(s.download(psi_f=True, fine_flux=False, fine_source=False)["psi_f"])
        assert np.array_equal(psis[0], psis[1]), (tpw, cpl)
        ran += 1
    assert ran >= 1


def test_staged_pipeline_power_iterations(gpu_available, port):
    """Ten PLAIN power iterations through the staged sweep against the oracle,
    several tracks per block and ragged track counts (13 x 3 x 7 tracks)."""
    import simplemoc_gb300 as sm
    spec = _spec(n_tracks_2d=13, n_polar=6, z_stacked=7, n_groups=40)
    hp = sm.generate(spec)
    st = oracle.fresh_state(hp)
    ref_hist = port.iterate(hp, st, 10, threads=8)
    with _solver(hp) as s:
        s.set_pipeline(4)
        hist = s.run(10)
        out = s.download(psi_f=True, psi_b=True)
    assert abs(hist[-1][0] - ref_hist[-1][0]) <= KEFF_TOL * abs(ref_hist[-1][0])
    assert rel_err(out["psi_f"], st["psi_f"]) <= PHI_TOL


@pytest.mark.parametrize("axial_exp", [2, 0])
def test_plain_ten_power_iterations_vs_oracle(gpu_available, port, axial_exp):
    import simplemoc_gb300 as sm
    spec = _spec(axial_exp=axial_exp)
    hp = sm.generate(spec)
    st = oracle.fresh_state(hp)
    ref_hist = port.iterate(hp, st, 10, threads=8)
    with _solver(hp) as s:
        hist = s.run(10)
        out = s.download(psi_f=True, psi_b=True)
    np.testing.assert_allclose(np.asarray(hist)[:, 0], np.asarray(ref_hist)[:, 0],
                               rtol=KEFF_TOL)
    for k in ("fine_flux", "fine_source", "psi_f", "psi_b"):
        assert rel_err(out[k], st[k]) <= PHI_TOL, k


def test_power_iteration_equals_separate_calls(gpu_available):
    """moc_power_iteration (fused update + keff) and the four separate calls
    give the same results; two sweeps differ only in the order of their FP32
    tally additions, so the comparison is to rounding."""
    import simplemoc_gb300 as sm
    hp = sm.generate(_spec(n_tracks_2d=16, z_stacked=10))
    with _solver(hp) as a, _solver(hp) as b:
        ka, ra = a.power_iteration(1.0)
        b.transport_sweep()
        b.renormalize_flux()
        rb = b.update_sources(1.0)
        kb = b.compute_keff(0.0)
        oa, ob = a.download(), b.download()
    assert abs(ra - rb) <= 1e-6 * abs(rb)
    assert abs(ka - kb) <= 1e-7 * abs(kb)
    assert rel_err(oa["fine_flux"], ob["fine_flux"]) <= PHI_TOL
    assert rel_err(oa["fine_source"], ob["fine_source"]) <= PHI_TOL


@pytest.mark.parametrize("axial_exp", [2, 0])
def test_fp64_mode_matches_fp64_oracle(gpu_available, port, axial_exp):
    import simplemoc_gb300 as sm
    spec = _spec(n_groups=24, n_tracks_2d=16, z_stacked=10, axial_exp=axial_exp)
    hp = sm.generate(spec)
    st = oracle.fresh_state(hp, np.float64)
    ref_hist = port.iterate64(hp, st, 4)
    with _solver(hp, mode="fp64") as s:
        hist = s.run(4)
        out = s.download64(fine_flux=True, fine_source=True, psi_f=True)
    np.testing.assert_allclose(np.asarray(hist)[:, 0], np.asarray(ref_hist)[:, 0], rtol=1e-11)
    for k in ("fine_flux", "fine_source", "psi_f"):
        assert rel_err(out[k], st[k]) <= 1e-11, k


@pytest.mark.parametrize("compensated", [False, True])
def test_mixed_mode_error_vs_fp64(gpu_available, compensated):
    """The fast mode's accuracy contract, measured against the FP64 mode over
    ten power iterations of a mid-size problem."""
    import simplemoc_gb300 as sm
    spec = _spec(n_tracks_2d=128, z_stacked=40)
    hp = sm.generate(spec)
    with _solver(hp, mode="fp64") as s64:
        h64 = s64.run(10)
        o64 = s64.download64(fine_flux=True, fine_source=True)
    with _solver(hp, mode="mixed", compensated=compensated) as s:
        h = s.run(10)
        o = s.download()
    assert abs(h[-1][0] - h64[-1][0]) <= 1e-6 * abs(h64[-1][0])
    assert rel_err(o["fine_flux"], o64["fine_flux"]) <= 1e-5
    assert rel_err(o["fine_source"], o64["fine_source"]) <= 1e-5


def test_mixed_matches_oracle_fp64_small(gpu_available, port):
    import simplemoc_gb300 as sm
    spec = _spec(n_groups=40, n_tracks_2d=16, z_stacked=10)
    hp = sm.generate(spec)
    st = oracle.fresh_state(hp, np.float64)
    ref_hist = port.iterate64(hp, st, 3)
    with _solver(hp, mode="mixed") as s:
        hist = s.run(3)
        o = s.download()
    assert abs(hist[-1][0] - ref_hist[-1][0]) <= 1e-6 * abs(ref_hist[-1][0])
    assert rel_err(o["fine_flux"], st["fine_flux"]) <= 1e-5
    assert elem_rel_err(o["fine_flux"], st["fine_flux"], 1e-2) <= 1e-4


def test_full_small_problem_track_sample_bit_exact(gpu_available, port):
    """The small problem at full size (1.2 M tracks, 6.1e9 integrations): the
    angular flux of a random sample of tracks equals the oracle's bit for bit."""
    import simplemoc_gb300 as sm
    hp = sm.generate(sm.CONFIG_SMALL)
    with _solver(hp) as s:
        s.transport_sweep()
        out = s.download(psi_f=True, fine_flux=True, fine_source=False)
    rng = np.random.default_rng(0)
    tracks = np.sort(rng.choice(hp.spec.n_tracks_3d, 3000, replace=False))
    psi0 = np.zeros(hp.spec.n_tracks_3d * hp.spec.n_groups, dtype=np.float32)
    op = oracle.make_problem(hp)
    ref = port.sweep_tracks(op, hp.fine_source, tracks, psi0)
    G = hp.spec.n_groups
    got = out["psi_f"].reshape(-1, G)[tracks].ravel()
    assert np.array_equal(got, ref)
    assert np.isfinite(out["fine_flux"]).all()
    assert np.abs(out["fine_flux"]).max() > 0


@pytest.mark.parametrize("config", ["default", "flat"])
def test_default_problem_track_sample_bit_exact(gpu_available, port, config):
    """The default problem at full size (13.1 M tracks, 6.55e10 integrations,
    2.5 M FSRs), quadratic and flat source: after one PLAIN sweep the angular
    flux of a random sample of tracks equals the oracle's bit for bit (each
    track's psi depends only on its own segments and the source storage)."""
    import simplemoc_gb300 as sm
    spec = sm.CONFIGS[config]
    hp = sm.generate(spec)
    with _solver(hp) as s:
        s.transport_sweep()
        out = s.download(psi_f=True, fine_flux=False, fine_source=False)
    rng = np.random.default_rng(1)
    tracks = np.sort(rng.choice(spec.n_tracks_3d, 2000, replace=False))
    psi0 = np.zeros(spec.n_tracks_3d * spec.n_groups, dtype=np.float32)
    ref = port.sweep_tracks(oracle.make_problem(hp), hp.fine_source, tracks, psi0)
    got = out["psi_f"].reshape(-1, spec.n_groups)[tracks].ravel()
    assert np.array_equal(got, ref)


def test_full_small_problem_fluxes_vs_parallel_oracle(gpu_available, port):
    """The small problem at full size: every FSR flux after one sweep agrees
    with the oracle's OpenMP sweep of all 1.2 M tracks (normwise 1e-5)."""
    import simplemoc_gb300 as sm
    hp = sm.generate(sm.CONFIG_SMALL)
    st = oracle.fresh_state(hp)
    op = oracle.make_problem(hp)
    port.sweep_omp(op, st["fine_source"], st["fine_flux"], st["psi_f"], 0)
    with _solver(hp) as s:
        s.transport_sweep()
        out = s.download(psi_f=True, fine_flux=True, fine_source=False)
    assert np.array_equal(out["psi_f"], st["psi_f"])
    assert rel_err(out["fine_flux"], st["fine_flux"]) <= PHI_TOL
