"""Deterministic-order tallies (MOC_FLAG_DETERMINISTIC).

The FSR fluxes of a PLAIN sweep in this mode equal the serial reference's bit
for bit: the golden fixtures' scalar flux after one sweep (made by the
reference's own compiled solver), and the oracle's serial sweep on a problem
large enough for several record chunks.  In MIXED the mode makes the fluxes
the same in every run.  Reference tally order: src/solver.c:212-228.
"""
import numpy as np
import pytest

import oracle
from tests._util import GOLDEN_CASES, load_golden, rel_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_plain_flux_bit_exact_to_reference_golden(gpu_available, name):
    import simplemoc_gb300 as sm
    hp, z = load_golden(name)
    with sm.Solver(hp, mode="plain", deterministic=True) as s:
        s.transport_sweep()
        out = s.download(fine_flux=True, fine_source=False, psi_f=True)
    assert np.array_equal(out["psi_f"], z["sweep1_psi_f"])
    assert np.array_equal(out["fine_flux"], z["sweep1_fine_flux"])


def test_plain_flux_bit_exact_to_serial_oracle_over_chunks(gpu_available, port):
    """200 2D tracks of the small problem's shape (1.2e9 integrations): the
    records take three chunks of whole 2D tracks; two sweeps in a row (the flux
    accumulates across sweeps) equal the oracle's serial sweeps bit for bit."""
    import simplemoc_gb300 as sm
    hp = sm.generate(sm.CONFIG_SMALL.with_(n_tracks_2d=200))
    st = oracle.fresh_state(hp)
    op = oracle.make_problem(hp)
    with sm.Solver(hp, mode="plain", deterministic=True) as s:
        for _ in range(2):
            s.transport_sweep()
            port.sweep(op, st["fine_source"], st["fine_flux"], st["psi_f"])
        out = s.download(fine_flux=True, fine_source=False, psi_f=True)
    assert np.array_equal(out["psi_f"], st["psi_f"])
    assert np.array_equal(out["fine_flux"], st["fine_flux"])


@pytest.mark.parametrize("axial_exp", [2, 0])
def test_mixed_runs_are_identical(gpu_available, axial_exp):
    """Two handles, three MIXED power iterations each: the same bits, and
    within the tally-order tolerance of the regular (unordered) MIXED sweep."""
    import simplemoc_gb300 as sm
    spec = sm.ProblemSpec(n_groups=40, fai=5, cai=4, height=200.0, n_sources=300,
                          n_tracks_2d=24, n_polar=4, z_stacked=16, n_seg=50, seed=4040,
                          axial_exp=axial_exp)
    hp = sm.generate(spec)
    outs, hists = [], []
    for _ in range(2):
        with sm.Solver(hp, mode="mixed", deterministic=True) as s:
            hists.append(s.run(3))
            outs.append(s.download(fine_flux=True, fine_source=True, psi_f=True))
    assert hists[0] == hists[1]
    for k in ("fine_flux", "fine_source", "psi_f"):
        assert np.array_equal(outs[0][k], outs[1][k]), k
    with sm.Solver(hp, mode="mixed") as s:
        h = s.run(3)
        o = s.download(fine_flux=True, fine_source=True, psi_f=True)
    # k_eff is a ratio of sums of the fluxes: the same tally-order tolerance
    assert abs(h[-1][0] - hists[0][-1][0]) <= 1e-5 * abs(h[-1][0])
    for k in ("fine_flux", "fine_source", "psi_f"):
        assert rel_err(outs[0][k], o[k]) <= 1e-5, k


def test_deterministic_mode_rejects_what_it_does_not_cover(gpu_available):
    import simplemoc_gb300 as sm
    hp = sm.generate(sm.ProblemSpec(n_groups=8, fai=3, cai=2, height=60.0, n_sources=20,
                                    n_tracks_2d=4, n_polar=2, z_stacked=4, n_seg=10, seed=3))
    with sm.Solver(hp) as s:
        with pytest.raises(sm.MocError):
            s.set_mode("fp64", deterministic=True)
        with pytest.raises(sm.MocError):
            s.set_mode("mixed", compensated=True, deterministic=True)
        s.set_mode("plain", deterministic=True)
        s.transport_sweep()
        s.synchronize()
