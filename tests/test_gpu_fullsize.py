"""Parity and accuracy at the full sizes of the small and default problems.

* The small problem (2x2 assemblies, 1.2 M tracks, 100 groups): ten PLAIN power
  iterations against the oracle's OpenMP power iteration (src/main.c:57-92,
  src/solver.c:1143-1437), and the MIXED accuracy contract against the FP64
  mode over 20 power iterations, per FSR and per element.
* The default problem (17x17 assemblies, 13.1 M tracks, 2.5 M FSRs): one
  PLAIN sweep with the angular flux of EVERY track bit for bit and every FSR
  flux against the oracle's OpenMP sweep of all tracks.
* update_sources on the tensor cores (MIXED) directly against the oracle's
  update_sources (src/solver.c:1235-1320) on the golden fixtures' states.

Tolerances: PLAIN fluxes, sources and k_eff 1e-5 relative (FP32 tally order
only; the device sums in FP64, the reference pairwise in FP32); MIXED against
FP64: FSR flux 1e-5 per FSR and per element, k_eff 1e-6 (the accuracy
contract); tensor-core source 1e-6 normwise (split TF32, FP32 accumulation).
"""
import numpy as np
import pytest

import oracle
from tests._util import GOLDEN_CASES, load_golden, rel_err

pytestmark = pytest.mark.gpu

PHI_TOL = 1e-5
KEFF_TOL = 1e-5
CONTRACT = 1e-5
KEFF_CONTRACT = 1e-6


def _per_fsr(a, ref, G):
    """max over FSRs of max_g |a - ref| / max_g |ref| (each FSR's group vector)."""
    d = np.abs(np.asarray(a, np.float64) - ref).reshape(-1, G).max(1)
    r = np.abs(np.asarray(ref, np.float64)).reshape(-1, G).max(1)
    return float((d[r > 0] / r[r > 0]).max())


def _per_element(a, ref):
    a = np.asarray(a, np.float64)
    r = np.abs(np.asarray(ref, np.float64))
    m = r > 0
    return float((np.abs(a - ref)[m] / r[m]).max())


def test_small_problem_ten_plain_iterations_vs_openmp_oracle(gpu_available, port):
    import simplemoc_gb300 as sm
    hp = sm.generate(sm.CONFIG_SMALL)
    st = oracle.fresh_state(hp)
    ref_hist = port.iterate(hp, st, 10, threads=0)
    with sm.Solver(hp) as s:
        hist = s.run(10)
        out = s.download(psi_f=True, psi_b=True)
    np.testing.assert_allclose(np.asarray(hist)[:, 0], np.asarray(ref_hist)[:, 0],
                               rtol=KEFF_TOL)
    for k in ("fine_flux", "fine_source", "psi_f", "psi_b"):
        assert rel_err(out[k], st[k]) <= PHI_TOL, k


@pytest.mark.parametrize("compensated", [False, True])
def test_small_problem_mixed_contract_per_fsr(gpu_available, compensated):
    """The accuracy contract at full size over 20 power iterations: every FSR's
    flux within 1e-5 of the FP64 mode (per FSR and per element), k_eff 1e-6."""
    import simplemoc_gb300 as sm
    hp = sm.generate(sm.CONFIG_SMALL, with_state=False)
    G = hp.spec.n_groups
    with sm.Solver(hp, mode="fp64") as s64:
        h64 = s64.run(20)
        o64 = s64.download64(fine_flux=True, fine_source=True)
    with sm.Solver(hp, mode="mixed", compensated=compensated) as s:
        h = s.run(20)
        o = s.download(psi_f=False)
    assert abs(h[-1][0] - h64[-1][0]) <= KEFF_CONTRACT * abs(h64[-1][0])
    for k in ("fine_flux", "fine_source"):
        e_fsr = _per_fsr(o[k], o64[k], G)
        e_el = _per_element(o[k], o64[k])
        print(f"{k}: per FSR {e_fsr:.2e}, per element {e_el:.2e}")
        assert e_fsr <= CONTRACT, (k, e_fsr)
        assert e_el <= CONTRACT, (k, e_el)


def test_default_problem_one_sweep_every_track_vs_openmp_oracle(gpu_available, port):
    """13.1 M tracks x 50 segments x 100 groups: psi of every track equals the
    oracle's bit for bit; every FSR flux agrees normwise (tally order)."""
    import simplemoc_gb300 as sm
    hp = sm.generate(sm.CONFIG_DEFAULT, with_state=False)
    st = oracle.fresh_state(hp)
    del st["psi_b"]
    with sm.Solver(hp) as s:
        s.transport_sweep()
        out = s.download(fine_flux=True, fine_source=False, psi_f=True)
    port.sweep_omp(oracle.make_problem(hp), st["fine_source"], st["fine_flux"], st["psi_f"], 0)
    assert np.array_equal(out["psi_f"], st["psi_f"])
    assert rel_err(out["fine_flux"], st["fine_flux"]) <= PHI_TOL


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_tensor_core_update_vs_oracle_on_golden_states(gpu_available, port, name):
    """MIXED update_sources (split-TF32 tcgen05 contraction) on the state the
    reference reached (the fixture's final scalar flux, its initial source and
    final k_eff) against the oracle's update_sources on the same state."""
    import simplemoc_gb300 as sm
    hp, z = load_golden(name)
    keff = float(z["hist"][-1][0])
    hp = hp.copy_state()
    hp.fine_flux = z["final_fine_flux"].copy()
    q_old = hp.fine_source.copy()
    op = oracle.make_problem(hp)
    q_ref = q_old.copy()
    res_ref = port.update_sources(op, hp.fine_flux, q_ref, keff)
    with sm.Solver(hp, mode="mixed") as s:
        res = s.update_sources(keff)
        q = s.download(fine_flux=False, fine_source=True, psi_f=False)["fine_source"]
    assert rel_err(q, q_ref) <= 1e-6, rel_err(q, q_ref)
    assert abs(res - res_ref) <= 1e-5 * abs(res_ref)
