"""CPU test of the FP64 adjoint of the oracle (oracle_adjoint64), the yardstick
the GPU reverse sweep is compared with: its gradients against central
differences of the FP64 oracle sweep itself, for a linear loss
L = sum(dphi * phi).

phi is linear in the fine source and in the incoming angular flux, so those
differences are exact up to rounding; sigma_t enters non-linearly (relative
step 1e-4, truncation error ~1e-8 relative).
"""
import numpy as np
import pytest

import oracle


def _loss(port, op, hp, q, dphi, psi_in):
    st = oracle.fresh_state(hp, np.float64)
    psi = psi_in.copy()
    port.sweep64(op, q, st["fine_flux"], psi)
    return float(dphi @ st["fine_flux"])


@pytest.mark.parametrize("axial_exp", [2, 0])
def test_oracle_adjoint_matches_central_differences(port, lib, axial_exp):
    import simplemoc_gb300 as sm
    spec = sm.ProblemSpec(n_groups=4, fai=5, cai=4, height=200.0, n_sources=30, n_tracks_2d=3,
                          n_polar=2, z_stacked=3, n_seg=20, axial_exp=axial_exp, seed=77)
    hp = sm.generate(spec)
    op = oracle.make_problem(hp)
    G = spec.n_groups
    rng = np.random.default_rng(5)
    q = hp.fine_source.astype(np.float64)
    dphi = rng.random(spec.n_fsr * G)
    psi_in = rng.random(spec.n_tracks_3d * G)
    dq, dsig, dpsi = port.adjoint64(op, q, dphi, psi_in)

    errs = []
    for k in rng.choice(q.size, 12, replace=False):
        d = 1e-3 * max(abs(q[k]), 1e-3)
        qp, qm = q.copy(), q.copy()
        qp[k] += d
        qm[k] -= d
        fd = (_loss(port, op, hp, qp, dphi, psi_in) - _loss(port, op, hp, qm, dphi, psi_in)) / (2 * d)
        errs.append(abs(dq[k] - fd) / max(abs(fd), 1e-12 * np.abs(dq).max()))
    for k in rng.choice(psi_in.size, 8, replace=False):
        d = 1e-3
        pp, pm = psi_in.copy(), psi_in.copy()
        pp[k] += d
        pm[k] -= d
        fd = (_loss(port, op, hp, q, dphi, pp) - _loss(port, op, hp, q, dphi, pm)) / (2 * d)
        errs.append(abs(dpsi[k] - fd) / max(abs(fd), 1e-12))
    # sigma_t rows that some source uses; the oracle reads hp.sigt in place
    used = np.unique(hp.src_sigt)
    sig = hp.sigt.reshape(-1, G)
    for _ in range(8):
        m, g = int(rng.choice(used)), int(rng.integers(G))
        s0 = sig[m, g]
        sp, sm_ = np.float32(s0 * (1 + 1e-4)), np.float32(s0 * (1 - 1e-4))
        sig[m, g] = sp
        lp = _loss(port, op, hp, q, dphi, psi_in)
        sig[m, g] = sm_
        lm = _loss(port, op, hp, q, dphi, psi_in)
        sig[m, g] = s0
        fd = (lp - lm) / (float(sp) - float(sm_))
        errs.append(abs(dsig[m * G + g] - fd) / max(abs(fd), 1e-12))
    assert max(errs) <= 1e-5, errs
