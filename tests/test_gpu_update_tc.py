"""GPU tests of update_sources on the tensor cores (MIXED mode): the split-TF32
tcgen05 contraction against the CUDA-core kernel (MOC_FLAG_SIMT_UPDATE) on the
same state, and against the FP64 mode.

Tolerances: the new fine source normwise <= 1e-6 of the CUDA-core result (both
are FP32-accurate: the split product drops only lo x lo, ~2^-22 relative);
residual and k_eff sums <= 1e-5 relative.  Group counts cover one and several
K steps, ragged last column chunks and the 104-group limit; 105 groups fall
back to the CUDA cores.  Material counts give ragged last tiles.
"""
import numpy as np
import pytest

from tests._util import rel_err

pytestmark = pytest.mark.gpu


def _problem(G, F, n_mat, seed, n_sources=230):
    import simplemoc_gb300 as sm
    spec = sm.ProblemSpec(n_groups=G, fai=F, cai=4, height=200.0, n_sources=n_sources,
                          n_materials=n_mat, n_fuel=max(1, n_mat // 2), n_tracks_2d=8,
                          n_polar=2, z_stacked=4, n_seg=20, axial_exp=2 if F >= 3 else 0,
                          seed=seed)
    hp = sm.generate(spec)
    rng = np.random.default_rng(seed)
    hp.fine_flux[:] = rng.random(hp.fine_flux.size, dtype=np.float32) + 0.01
    return hp


@pytest.mark.parametrize("G,F,n_mat", [(100, 5, 8), (40, 5, 8), (7, 3, 3), (104, 4, 5),
                                       (33, 7, 600), (1, 5, 2), (105, 5, 8)])
def test_tensor_core_update_matches_cuda_core(gpu_available, G, F, n_mat):
    import simplemoc_gb300 as sm
    hp = _problem(G, F, n_mat, seed=1000 + G)
    out = {}
    for simt in (False, True):
        with sm.Solver(hp, mode="mixed", simt_update=simt) as s:
            res = s.update_sources(1.37)
            q = s.download(fine_flux=False, fine_source=True, psi_f=False)["fine_source"]
            n0 = s.launch_count()
            k, res2 = s.power_iteration(1.21)
            out[simt] = (res, q, k, res2, s.launch_count() - n0)
    (ra, qa, ka, r2a, _), (rb, qb, kb, r2b, _) = out[False], out[True]
    assert rel_err(qa, qb) <= 1e-6, rel_err(qa, qb)
    assert abs(ra - rb) <= 1e-5 * abs(rb)
    assert abs(ka - kb) <= 1e-5 * abs(kb)
    assert abs(r2a - r2b) <= 1e-5 * abs(r2b)


def test_tensor_core_update_close_to_fp64(gpu_available):
    import simplemoc_gb300 as sm
    hp = _problem(100, 5, 8, seed=7)
    qs = {}
    for name, kw in (("tc", {}), ("simt", {"simt_update": True})):
        with sm.Solver(hp, mode="mixed", **kw) as a:
            a.update_sources(1.1)
            qs[name] = a.download(fine_flux=False, fine_source=True, psi_f=False)["fine_source"]
    with sm.Solver(hp, mode="fp64") as b:
        rb = b.update_sources(1.1)
        q64 = b.download64(fine_flux=False, fine_source=True)["fine_source"]
    e_tc = rel_err(qs["tc"].astype(np.float64), q64)
    e_simt = rel_err(qs["simt"].astype(np.float64), q64)
    print(f"new source vs FP64: tensor cores {e_tc:.2e}, CUDA cores {e_simt:.2e}")
    assert e_tc <= 1e-6, (e_tc, e_simt)
