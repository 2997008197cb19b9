"""The allocation-free renormalize_flux entry point (moc_renormalize_flux_noalloc).

It exists for callers that cannot let the library call cudaMalloc -- a
framework or pool allocator that must account for every device byte, a
real-time loop that allocates nothing after start-up, or buffers mapped in
from another process.  Such a caller owns every buffer; the entry point's only
scratch is a fixed static device array.  These tests drive it through the C ABI
on caller-owned device buffers (allocated here by the test, never by the
library) and compare it with the existing moc_renormalize_flux, and with the
oracle's renormalize_flux, on two calls in a row.  This file is collected last
so that a run stopping at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from tests._util import rel_err

PHI_TOL = 1e-5          # the FSR-flux tolerance of the other GPU parity tests


def test_noalloc_rejects_sizes_beyond_its_scratch(lib):
    """More source regions than the static scratch holds, element counts that
    overflow, or missing buffers: MOC_ERR_ARG, checked before any device call."""
    fn = lib.moc_renormalize_flux_noalloc
    dummy = C.c_void_p(256)
    too_many = (1 << 20) + 1            # MOC_NOALLOC_MAX_SOURCES + 1
    rc = fn(dummy, dummy, dummy, dummy, dummy, dummy, too_many, 5, 100, 10, None, None)
    assert rc == 1
    rc = fn(None, dummy, dummy, dummy, dummy, dummy, 10, 5, 100, 10, None, None)
    assert rc == 1
    # tracks but no angular-flux buffers
    rc = fn(dummy, None, dummy, dummy, dummy, dummy, 10, 5, 100, 10, None, None)
    assert rc == 1
    # 2^20 sources x 2^30 fine intervals x 2^30 groups, and 2^62 tracks:
    # beyond 2^50 elements, rejected before any count is formed
    rc = fn(dummy, dummy, dummy, dummy, dummy, dummy, 1 << 20, 1 << 30, 1 << 30, 10, None, None)
    assert rc == 1
    rc = fn(dummy, dummy, dummy, dummy, dummy, dummy, 10, 5, 100, 1 << 62, None, None)
    assert rc == 1


def _case(n_groups, fai, n_sources, seed):
    import simplemoc_gb300 as sm
    return sm.ProblemSpec(n_groups=n_groups, fai=fai, cai=4, height=200.0, n_sources=n_sources,
                          n_tracks_2d=32, n_polar=4, z_stacked=12, n_seg=50, seed=seed)


@pytest.mark.gpu
@pytest.mark.parametrize("n_groups,fai", [(100, 5), (7, 3)])
def test_noalloc_matches_existing_entry_point_two_calls(gpu_available, lib, port, n_groups,
                                                        fai):
    """Two calls in a row on caller-owned buffers equal two calls of
    moc_renormalize_flux and two of the oracle's renormalize_flux.  G = 7 has
    rows that are not a multiple of 16 bytes.  psi_b starts non-zero (a copy of
    the swept psi_f), so its rescaling is checked too."""
    import torch

    import simplemoc_gb300 as sm
    spec = _case(n_groups, fai, 300, 515 + n_groups)
    hp = sm.generate(spec)
    with sm.Solver(hp) as s:
        s.transport_sweep()
        swept = s.download(fine_flux=True, fine_source=False, psi_f=True)
    # the state before renormalisation, psi_b non-zero
    hp.fine_flux[:] = swept["fine_flux"]
    hp.psi_f[:] = swept["psi_f"]
    hp.psi_b[:] = swept["psi_f"][::-1]
    assert np.abs(hp.psi_b).max() > 0
    before = {k: getattr(hp, k).copy() for k in ("fine_flux", "psi_f", "psi_b")}
    expected = []
    with sm.Solver(hp) as s:
        for _ in range(2):
            s.renormalize_flux()
            expected.append(s.download(fine_flux=True, fine_source=False, psi_f=True,
                                       psi_b=True))
    op = oracle.make_problem(hp)
    ost = {k: v.copy() for k, v in before.items()}
    oracle_out = []
    for _ in range(2):
        port.renormalize(op, ost["fine_flux"], ost["psi_f"], ost["psi_b"])
        oracle_out.append({k: v.copy() for k, v in ost.items()})

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    phi = torch.from_numpy(before["fine_flux"].copy()).to(dev)
    psi_f = torch.from_numpy(before["psi_f"].copy()).to(dev)
    psi_b = torch.from_numpy(before["psi_b"].copy()).to(dev)
    vol = torch.from_numpy(hp.vol).to(dev)
    src_xs = torch.from_numpy(hp.src_xs).to(dev)
    xs = torch.from_numpy(hp.xs).to(dev)
    norm = torch.zeros(2, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    fn = lib.moc_renormalize_flux_noalloc

    def call():
        rc = fn(phi.data_ptr(), psi_f.data_ptr(), psi_b.data_ptr(), vol.data_ptr(),
                src_xs.data_ptr(), xs.data_ptr(), spec.n_sources, spec.fai, spec.n_groups,
                spec.n_tracks_3d, norm.data_ptr(), stream)
        assert rc == 0
        torch.cuda.synchronize(dev)

    for want, ref in zip(expected, oracle_out):
        call()
        for k in ("fine_flux", "psi_f", "psi_b"):
            got = {"fine_flux": phi, "psi_f": psi_f, "psi_b": psi_b}[k].cpu().numpy()
            assert rel_err(got, want[k]) <= PHI_TOL, k
            assert rel_err(got, ref[k]) <= PHI_TOL, k
        total, nf = norm.cpu().numpy()
        assert total > 0 and nf == np.float64(np.float32(1.0 / total))


@pytest.mark.gpu
def test_noalloc_without_tracks_takes_null_angular_flux(gpu_available, lib):
    """With no tracks the angular-flux buffers may be NULL: only the scalar
    flux is renormalised, as by the handle's entry point."""
    import torch

    import simplemoc_gb300 as sm
    spec = _case(7, 3, 40, 616)
    hp = sm.generate(spec)
    with sm.Solver(hp) as s:
        s.transport_sweep()
        swept = s.download(fine_flux=True, fine_source=False, psi_f=False)
        s.renormalize_flux()
        want = s.download(fine_flux=True, fine_source=False, psi_f=False)
    dev = torch.device("cuda", 0)
    phi = torch.from_numpy(swept["fine_flux"].copy()).to(dev)
    vol = torch.from_numpy(hp.vol).to(dev)
    src_xs = torch.from_numpy(hp.src_xs).to(dev)
    xs = torch.from_numpy(hp.xs).to(dev)
    rc = lib.moc_renormalize_flux_noalloc(phi.data_ptr(), None, None, vol.data_ptr(),
                                          src_xs.data_ptr(), xs.data_ptr(), spec.n_sources,
                                          spec.fai, spec.n_groups, 0, None,
                                          torch.cuda.current_stream(dev).cuda_stream)
    assert rc == 0
    torch.cuda.synchronize(dev)
    assert rel_err(phi.cpu().numpy(), want["fine_flux"]) <= PHI_TOL
