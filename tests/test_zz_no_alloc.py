"""The allocation-free renormalize_flux entry point (moc_renormalize_flux_noalloc).

It exists for callers that cannot let the library call cudaMalloc -- a
framework or pool allocator that must account for every device byte, a
real-time loop that allocates nothing after start-up, or buffers mapped in
from another process.  Such a caller owns every buffer; the entry point's only
scratch is a fixed static device array.  These tests drive it through the C ABI
on caller-owned device buffers (allocated here by the test, never by the
library) and compare it with the existing moc_renormalize_flux on two calls in
a row.  This file is collected last so that a run stopping at the first
failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from tests._util import rel_err

PHI_TOL = 1e-5          # the FSR-flux tolerance of the other GPU parity tests


def test_noalloc_rejects_sizes_beyond_its_scratch(lib):
    """More source regions than the static scratch holds: MOC_ERR_ARG, checked
    before any device call."""
    fn = lib.moc_renormalize_flux_noalloc
    dummy = C.c_void_p(256)
    too_many = (1 << 20) + 1            # MOC_NOALLOC_MAX_SOURCES + 1
    rc = fn(dummy, dummy, dummy, dummy, dummy, dummy, too_many, 5, 100, 10, None, None)
    assert rc == 1
    rc = fn(None, dummy, dummy, dummy, dummy, dummy, 10, 5, 100, 10, None, None)
    assert rc == 1


@pytest.mark.gpu
def test_noalloc_matches_existing_entry_point_two_calls(gpu_available, lib):
    import torch

    import simplemoc_gb300 as sm
    spec = sm.ProblemSpec(n_groups=100, fai=5, cai=4, height=200.0, n_sources=300,
                          n_tracks_2d=32, n_polar=4, z_stacked=12, n_seg=50, seed=515)
    hp = sm.generate(spec)
    with sm.Solver(hp) as s:
        s.transport_sweep()
        before = s.download(fine_flux=True, fine_source=False, psi_f=True, psi_b=True)
        s.renormalize_flux()
        first = s.download(fine_flux=True, fine_source=False, psi_f=True, psi_b=True)
        s.renormalize_flux()
        second = s.download(fine_flux=True, fine_source=False, psi_f=True, psi_b=True)

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

    for expected in (first, second):
        call()
        assert rel_err(phi.cpu().numpy(), expected["fine_flux"]) <= PHI_TOL
        assert rel_err(psi_f.cpu().numpy(), expected["psi_f"]) <= PHI_TOL
        np.testing.assert_array_equal(psi_b.cpu().numpy(), expected["psi_b"])
        total, nf = norm.cpu().numpy()
        assert total > 0 and nf == np.float64(np.float32(1.0 / total))
