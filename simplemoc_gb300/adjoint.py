"""Differentiable transport sweep for PyTorch.

`TransportSweep` is a torch.autograd.Function over the C ABI: its forward is
one fixed-source sweep on the GPU (MIXED arithmetic, tallies from zero, psi
checkpointed every k segments) and its backward is the hand-written reverse
sweep (moc_adjoint_backward), which returns dL/d fine_source and dL/d sigma_t
for whatever loss the caller builds on the scalar flux.

`UpdateSources` is a torch.autograd.Function over the library's update_sources
(src/solver.c:1235-1300) as the adjoint workload uses it: one step from a given
scalar flux phi0,
    q = (chi * (nuSigmaF . phi0) / k + S phi0) / (4 pi),
with the scatter matrices and nu*SigmaF as inputs; its backward is the
hand-written reverse of the step (moc_update_sources_adjoint): dL/dS, dL/dnuSigmaF
and dL/dphi0 per material and group.

`FixedSourceLoss` is the adjoint workload: q from UpdateSources, phi from
TransportSweep, and the loss sum over fine regions of vol * nuSigmaF * phi.
Every derivative of the solver -- sigma_t, scatter, nuSigmaF, fine source --
comes from the library's reverse kernels; only the loss's own direct
dependence on nuSigmaF is torch's.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from . import _lib as L
from .problem import HostProblem
from .solver import Solver


def _sync_torch(device: torch.device) -> None:
    torch.cuda.current_stream(device).synchronize()


class TransportSweep(torch.autograd.Function):
    """phi = sweep(q, sigma_t); q [NS*F*G] float32 CUDA, sigma_t [n_sigt, G]."""

    @staticmethod
    def forward(ctx, q: torch.Tensor, sigma_t: torch.Tensor, solver: Solver, k_ckpt: int = 8):
        lib = solver._lib
        h = solver.handle
        dev = q.device
        qc = q.detach().contiguous()
        sig = np.ascontiguousarray(sigma_t.detach().to("cpu", torch.float32).numpy().ravel())
        _sync_torch(dev)
        L.check(lib.moc_set_sigma_t(h, L.ptr(sig, C.c_float)), "moc_set_sigma_t")
        L.check(lib.moc_set_fine_source_device(h, qc.data_ptr()), "moc_set_fine_source_device")
        L.check(lib.moc_zero_state(h, 1, 1), "moc_zero_state")
        L.check(lib.moc_adjoint_forward(h, k_ckpt), "moc_adjoint_forward")
        phi = torch.empty_like(qc)
        L.check(lib.moc_get_fine_flux_device(h, phi.data_ptr()), "moc_get_fine_flux_device")
        solver.synchronize()
        ctx.solver = solver
        ctx.sig_shape = sigma_t.shape
        ctx.sig_dtype = sigma_t.dtype
        ctx.sig_device = sigma_t.device
        return phi

    @staticmethod
    def backward(ctx, dphi: torch.Tensor):
        solver = ctx.solver
        lib = solver._lib
        dphi = dphi.detach().to(torch.float32).contiguous()
        dq = torch.empty_like(dphi)
        dsig = torch.empty(int(np.prod(ctx.sig_shape)), dtype=torch.float64, device=dphi.device)
        _sync_torch(dphi.device)
        L.check(lib.moc_adjoint_backward(solver.handle, dphi.data_ptr(), dq.data_ptr(),
                                         dsig.data_ptr(), None), "moc_adjoint_backward")
        solver.synchronize()
        return (dq, dsig.reshape(ctx.sig_shape).to(ctx.sig_device, ctx.sig_dtype), None, None)


class UpdateSources(torch.autograd.Function):
    """q = update_sources(phi0; S, nuSigmaF) on the library; phi0 [NS*F*G]
    CUDA, scatter [n_xs, G, G] (row g = destination), nusf [n_xs, G].  The
    handle's other cross sections (chi, SigmaA) are the problem's."""

    @staticmethod
    def forward(ctx, phi0: torch.Tensor, scatter: torch.Tensor, nusf: torch.Tensor,
                solver: Solver, xs_base: np.ndarray, keff: float):
        lib, h = solver._lib, solver.handle
        G = solver.spec.n_groups
        n_xs = xs_base.size // (3 * G)
        xs = xs_base.reshape(n_xs, G, 3).copy()
        xs[:, :, 0] = nusf.detach().to("cpu", torch.float32).numpy()
        xs = np.ascontiguousarray(xs.ravel(), dtype=np.float32)
        sc = np.ascontiguousarray(scatter.detach().to("cpu", torch.float32).numpy().ravel())
        ph = phi0.detach().to(torch.float32).contiguous()
        _sync_torch(ph.device)
        L.check(lib.moc_set_cross_sections(h, L.ptr(xs, C.c_float), L.ptr(sc, C.c_float)),
                "moc_set_cross_sections")
        L.check(lib.moc_set_fine_flux_device(h, ph.data_ptr()), "moc_set_fine_flux_device")
        res = C.c_double()
        L.check(lib.moc_update_sources(h, keff, C.byref(res)), "moc_update_sources")
        q = torch.empty_like(ph)
        L.check(lib.moc_get_fine_source_device(h, q.data_ptr()), "moc_get_fine_source_device")
        solver.synchronize()
        ctx.save_for_backward(ph)
        ctx.solver, ctx.keff = solver, keff
        ctx.shapes = (phi0.dtype, scatter.shape, scatter.dtype, nusf.shape, nusf.dtype)
        return q

    @staticmethod
    def backward(ctx, dq: torch.Tensor):
        (ph,) = ctx.saved_tensors
        solver = ctx.solver
        phi_dtype, s_shape, s_dtype, n_shape, n_dtype = ctx.shapes
        dq = dq.detach().to(torch.float32).contiguous()
        dev = dq.device
        dS = torch.empty(int(np.prod(s_shape)), dtype=torch.float64, device=dev)
        dN = torch.empty(int(np.prod(n_shape)), dtype=torch.float64, device=dev)
        dP = torch.empty_like(ph)
        _sync_torch(dev)
        L.check(solver._lib.moc_update_sources_adjoint(solver.handle, ph.data_ptr(), dq.data_ptr(),
                                                       ctx.keff, dS.data_ptr(), dN.data_ptr(),
                                                       dP.data_ptr()),
                "moc_update_sources_adjoint")
        solver.synchronize()
        return (dP.to(phi_dtype), dS.reshape(s_shape).to(s_dtype), dN.reshape(n_shape).to(n_dtype),
                None, None, None)


def sweep(q: torch.Tensor, sigma_t: torch.Tensor, solver: Solver, k_ckpt: int = 8) -> torch.Tensor:
    return TransportSweep.apply(q, sigma_t, solver, k_ckpt)


def fit_gradients(solver: Solver, dphi: torch.Tensor) -> torch.Tensor:
    """dL/d(c0, c1, c2) of each quadratic source fit (src/solver.c:69-81) for
    dL/dphi, after a forward sweep with checkpoints (TransportSweep.forward or
    moc_adjoint_forward): [NS, F-2, 3, G], window w fitting fine rows w, w+1,
    w+2 of a source.  Quadratic source only."""
    s = solver.spec
    dphi = dphi.detach().to(torch.float32).contiguous()
    out = torch.empty((s.n_sources, s.fai - 2, 3, s.n_groups), dtype=torch.float32,
                      device=dphi.device)
    _sync_torch(dphi.device)
    L.check(solver._lib.moc_adjoint_backward_fit(solver.handle, dphi.data_ptr(), None, None, None,
                                                 out.data_ptr()), "moc_adjoint_backward_fit")
    solver.synchronize()
    return out


class FixedSourceLoss:
    """Loss of the adjoint workload as a function of (sigma_t, S, nu*SigmaF, phi0)."""

    def __init__(self, hp: HostProblem, solver: Solver, device: str = "cuda", keff: float = 1.0,
                 k_ckpt: int = 8):
        s = hp.spec
        self.hp, self.solver, self.keff, self.k = hp, solver, keff, k_ckpt
        self.G, self.F, self.NS = s.n_groups, s.fai, s.n_sources
        n_xs = hp.xs.size // (3 * self.G)
        self.dev = torch.device(device)
        xs = torch.from_numpy(hp.xs.reshape(n_xs, self.G, 3).copy())
        self.chi = xs[:, :, 2].to(self.dev)
        self.src_xs = torch.from_numpy(hp.src_xs.astype(np.int64)).to(self.dev)
        self.vol = torch.from_numpy(hp.vol.copy()).to(self.dev)

    def source(self, phi0, scatter, nusf):
        """update_sources from phi0 [NS, F, G] on the library (UpdateSources):
        q [NS*F*G] float32."""
        return UpdateSources.apply(phi0.reshape(-1), scatter, nusf, self.solver, self.hp.xs,
                                   self.keff)

    def source_reference(self, phi0, scatter, nusf):
        """The same step in torch, in the precision of its inputs: a yardstick
        for the library's step and its reverse (src/solver.c:1266-1290)."""
        Sm = scatter[self.src_xs]                      # [NS, G, G], row g = destination
        nf = nusf[self.src_xs]                         # [NS, G]
        fission = torch.einsum("sfg,sg->sf", phi0, nf) / self.keff
        scat = torch.einsum("sgh,sfh->sfg", Sm, phi0)
        return (fission[:, :, None] * self.chi[self.src_xs][:, None, :] + scat) / (4.0 * math.pi)

    def loss_of_flux(self, phi, nusf):
        """sum over fine regions of vol * nuSigmaF * phi."""
        w = self.vol[:, None, None] * nusf[self.src_xs][:, None, :]
        return (w * phi.reshape(self.NS, self.F, self.G)).sum()

    def __call__(self, sigma_t, scatter, nusf, phi0):
        q = self.source(phi0, scatter, nusf)
        phi = sweep(q, sigma_t, self.solver, self.k)
        return self.loss_of_flux(phi.to(nusf.dtype), nusf), q
