"""GPU tests of the adjoint sweep and its torch.autograd.Function binding.

* against the FP64 CPU adjoint (oracle_adjoint64) on the same inputs:
  dL/dq and dL/dsigma_t normwise <= 1e-4 (the GPU runs the FP32 MIXED sweep);
* against central finite differences (h = 1e-3 relative) of the FP64 GPU
  sweep on 64 random parameters of the fixed-source loss -- sigma_t, scatter,
  nu*SigmaF, fine source: <= 1e-4 relative;
* the adjoint (forward with checkpoints + reverse) takes <= 3x the time of a
  plain forward sweep on the adjoint workload geometry.
"""
import ctypes as C

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _lib():
    from simplemoc_gb300 import _lib as L
    return L


def _adjoint_spec(n2d=1024, z=300, axial_exp=2, seed=20260104):
    import simplemoc_gb300 as sm
    # the small problem's geometry with 40 groups
    return sm.CONFIG_SMALL.with_(n_groups=40, n_tracks_2d=n2d, z_stacked=z, axial_exp=axial_exp,
                                 seed=seed)


# widths: automatic (3 lanes a track, 10 tracks a warp, 2 lanes idle), two
# chunks a lane, one track a warp; 600 materials put the dL/dsigma_t
# accumulators past shared memory (FP64 atomics to global memory instead)
@pytest.mark.parametrize("axial_exp,width,n_materials", [
    (2, (0, 0), 8), (0, (0, 0), 8), (2, (2, 2), 8), (0, (2, 2), 8), (2, (32, 1), 8),
    (2, (0, 0), 600)])
def test_adjoint_matches_fp64_cpu_adjoint(gpu_available, port, axial_exp, width, n_materials):
    import torch

    import simplemoc_gb300 as sm
    L = _lib()
    spec = sm.ProblemSpec(n_groups=12, fai=5, cai=4, height=200.0, n_sources=60, n_tracks_2d=12,
                          n_polar=4, z_stacked=10, n_seg=50, axial_exp=axial_exp,
                          n_materials=n_materials, seed=31)
    hp = sm.generate(spec)
    rng = np.random.default_rng(3)
    dphi = rng.random(spec.n_fsr * spec.n_groups).astype(np.float32)
    dev = torch.device("cuda", 0)
    with sm.Solver(hp) as s:
        lib, h = s._lib, s.handle
        L.check(lib.moc_set_adjoint_width(h, *width), "width")
        L.check(lib.moc_zero_state(h, 1, 1), "zero")
        L.check(lib.moc_adjoint_forward(h, 8), "fwd")
        dphi_t = torch.from_numpy(dphi).to(dev)
        dq = torch.empty_like(dphi_t)
        dsig = torch.empty(hp.sigt.size, dtype=torch.float64, device=dev)
        dpsi = torch.empty(spec.n_tracks_3d * spec.n_groups, dtype=torch.float32, device=dev)
        torch.cuda.synchronize()
        L.check(lib.moc_adjoint_backward(h, dphi_t.data_ptr(), dq.data_ptr(), dsig.data_ptr(),
                                         dpsi.data_ptr()), "bwd")
        s.synchronize()
        phi = s.download(fine_flux=True, fine_source=False, psi_f=False)["fine_flux"]
    op = oracle.make_problem(hp)
    q64 = hp.fine_source.astype(np.float64)
    st = oracle.fresh_state(hp, np.float64)
    port.sweep64(op, q64, st["fine_flux"], st["psi_f"])
    rq, rs, rp = port.adjoint64(op, q64, dphi.astype(np.float64))
    rel = lambda a, b: np.abs(a - b).max() / np.abs(b).max()
    assert rel(phi, st["fine_flux"]) <= 1e-5
    assert rel(dq.cpu().numpy(), rq) <= 1e-4
    assert rel(dsig.cpu().numpy(), rs) <= 1e-4
    assert rel(dpsi.cpu().numpy(), rp) <= 1e-4


def test_adjoint_gradients_vs_central_differences(gpu_available):
    """64 random parameters of the fixed-source loss, 16 of each kind, on the
    whole adjoint workload (1024 2D tracks, 1.2 M 3D tracks, 40 groups): every
    gradient from the library's reverse kernels (sweep and update_sources)."""
    import torch

    import simplemoc_gb300 as sm
    from simplemoc_gb300.adjoint import FixedSourceLoss
    L = _lib()
    spec = _adjoint_spec()
    hp = sm.generate(spec)
    G, n_xs = spec.n_groups, hp.xs.size // (3 * spec.n_groups)
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(17)
    phi0 = torch.from_numpy(rng.random((spec.n_sources, spec.fai, G))).to(dev)
    sig0 = torch.from_numpy(hp.sigt.reshape(-1, G).copy())
    S0 = torch.from_numpy(hp.scatter.reshape(n_xs, G, G).astype(np.float64)).to(dev)
    nf0 = torch.from_numpy(hp.xs.reshape(n_xs, G, 3)[:, :, 0].astype(np.float64)).to(dev)
    # fuel materials only have nu*SigmaF
    s_ad = sm.Solver(hp)
    fl = FixedSourceLoss(hp, s_ad)
    sig = sig0.clone().requires_grad_(True)
    S = S0.clone().requires_grad_(True)
    nf = nf0.clone().requires_grad_(True)
    loss, q = fl(sig, S, nf, phi0)
    q.retain_grad()
    loss.backward()
    g_sig, g_S, g_nf, g_q = sig.grad.numpy(), S.grad.cpu().numpy(), nf.grad.cpu().numpy(), \
        q.grad.cpu().numpy()

    s64 = sm.Solver(hp, mode="fp64")
    lib, h = s64._lib, s64.handle
    NS, F = spec.n_sources, spec.fai

    def weights(nusf):
        return (fl.vol[:, None, None] * nusf[fl.src_xs][:, None, :]).expand(NS, F, G).reshape(-1)

    w = weights(nf0)

    def loss64(sigma=None, q64=None, nusf=None):
        if sigma is not None:
            L.check(lib.moc_set_sigma_t(h, L.ptr(np.ascontiguousarray(sigma, np.float32).ravel(),
                                                 C.c_float)), "sig")
        L.check(lib.moc_zero_state(h, 1, 1), "zero")
        torch.cuda.synchronize()
        L.check(lib.moc_set_fine_source64_device(h, q64.data_ptr()), "q64")
        L.check(lib.moc_transport_sweep(h, None), "sweep")
        phi = torch.empty(spec.n_fsr * G, dtype=torch.float64, device=dev)
        L.check(lib.moc_get_fine_flux64_device(h, phi.data_ptr()), "phi")
        s64.synchronize()
        ww = w if nusf is None else weights(nusf)
        return float((ww * phi).sum())

    q_base = fl.source_reference(phi0, S0, nf0).reshape(-1).contiguous()
    h_rel = 1e-3
    errs = []
    fuel = [m for m in range(n_xs) if np.abs(hp.xs.reshape(n_xs, G, 3)[m, :, 0]).max() > 0]
    for kind in ("sigma_t", "scatter", "nusf", "q"):
        for _ in range(16):
            if kind == "sigma_t":
                m, g = int(rng.integers(sig0.shape[0])), int(rng.integers(G))
                sp, sm_ = sig0.numpy().copy(), sig0.numpy().copy()
                sp[m, g] = np.float32(sp[m, g] * (1 + h_rel))
                sm_[m, g] = np.float32(sm_[m, g] * (1 - h_rel))
                fd = (loss64(sigma=sp, q64=q_base) - loss64(sigma=sm_, q64=q_base)) / \
                    (float(sp[m, g]) - float(sm_[m, g]))
                loss64(sigma=sig0.numpy(), q64=q_base)
                ad = g_sig[m, g]
            elif kind == "scatter":
                m, g, g2 = int(rng.integers(n_xs)), int(rng.integers(G)), int(rng.integers(G))
                d = h_rel * float(S0[m, g, g2])
                Sp, Sm = S0.clone(), S0.clone()
                Sp[m, g, g2] += d
                Sm[m, g, g2] -= d
                fd = (loss64(q64=fl.source_reference(phi0, Sp, nf0).reshape(-1).contiguous()) -
                      loss64(q64=fl.source_reference(phi0, Sm, nf0).reshape(-1).contiguous())) / (2 * d)
                ad = g_S[m, g, g2]
            elif kind == "nusf":
                m, g = int(rng.choice(fuel)), int(rng.integers(G))
                d = h_rel * float(nf0[m, g])
                Np, Nm = nf0.clone(), nf0.clone()
                Np[m, g] += d
                Nm[m, g] -= d
                fd = (loss64(q64=fl.source_reference(phi0, S0, Np).reshape(-1).contiguous(), nusf=Np) -
                      loss64(q64=fl.source_reference(phi0, S0, Nm).reshape(-1).contiguous(), nusf=Nm)) / (2 * d)
                ad = g_nf[m, g]
            else:
                k = int(rng.integers(q_base.numel()))
                d = h_rel * float(q_base[k])
                qp, qm = q_base.clone(), q_base.clone()
                qp[k] += d
                qm[k] -= d
                fd = (loss64(q64=qp) - loss64(q64=qm)) / (2 * d)
                ad = g_q[k]
            errs.append((kind, abs(ad - fd) / abs(fd), ad, fd))
    s_ad.close()
    s64.close()
    worst = max(errs, key=lambda e: e[1])
    assert worst[1] <= 1e-4, worst


def test_adjoint_time_within_three_forward_sweeps(gpu_available):
    """The reverse (adjoint) sweep within 3x a forward sweep of the same MIXED
    problem, both timed on the device (events on the library's stream, median
    of 5 after a warm-up).  The checkpointed forward that precedes it stands in
    for the plain forward (it must cost no more than 5 % above it), so the
    gradient costs the reverse sweep; forward + reverse is printed beside it."""
    import torch

    import simplemoc_gb300 as sm
    L = _lib()
    spec = _adjoint_spec()
    hp = sm.generate(spec, with_state=False)
    with sm.Solver(hp, mode="mixed") as s:
        lib, h = s._lib, s.handle
        s.autotune()
        s.time_sweep(1)
        t_fwd = s.time_sweep(5)
        dev = torch.device("cuda", 0)
        dphi = torch.rand(spec.n_fsr * spec.n_groups, device=dev)
        torch.cuda.synchronize()
        f, r = C.c_double(), C.c_double()
        L.check(lib.moc_time_adjoint(h, 8, dphi.data_ptr(), C.byref(f), C.byref(r)), "warm")
        fw, rv = [], []
        for _ in range(5):
            L.check(lib.moc_time_adjoint(h, 8, dphi.data_ptr(), C.byref(f), C.byref(r)), "time")
            fw.append(f.value)
            rv.append(r.value)
    f_ck, rev = float(np.median(fw)), float(np.median(rv))
    ratio = rev / t_fwd
    print(f"forward sweep {t_fwd:.2f} ms, forward with checkpoints {f_ck:.2f} ms, reverse "
          f"{rev:.2f} ms: reverse / forward {ratio:.2f}, (checkpointed forward + reverse) / "
          f"forward {(f_ck + rev) / t_fwd:.2f}")
    assert f_ck <= 1.05 * t_fwd
    assert ratio <= 3.0


def test_adjoint_fit_coefficient_gradients(gpu_available):
    """dL/d(c0, c1, c2) per fit window (src/solver.c:69-81), mapped back through
    c0 = y2, c1 = (y1 - y3)/(2dz), c2 = (y1 - 2 y2 + y3)/(2dz^2), give the
    kernel's dL/d fine_source (<= 1e-5 normwise: FP32 sums in other orders);
    a flat source has no fit."""
    import torch

    import simplemoc_gb300 as sm
    L = _lib()
    spec = sm.ProblemSpec(n_groups=12, fai=5, cai=4, height=200.0, n_sources=60, n_tracks_2d=12,
                          n_polar=4, z_stacked=10, n_seg=50, seed=31)
    hp = sm.generate(spec)
    G, F, NS = spec.n_groups, spec.fai, spec.n_sources
    dev = torch.device("cuda", 0)
    dphi = torch.from_numpy(np.random.default_rng(4).random(NS * F * G).astype(np.float32)).to(dev)
    with sm.Solver(hp, mode="mixed") as s:
        lib, h = s._lib, s.handle
        L.check(lib.moc_zero_state(h, 1, 1), "zero")
        L.check(lib.moc_adjoint_forward(h, 8), "fwd")
        dq = torch.empty(NS * F * G, dtype=torch.float32, device=dev)
        dfit = torch.empty(NS * (F - 2) * 3 * G, dtype=torch.float32, device=dev)
        torch.cuda.synchronize()
        L.check(lib.moc_adjoint_backward_fit(h, dphi.data_ptr(), dq.data_ptr(), None, None,
                                             dfit.data_ptr()), "bwd_fit")
        s.synchronize()
    dz = np.float32(spec.height) / np.float32(F * spec.decomp_ax * spec.cai)
    rd1 = np.float64(np.float32(1.0) / (np.float32(2.0) * dz))
    rd2 = np.float64(np.float32(1.0) / (np.float32(2.0) * dz * dz))
    fit = dfit.cpu().numpy().astype(np.float64).reshape(NS, F - 2, 3, G)
    back = np.zeros((NS, F, G))
    c0, c1, c2 = fit[:, :, 0], fit[:, :, 1], fit[:, :, 2]
    back[:, 0:F - 2] += c1 * rd1 + c2 * rd2
    back[:, 1:F - 1] += c0 - 2.0 * c2 * rd2
    back[:, 2:F] += c2 * rd2 - c1 * rd1
    ref = dq.cpu().numpy().astype(np.float64).reshape(NS, F, G)
    assert np.abs(ref).max() > 0 and np.abs(fit).max() > 0
    assert np.abs(back - ref).max() / np.abs(ref).max() <= 1e-5
    flat = sm.generate(spec.with_(axial_exp=0))
    with sm.Solver(flat, mode="mixed") as s:
        lib, h = s._lib, s.handle
        L.check(lib.moc_adjoint_forward(h, 8), "fwd")
        torch.cuda.synchronize()
        rc = lib.moc_adjoint_backward_fit(h, dphi.data_ptr(), None, None, None, dfit.data_ptr())
        assert rc == 6          # MOC_ERR_UNSUPPORTED


@pytest.mark.parametrize("G,F,n_mat", [(40, 5, 8), (7, 3, 3), (100, 5, 8), (130, 4, 5)])
def test_update_sources_adjoint_vs_torch_fp64(gpu_available, G, F, n_mat):
    """moc_update_sources_adjoint (hand-written) against torch autograd of the
    same update step in FP64, on random phi0 and dL/dq: dL/dS, dL/dnuSigmaF and
    dL/dphi0 to 1e-6 normwise; the library's forward step to 1e-6 of FP64."""
    import torch

    import simplemoc_gb300 as sm
    from simplemoc_gb300.adjoint import FixedSourceLoss, UpdateSources
    spec = sm.ProblemSpec(n_groups=G, fai=F, cai=4, height=200.0, n_sources=150,
                          n_materials=n_mat, n_fuel=max(1, n_mat // 2), n_tracks_2d=4, n_polar=2,
                          z_stacked=4, n_seg=10, axial_exp=2 if F >= 3 else 0, seed=900 + G)
    hp = sm.generate(spec)
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(G)
    n_xs = hp.xs.size // (3 * G)
    phi0 = torch.from_numpy(rng.random((spec.n_sources, F, G))).to(dev)
    dq = torch.from_numpy(rng.standard_normal(spec.n_fsr * G)).to(dev)
    S0 = torch.from_numpy(hp.scatter.reshape(n_xs, G, G).astype(np.float64)).to(dev)
    N0 = torch.from_numpy(hp.xs.reshape(n_xs, G, 3)[:, :, 0].astype(np.float64)).to(dev)
    keff = 1.17
    with sm.Solver(hp, mode="mixed") as s:
        fl = FixedSourceLoss(hp, s, keff=keff)
        # library step and its reverse
        p1 = phi0.clone().requires_grad_(True)
        S1, N1 = S0.clone().requires_grad_(True), N0.clone().requires_grad_(True)
        q1 = UpdateSources.apply(p1.reshape(-1), S1, N1, s, hp.xs, keff)
        (q1.double() * dq).sum().backward()
        # torch FP64 yardstick
        p2 = phi0.clone().requires_grad_(True)
        S2, N2 = S0.clone().requires_grad_(True), N0.clone().requires_grad_(True)
        q2 = fl.source_reference(p2, S2, N2).reshape(-1)
        (q2 * dq).sum().backward()
    rel = lambda a, b: float((a - b).detach().abs().max() / b.detach().abs().max())
    assert rel(q1.double(), q2.detach()) <= 1e-6
    assert rel(S1.grad, S2.grad) <= 1e-6
    fuel = N2.grad.abs().amax(dim=1) > 0
    assert rel(N1.grad[fuel], N2.grad[fuel]) <= 1e-6
    assert rel(p1.grad, p2.grad) <= 1e-6
