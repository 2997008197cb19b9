"""GPU tests of the batched persistent sweep: every core of a batch against the
same core swept on its own (and against the oracle), with and without the
CUDA-graph power iteration.

Tolerances as in test_gpu_sweep: psi bit-identical after one PLAIN sweep;
fluxes normwise <= 1e-5 (tally order); k_eff <= 1e-5.
"""
import numpy as np
import pytest

import oracle
from tests._util import rel_err

pytestmark = pytest.mark.gpu


def _specs():
    import simplemoc_gb300 as sm
    out = []
    for c, (g, p, s, n2d, ns) in enumerate([(100, 4, 50, 24, 300), (20, 2, 80, 40, 150),
                                            (37, 6, 20, 16, 200), (64, 4, 33, 20, 250),
                                            (7, 2, 45, 12, 90), (128, 6, 26, 8, 120)]):
        out.append(sm.ProblemSpec(n_groups=g, fai=5, cai=4, height=200.0, n_sources=ns,
                                  n_tracks_2d=n2d, n_polar=p, z_stacked=10, n_seg=s,
                                  seed=7000 + c))
    return out


@pytest.mark.parametrize("mode", ["plain", "mixed"])
def test_batched_sweep_equals_separate_sweeps(gpu_available, port, mode):
    import simplemoc_gb300 as sm
    from simplemoc_gb300.batch import Batch
    specs = _specs()
    hps = [sm.generate(s) for s in specs]
    solvers = [sm.Solver(h, mode=mode) for h in hps]
    with Batch(solvers) as b:
        widths = b.autotune()
        assert all(w in (4, 8, 16, 32) for w in widths)
        b.sweep()
    for h, s, w in zip(hps, solvers, widths):
        out = s.download(psi_f=True, fine_flux=True, fine_source=False)
        with sm.Solver(h, mode=mode) as alone:
            alone.transport_sweep()
            ref = alone.download(psi_f=True, fine_flux=True, fine_source=False)
        assert np.array_equal(out["psi_f"], ref["psi_f"]), (h.spec.n_groups, w)
        assert rel_err(out["fine_flux"], ref["fine_flux"]) <= 1e-5
        if mode == "plain":
            st = oracle.fresh_state(h)
            op = oracle.make_problem(h)
            port.sweep(op, st["fine_source"], st["fine_flux"], st["psi_f"])
            assert np.array_equal(out["psi_f"], st["psi_f"])
        s.close()


@pytest.mark.parametrize("graph", [True, False])
def test_batched_power_iterations_match_separate_runs(gpu_available, graph):
    import simplemoc_gb300 as sm
    from simplemoc_gb300.batch import Batch
    specs = _specs()
    hps = [sm.generate(s) for s in specs]
    solvers = [sm.Solver(h, mode="plain") for h in hps]
    iters = 4
    with Batch(solvers) as b:
        b.power_iterations(iters, graph=graph)
        keff, res = b.results()
    for c, (h, s) in enumerate(zip(hps, solvers)):
        # exactly `iters` iterations, with or without the graph (its first
        # call runs one of them eagerly before capturing)
        with sm.Solver(h, mode="plain") as alone:
            hist = alone.run(iters)
            ref = alone.download(fine_flux=True, fine_source=True, psi_f=True)
        out = s.download(fine_flux=True, fine_source=True, psi_f=True)
        assert abs(keff[c] - hist[-1][0]) <= 1e-5 * abs(hist[-1][0]), c
        for k in ("fine_flux", "fine_source", "psi_f"):
            assert rel_err(out[k], ref[k]) <= 1e-5, (c, k)
        s.close()


def test_batch_rejects_mixed_modes(gpu_available):
    import simplemoc_gb300 as sm
    from simplemoc_gb300.batch import Batch
    specs = _specs()[:2]
    a = sm.Solver(sm.generate(specs[0]), mode="plain")
    b = sm.Solver(sm.generate(specs[1]), mode="mixed")
    with pytest.raises(sm.MocError):
        Batch([a, b])
    a.close()
    b.close()


def test_batch_reports_a_cores_bad_source_id(gpu_available):
    """A streamed upload leaves the source ids to the sweep: a batch that sweeps
    a core with an id out of range reports MOC_ERR_ARG for it, the core refuses
    work until a valid upload, and the other cores are untouched."""
    import simplemoc_gb300 as sm
    from simplemoc_gb300.batch import Batch
    specs = _specs()[:3]
    hps = [sm.generate(s) for s in specs]
    solvers = [sm.Solver(h, mode="plain") for h in hps]
    try:
        with Batch(solvers) as b:
            bad = hps[1].copy_state()
            bad.seg_src = hps[1].seg_src.copy()
            bad.seg_src[-1] = specs[1].n_sources
            solvers[1].upload(bad)
            with pytest.raises(sm.MocError) as e:
                b.sweep()
            assert e.value.status == 1                     # MOC_ERR_ARG
            with pytest.raises(sm.MocError) as e:
                b.sweep()
            assert e.value.status == 4                     # MOC_ERR_STATE: core 1 is stale
            for s in solvers:
                s.upload()
            b.sweep()
        for h, s in zip(hps, solvers):
            out = s.download(psi_f=True, fine_flux=False, fine_source=False)
            with sm.Solver(h, mode="plain") as alone:
                alone.transport_sweep()
                ref = alone.download(psi_f=True, fine_flux=False, fine_source=False)
            assert np.array_equal(out["psi_f"], ref["psi_f"])
    finally:
        for s in solvers:
            s.close()


def test_batch_graph_recaptured_after_an_upload(gpu_available):
    """The captured iteration bakes in each core's update work lists.  After a
    core is uploaded again with every source on one material (other work-list
    sizes), the next graph call captures afresh: its results equal separate
    runs of the new inputs (an upload does not reset the k_eff that the batch
    chains on the device, so those runs start from it)."""
    import simplemoc_gb300 as sm
    from simplemoc_gb300.batch import Batch
    specs = _specs()[:3]
    hps = [sm.generate(s) for s in specs]
    solvers = [sm.Solver(h, mode="plain") for h in hps]
    new = hps[1].copy_state()
    new.src_xs = np.zeros_like(hps[1].src_xs)
    inputs = [hps[0], new, hps[2]]
    try:
        with Batch(solvers) as b:
            b.power_iterations(2, graph=True)
            keff0, _ = b.results()
            for s, h in zip(solvers, inputs):
                s.upload(h)
            b.power_iterations(3, graph=True)
            keff, _ = b.results()
        for c, (h, s) in enumerate(zip(inputs, solvers)):
            with sm.Solver(h, mode="plain") as alone:
                hist = alone.run(3, keff=float(keff0[c]))    # exactly the 3 asked for
                ref = alone.download(fine_flux=True, fine_source=True, psi_f=True)
            out = s.download(fine_flux=True, fine_source=True, psi_f=True)
            assert abs(keff[c] - hist[-1][0]) <= 1e-5 * abs(hist[-1][0]), c
            for k in ("fine_flux", "fine_source", "psi_f"):
                assert rel_err(out[k], ref[k]) <= 1e-5, (c, k)
    finally:
        for s in solvers:
            s.close()
