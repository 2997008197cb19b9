"""The track-partitioned power iteration of one problem (tracks_parallel.py) on
CPU ranks: two gloo processes each sweep half of the 2D tracks with the oracle
as the sweep backend, sum the scalar flux with an all-reduce, and run
renormalize / update_sources / compute_keff replicated.  The result gathered
from both ranks equals one rank sweeping every track (reference multi-rank
reductions: src/solver.c:1189-1196, 1394-1418)."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")

ITERS = 3
TOL = 1e-5          # FP32 tally order only: the ranks' partial sums add in another order


def _spec():
    import simplemoc_gb300 as sm
    return sm.ProblemSpec(n_groups=12, fai=5, cai=2, height=60.0, n_sources=40, n_tracks_2d=7,
                          n_polar=4, z_stacked=6, n_seg=20, seed=4242)


class OracleBackend:
    """A CPU rank: the oracle's serial sweep and post-sweep steps on numpy
    state (test infrastructure standing in for the GPU library)."""

    def __init__(self, hp):
        import oracle
        self.port = oracle.Port()
        self.op = oracle.make_problem(hp)
        self.st = oracle.fresh_state(hp)

    def zero_flux(self):
        self.st["fine_flux"][:] = 0

    def transport_sweep(self):
        return self.port.sweep(self.op, self.st["fine_source"], self.st["fine_flux"],
                               self.st["psi_f"])

    def synchronize(self):
        pass

    def flux_tensor(self):
        return torch.from_numpy(self.st["fine_flux"])

    def after_collective(self):
        pass

    def renormalize_flux(self):
        self.port.renormalize(self.op, self.st["fine_flux"], self.st["psi_f"], self.st["psi_b"])

    def update_sources(self, keff):
        return self.port.update_sources(self.op, self.st["fine_flux"], self.st["fine_source"],
                                        keff)

    def compute_keff(self, leakage=0.0):
        return self.port.compute_keff(self.op, self.st["fine_flux"], leakage)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist

    import simplemoc_gb300 as sm
    from simplemoc_gb300.tracks_parallel import TrackPartitioned, partition, rank_problem
    dist.init_process_group("gloo", rank=rank, world_size=world)
    hp = sm.generate(_spec())
    lo, hi = partition(hp.spec.n_tracks_2d, world, rank)
    b = OracleBackend(rank_problem(hp, lo, hi))
    hist = TrackPartitioned(b, rank, world, dist).run(ITERS)
    q.put((rank, lo, hi, hist, {k: v.copy() for k, v in b.st.items()}))
    dist.barrier()
    dist.destroy_process_group()


def test_partition_covers_every_track_once():
    from simplemoc_gb300.tracks_parallel import partition
    for n in (1, 7, 16384):
        for world in (1, 2, 3, 8):
            if world > n:
                continue
            ranges = [partition(n, world, r) for r in range(world)]
            assert ranges[0][0] == 0 and ranges[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(ranges, ranges[1:]))
            sizes = [hi - lo for lo, hi in ranges]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        partition(8, 2, 2)


def test_rank_problem_is_the_tracks_of_its_range():
    import simplemoc_gb300 as sm
    from simplemoc_gb300.tracks_parallel import rank_problem
    hp = sm.generate(_spec())
    s = hp.spec
    sub = rank_problem(hp, 2, 5)
    PZ, S, G = s.n_polar * s.z_stacked, s.n_seg, s.n_groups
    assert sub.spec.n_tracks_2d == 3 and sub.spec.n_tracks_3d == 3 * PZ
    assert np.array_equal(sub.seg_len, hp.seg_len[2 * S:5 * S])
    assert np.array_equal(sub.seg_src, hp.seg_src[2 * PZ * S:5 * PZ * S])
    assert np.array_equal(sub.z0, hp.z0[2 * PZ:5 * PZ])
    assert sub.psi_f.size == 3 * PZ * G
    assert sub.fine_source is hp.fine_source          # the full source storage
    with pytest.raises(ValueError):
        rank_problem(hp, 3, 3)


def test_two_gloo_ranks_equal_one_rank(port):
    import oracle
    import simplemoc_gb300 as sm
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    p = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, p, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    out = sorted((q.get(timeout=180) for _ in procs), key=lambda t: t[0])
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    # one rank sweeping every track
    hp = sm.generate(_spec())
    st = oracle.fresh_state(hp)
    ref_hist = port.iterate(hp, st, ITERS)
    G = hp.spec.n_groups
    PZG = hp.spec.n_polar * hp.spec.z_stacked * G
    for rank, lo, hi, hist, rst in out:
        np.testing.assert_allclose(np.asarray(hist)[:, 0], np.asarray(ref_hist)[:, 0],
                                   rtol=TOL)
        for k in ("fine_flux", "fine_source"):          # replicated on every rank
            err = np.abs(rst[k] - st[k]).max() / np.abs(st[k]).max()
            assert err <= TOL, (rank, k, err)
        for k in ("psi_f", "psi_b"):                   # the rank's own tracks
            ref = st[k][lo * PZG:hi * PZG]
            den = max(np.abs(st[k]).max(), 1e-30)
            assert np.abs(rst[k] - ref).max() / den <= TOL, (rank, k)
    # the two ranks hold the same replicated state to the bit
    assert np.array_equal(out[0][4]["fine_flux"], out[1][4]["fine_flux"])
    assert np.array_equal(out[0][4]["fine_source"], out[1][4]["fine_source"])
    assert out[0][3] == out[1][3]


def test_one_rank_needs_no_group(port):
    """World 1: the partitioned iteration is the plain one, bit for bit."""
    import oracle
    import simplemoc_gb300 as sm
    from simplemoc_gb300.tracks_parallel import TrackPartitioned
    hp = sm.generate(_spec())
    b = OracleBackend(hp)
    hist = TrackPartitioned(b).run(ITERS)
    st = oracle.fresh_state(hp)
    ref = port.iterate(hp, st, ITERS)
    assert hist == ref
    for k in ("fine_flux", "fine_source", "psi_f", "psi_b"):
        assert np.array_equal(b.st[k], st[k]), k
    with pytest.raises(ValueError):
        TrackPartitioned(b, 0, 2, None)
