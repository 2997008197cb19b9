"""Track-partitioned power iteration of ONE problem over several ranks.

The reference's multi-rank path decomposes space: each MPI rank owns a block
of the core, exchanges the boundary angular flux with its six neighbours
(src/comms.c:5-196, on the fixed 2x2x1 grid of src/init.c:169) and reduces
scalars across ranks (MPI_Allreduce of the fission rate,
src/solver.c:1189-1196; MPI_Reduce of absorption, fission and leakage,
src/solver.c:1394-1418).

3D tracks are independent of one another, so on GPUs the sweep shards by
tracks instead, with no halo exchange:

* each rank owns a contiguous range of whole 2D tracks -- with all of their
  polar angles and stacked rays, which are a contiguous range of 3D tracks --
  and sweeps them against the full source storage;
* the one exchange is an all-reduce (SUM) of the scalar flux after each sweep,
  in place on the library's flux storage (moc_fine_flux_storage);
* renormalize_flux, update_sources and compute_keff then run replicated: every
  rank holds the same flux, so every rank computes the same norm, source and
  k_eff, and scales the angular flux of its own tracks.

The scalar flux accumulates across sweeps (the reference never zeroes
fine_flux between sweeps): rank 0 sweeps on top of the flux, the other ranks
tally from zero, so the sum is the single-rank flux up to the order of its FP32
additions, which are unordered anyway.

The backend is anything with the four reference entry points plus
zero_state / synchronize / flux_tensor: a `SolverBackend` over the GPU library
(NCCL process group), or a CPU stand-in in the tests (gloo).
"""
from __future__ import annotations

from dataclasses import replace

from .problem import HostProblem


def partition(n_tracks_2d: int, world: int, rank: int) -> tuple[int, int]:
    """[lo, hi) of the 2D tracks rank `rank` of `world` sweeps: contiguous,
    sizes differing by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    return n_tracks_2d * rank // world, n_tracks_2d * (rank + 1) // world


def rank_problem(hp: HostProblem, lo: int, hi: int) -> HostProblem:
    """The problem of 2D tracks [lo, hi): views of the per-track arrays (2D
    track i owns 3D tracks i*P*Z .. (i+1)*P*Z - 1, src/tracks.c:100-101) and the
    full source and cross-section storage."""
    s = hp.spec
    if not 0 <= lo < hi <= s.n_tracks_2d:
        raise ValueError("empty or out-of-range track range")
    S, G, PZ = s.n_seg, s.n_groups, s.n_polar * s.z_stacked
    t0, t1 = lo * PZ, hi * PZ

    def tracks(a, per):
        return None if a is None else a[t0 * per:t1 * per]

    return replace(hp, spec=s.with_(n_tracks_2d=hi - lo), seg_len=hp.seg_len[lo * S:hi * S],
                   seg_src=tracks(hp.seg_src, S), az_weight=hp.az_weight[lo:hi],
                   p_weight=tracks(hp.p_weight, 1), z0=tracks(hp.z0, 1),
                   psi_f=tracks(hp.psi_f, G), psi_b=tracks(hp.psi_b, G), _keep=[hp])


class _CudaArray:
    """A device buffer described by the CUDA array interface, so that torch can
    wrap the library's own storage without a copy."""

    def __init__(self, ptr: int, n: int, typestr: str):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr,
                                         "data": (ptr, False), "version": 3, "strides": None}


class SolverBackend:
    """The GPU library as a track-partitioned rank (one Solver, one device)."""

    def __init__(self, solver, device: int):
        self.s = solver
        self.device = device

    def zero_flux(self) -> None:
        self.s.zero_state(flux=True, psi=False)

    def transport_sweep(self) -> int:
        return self.s.transport_sweep()

    def synchronize(self) -> None:
        self.s.synchronize()

    def flux_tensor(self):
        import torch
        st = self.s.flux_storage()
        ts = "<f8" if st["elem_bytes"] == 8 else "<f4"
        return torch.as_tensor(_CudaArray(st["ptr"], st["n"], ts),
                               device=torch.device("cuda", self.device))

    def after_collective(self) -> None:
        import torch
        torch.cuda.current_stream(self.device).synchronize()

    def renormalize_flux(self) -> None:
        self.s.renormalize_flux()

    def update_sources(self, keff: float) -> float:
        return self.s.update_sources(keff)

    def compute_keff(self, leakage: float = 0.0) -> float:
        return self.s.compute_keff(leakage)


class TrackPartitioned:
    """One rank of a track-partitioned power iteration (src/main.c:57-92 with
    the flux summed across ranks between the sweep and renormalize_flux).
    `dist` is torch.distributed with an initialised process group (NCCL for
    GPU backends, gloo for CPU ones); world 1 needs none."""

    def __init__(self, backend, rank: int = 0, world: int = 1, dist=None, group=None):
        if world > 1 and dist is None:
            raise ValueError("several ranks need a process group")
        self.b, self.rank, self.world, self.dist, self.group = backend, rank, world, dist, group

    def transport_sweep(self) -> int:
        """This rank's sweep, then the all-reduce of the scalar flux; returns
        this rank's segments processed."""
        if self.world > 1 and self.rank != 0:
            self.b.zero_flux()
        n = self.b.transport_sweep()
        if self.world > 1:
            self.b.synchronize()
            t = self.b.flux_tensor()
            self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM, group=self.group)
            self.b.after_collective()
        return n

    def power_iteration(self, keff: float) -> tuple[float, float]:
        self.transport_sweep()
        self.b.renormalize_flux()
        res = self.b.update_sources(keff)
        return self.b.compute_keff(0.0), res

    def run(self, n_iters: int, keff: float = 1.0) -> list[tuple[float, float]]:
        out = []
        for _ in range(n_iters):
            keff, res = self.power_iteration(keff)
            out.append((keff, res))
        return out
