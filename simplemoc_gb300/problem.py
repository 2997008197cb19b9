"""Problem description, seeded generation and the named workloads.

A problem is the flat storage of include/simplemoc_gb300.h held in numpy
arrays: the explicit 3D segment streams that replace the random traversal of
transport_sweep (src/solver.c:379-483) and the source / cross-section storage of
src/source.c.  Generation runs in the C library (counter-based, seeded), so a
problem is reproducible on any machine and with any thread count.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field, replace

import numpy as np

from . import _lib as L


@dataclass(frozen=True)
class ProblemSpec:
    n_groups: int = 100
    fai: int = 5
    cai: int = 4
    decomp_ax: int = 1
    height: float = 200.0
    axial_exp: int = 2
    n_sources: int = 4624
    n_materials: int = 8
    n_tracks_2d: int = 1024
    n_polar: int = 4
    z_stacked: int = 300
    n_seg: int = 50
    precision: float = 0.01          # exp table precision (Input.precision)
    seed: int = 20260101
    n_fuel: int = 4
    len_lo: float = 0.05
    len_hi: float = 1.5
    sigt_lo: float = 0.1
    sigt_hi: float = 2.0
    scatter_ratio: float = 0.7
    nusf_hi: float = 0.05
    siga_ratio: float = 0.3
    vol_lo: float = 0.5
    vol_hi: float = 1.5
    axial_z_sep: float = 0.0         # 0: height / z_stacked

    @property
    def n_tracks_3d(self) -> int:
        return self.n_tracks_2d * self.n_polar * self.z_stacked

    @property
    def n_fsr(self) -> int:
        return self.n_sources * self.fai

    @property
    def integrations_per_sweep(self) -> int:
        """Segment-group integrations of one sweep (N3D * S * G)."""
        return self.n_tracks_3d * self.n_seg * self.n_groups

    def algorithmic_bytes(self) -> int:
        """HBM bytes one sweep must move at minimum:
        3 fine-source rows read + tally read-modify-write per integration
        (20 B), psi read + write per track-group (8 B), 3D segment stream
        (source id, 4 B per segment) and 3D lengths (4 B per 2D segment and
        polar angle)."""
        quad_rows = 3 if self.axial_exp == 2 else 1
        per_int = 4 * quad_rows + 8
        return (per_int * self.integrations_per_sweep
                + 8 * self.n_tracks_3d * self.n_groups
                + 4 * self.n_tracks_3d * self.n_seg
                + 4 * self.n_tracks_2d * self.n_polar * self.n_seg)

    def with_(self, **kw) -> "ProblemSpec":
        return replace(self, **kw)


def pins(assemblies_x: int, assemblies_y: int, pins_per_side: int = 17) -> int:
    return assemblies_x * assemblies_y * pins_per_side * pins_per_side


# Geometry of the small problem: 2x2 assemblies of 17x17 pins, 200 cm tall,
# 20 axial source regions per pin as 4 coarse x 5 fine; 16 azimuthal angles x
# 64 tracks, 4 polar angles, 300 stacked rays, 50 segments per 3D track.
CONFIG_SMALL = ProblemSpec(
    n_groups=100, fai=5, cai=4, height=200.0, n_sources=pins(2, 2) * 4,
    n_tracks_2d=16 * 64, n_polar=4, z_stacked=300, n_seg=50, seed=20260101)

# Default strawman problem: 17x17 assemblies of 17x17 pins, 400 cm tall, 30
# axial regions per pin as 6 x 5; 64 azimuthal angles x 256 tracks, 10 polar
# angles, 80 stacked rays (the reference default z_stacked), 50 segments.
CONFIG_DEFAULT = ProblemSpec(
    n_groups=100, fai=5, cai=6, height=400.0, n_sources=pins(17, 17) * 6,
    n_tracks_2d=64 * 256, n_polar=10, z_stacked=80, n_seg=50, seed=20260102)

# The default problem's full source storage (2 GB of FSR arrays, larger than
# L2) swept by 1024 of its 16384 2D tracks: the profiling case (~3 GB).
CONFIG_DEFAULT_1K = CONFIG_DEFAULT.with_(n_tracks_2d=1024)

# The default problem with the flat source (axial_exp = 0,
# attenuate_FSR_fluxes): one fine-source row per segment instead of three.
CONFIG_DEFAULT_FLAT = CONFIG_DEFAULT.with_(axial_exp=0)

CONFIGS = {"small": CONFIG_SMALL, "default": CONFIG_DEFAULT, "default_1k": CONFIG_DEFAULT_1K,
           "flat": CONFIG_DEFAULT_FLAT}


def exp_table(precision: float, maxval: float = 10.0):
    """(values[2N], dx, maxval_reduced, N) as buildExponentialTable (src/utils.c:48-78)."""
    lib = L._lib()
    n = int(lib.moc_exp_table_size(precision, maxval))
    if n < 1:
        raise ValueError("table precision must be positive")
    vals = np.empty(2 * n, dtype=np.float32)
    dx = C.c_float()
    mv = C.c_float()
    L.check(lib.moc_build_exp_table(precision, maxval, L.ptr(vals, C.c_float), n,
                                    C.byref(dx), C.byref(mv)), "moc_build_exp_table")
    return vals, float(dx.value), float(mv.value), n


@dataclass
class HostProblem:
    """Host-side arrays of one problem (numpy, C-contiguous)."""
    spec: ProblemSpec
    seg_len: np.ndarray
    seg_src: np.ndarray
    az_weight: np.ndarray
    p_weight: np.ndarray
    z0: np.ndarray
    polar_angles: np.ndarray
    src_sigt: np.ndarray
    src_xs: np.ndarray
    vol: np.ndarray
    sigt: np.ndarray
    xs: np.ndarray
    scatter: np.ndarray
    fine_source: np.ndarray
    fine_flux: np.ndarray | None
    psi_f: np.ndarray | None
    psi_b: np.ndarray | None
    table: np.ndarray
    table_dx: float
    table_maxval: float
    table_n: int
    _keep: list = field(default_factory=list, repr=False)

    def dims(self) -> L.MocDims:
        s = self.spec
        return L.MocDims(
            n_groups=s.n_groups, fai=s.fai, cai=s.cai, decomp_ax=s.decomp_ax, height=s.height,
            axial_exp=s.axial_exp, n_sources=s.n_sources,
            n_sigt=int(self.sigt.size // s.n_groups), n_xs=int(self.xs.size // (3 * s.n_groups)),
            n_tracks_2d=s.n_tracks_2d, n_polar=s.n_polar, z_stacked=s.z_stacked, n_seg=s.n_seg,
            table_n=self.table_n, table_dx=self.table_dx, table_maxval=self.table_maxval)

    def host(self) -> L.MocHost:
        f, i = C.c_float, C.c_int32
        return L.MocHost(
            seg_len=L.ptr(self.seg_len, f), seg_src=L.ptr(self.seg_src, i),
            az_weight=L.ptr(self.az_weight, f), p_weight=L.ptr(self.p_weight, f),
            z0=L.ptr(self.z0, f), polar_angles=L.ptr(self.polar_angles, f),
            src_sigt=L.ptr(self.src_sigt, i), src_xs=L.ptr(self.src_xs, i),
            vol=L.ptr(self.vol, f), sigt=L.ptr(self.sigt, f), xs=L.ptr(self.xs, f),
            scatter=L.ptr(self.scatter, f), fine_source=L.ptr(self.fine_source, f),
            fine_flux=L.ptr(self.fine_flux, f), psi_f=L.ptr(self.psi_f, f),
            psi_b=L.ptr(self.psi_b, f), table=L.ptr(self.table, f))

    def input_nbytes(self) -> int:
        arrs = [self.seg_len, self.seg_src, self.az_weight, self.p_weight, self.z0,
                self.polar_angles, self.src_sigt, self.src_xs, self.vol, self.sigt, self.xs,
                self.scatter, self.fine_source, self.table]
        arrs += [a for a in (self.fine_flux, self.psi_f, self.psi_b) if a is not None]
        return int(sum(a.nbytes for a in arrs))

    def copy_state(self) -> "HostProblem":
        """Same inputs, private copies of the mutable state arrays."""
        c = replace(self)
        c.fine_source = self.fine_source.copy()
        c.fine_flux = None if self.fine_flux is None else self.fine_flux.copy()
        c.psi_f = None if self.psi_f is None else self.psi_f.copy()
        c.psi_b = None if self.psi_b is None else self.psi_b.copy()
        return c


def _empty(shape, dtype, alloc):
    return alloc(shape, dtype) if alloc is not None else np.empty(shape, dtype=dtype)


def generate(spec: ProblemSpec, with_state: bool = True, alloc=None) -> HostProblem:
    """Seeded synthetic problem.  `alloc(shape, dtype)` may supply (pinned) buffers.
    with_state=False leaves fine_flux / psi as None (zeros on upload)."""
    lib = L._lib()
    s = spec
    G, NS, F, N2D, P, Z, S = (s.n_groups, s.n_sources, s.fai, s.n_tracks_2d, s.n_polar,
                              s.z_stacked, s.n_seg)
    N3D = N2D * P * Z
    NM = s.n_materials
    table, dx, mv, n = exp_table(s.precision)
    arr = dict(
        seg_len=_empty((N2D * S,), np.float32, alloc),
        seg_src=_empty((N3D * S,), np.int32, alloc),
        az_weight=_empty((N2D,), np.float32, alloc),
        p_weight=_empty((N3D,), np.float32, alloc),
        z0=_empty((N3D,), np.float32, alloc),
        polar_angles=_empty((P,), np.float32, alloc),
        src_sigt=_empty((NS,), np.int32, alloc),
        src_xs=_empty((NS,), np.int32, alloc),
        vol=_empty((NS,), np.float32, alloc),
        sigt=_empty((NM * G,), np.float32, alloc),
        xs=_empty((NM * G * 3,), np.float32, alloc),
        scatter=_empty((NM * G * G,), np.float32, alloc),
        fine_source=_empty((NS * F * G,), np.float32, alloc),
    )
    gp = L.MocGenParams(seed=s.seed, n_materials=NM, n_fuel=s.n_fuel, len_lo=s.len_lo,
                        len_hi=s.len_hi, sigt_lo=s.sigt_lo, sigt_hi=s.sigt_hi,
                        scatter_ratio=s.scatter_ratio, nusf_hi=s.nusf_hi,
                        siga_ratio=s.siga_ratio, vol_lo=s.vol_lo, vol_hi=s.vol_hi,
                        axial_z_sep=s.axial_z_sep)
    f, i = C.c_float, C.c_int32
    dims = L.MocDims(n_groups=G, fai=F, cai=s.cai, decomp_ax=s.decomp_ax, height=s.height,
                     axial_exp=s.axial_exp, n_sources=NS, n_sigt=NM, n_xs=NM,
                     n_tracks_2d=N2D, n_polar=P, z_stacked=Z, n_seg=S, table_n=n,
                     table_dx=dx, table_maxval=mv)
    L.check(lib.moc_generate(
        C.byref(dims), C.byref(gp), L.ptr(arr["seg_len"], f), L.ptr(arr["seg_src"], i),
        L.ptr(arr["az_weight"], f), L.ptr(arr["p_weight"], f), L.ptr(arr["z0"], f),
        L.ptr(arr["polar_angles"], f), L.ptr(arr["src_sigt"], i), L.ptr(arr["src_xs"], i),
        L.ptr(arr["vol"], f), L.ptr(arr["sigt"], f), L.ptr(arr["xs"], f),
        L.ptr(arr["scatter"], f), L.ptr(arr["fine_source"], f)), "moc_generate")
    if with_state:
        phi = _empty((NS * F * G,), np.float32, alloc)
        psi_f = _empty((N3D * G,), np.float32, alloc)
        psi_b = _empty((N3D * G,), np.float32, alloc)
        phi[:] = 0
        psi_f[:] = 0
        psi_b[:] = 0
    else:
        phi = psi_f = psi_b = None
    return HostProblem(spec=spec, fine_flux=phi, psi_f=psi_f, psi_b=psi_b, table=table,
                       table_dx=dx, table_maxval=mv, table_n=n, **arr)
