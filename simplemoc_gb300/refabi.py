"""ctypes mirror of include/simplemoc_refabi.h: the reference's own structs
(src/SimpleMOC_header.h:28-158, serial build) and its four solver entry
points as exported by libsimplemoc_gb300.so.

`RefProblem` builds a reference-layout problem (Params / Input with the
reference's pointer-per-row storage) over numpy arrays, so that Python code can
drive the drop-in exactly as src/main.c does.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L

fp = C.POINTER(C.c_float)
fpp = C.POINTER(fp)


class Input(C.Structure):
    _fields_ = [
        ("x_assemblies", C.c_int), ("y_assemblies", C.c_int), ("cai", C.c_int),
        ("fai", C.c_int), ("axial_exp", C.c_int), ("radial_ray_sep", C.c_float),
        ("axial_z_sep", C.c_float), ("n_azimuthal", C.c_int), ("n_polar_angles", C.c_int),
        ("n_egroups", C.c_int), ("decompose", C.c_bool), ("decomp_assemblies_ax", C.c_int),
        ("segments_per_track", C.c_long), ("assembly_width", C.c_float), ("height", C.c_float),
        ("domain_height", C.c_float), ("precision", C.c_float), ("mype", C.c_long),
        ("ntracks_2D", C.c_long), ("z_stacked", C.c_int), ("ntracks", C.c_long),
        ("nthreads", C.c_int), ("papi_event_set", C.c_int),
        ("n_2D_source_regions_per_assembly", C.c_long), ("n_source_regions_per_node", C.c_long),
        ("load_tracks", C.c_bool), ("track_file", C.c_char_p), ("segments_processed", C.c_long),
    ]


class Segment(C.Structure):
    _fields_ = [("length", C.c_float), ("source_id", C.c_long)]


class Track2D(C.Structure):
    _fields_ = [("az_weight", C.c_float), ("n_segments", C.c_long),
                ("segments", C.POINTER(Segment)), ("n_3D_segments", C.c_int)]


class Track(C.Structure):
    _fields_ = [("p_weight", C.c_float), ("z_height", C.c_float), ("rank_in", C.c_long),
                ("rank_out", C.c_long), ("f_psi", fp), ("b_psi", fp)]


class Source(C.Structure):
    _fields_ = [("fine_flux", fpp), ("fine_source", fpp), ("vol", C.c_float), ("sigT", fp),
                ("XS", fpp), ("scattering_matrix", fpp)]


class Table(C.Structure):
    _fields_ = [("values", fp), ("dx", C.c_float), ("maxVal", C.c_float), ("N", C.c_int)]


class Params(C.Structure):
    _fields_ = [("tracks_2D", C.POINTER(Track2D)),
                ("tracks", C.POINTER(C.POINTER(C.POINTER(Track)))),
                ("sources", C.POINTER(Source)), ("polar_angles", fp), ("leakage", fp),
                ("expTable", Table)]


class CommGrid(C.Structure):
    _fields_ = [(n, C.c_int) for n in (
        "x_pos_src", "x_pos_dest", "x_neg_src", "x_neg_dest", "y_pos_src", "y_pos_dest",
        "y_neg_src", "y_neg_dest", "z_pos_src", "z_pos_dest", "z_neg_src", "z_neg_dest")]


RNG_LIBC = 0
RNG_HASH = 1

_BOUND = False


def lib() -> C.CDLL:
    global _BOUND
    lb = L._lib()
    if not _BOUND:
        lb.transport_sweep.argtypes = [C.POINTER(Params), C.POINTER(Input)]
        lb.transport_sweep.restype = None
        lb.renormalize_flux.argtypes = [Params, Input, CommGrid]
        lb.renormalize_flux.restype = None
        lb.update_sources.argtypes = [Params, Input, C.c_float]
        lb.update_sources.restype = C.c_float
        lb.compute_keff.argtypes = [Params, Input, CommGrid]
        lb.compute_keff.restype = C.c_float
        lb.moc_ref_set_rng.argtypes = [C.c_int, C.c_uint64]
        lb.moc_ref_set_rng.restype = C.c_int
        lb.moc_ref_sync_to_host.argtypes = [C.POINTER(Params), C.POINTER(Input)]
        lb.moc_ref_sync_to_host.restype = C.c_int
        lb.moc_ref_finalize.argtypes = []
        lb.moc_ref_finalize.restype = None
        lb.moc_ref_status.argtypes = []
        lb.moc_ref_status.restype = C.c_int
        lb.moc_ref_last_segments.argtypes = []
        lb.moc_ref_last_segments.restype = C.c_int64
        lb.moc_ref_last_rng_ms.argtypes = []
        lb.moc_ref_last_rng_ms.restype = C.c_double
        lb.moc_ref_libc_draws.argtypes = [C.POINTER(C.c_int32), C.c_int64, C.POINTER(C.c_int)]
        lb.moc_ref_libc_draws.restype = C.c_int
        _BOUND = True
    return lb


@dataclass
class RefGeometry:
    """2D tracks with their own segment counts, as src/tracks.c:21-59 builds them."""
    seg_off: np.ndarray        # [N2D+1] int64
    seg_len: np.ndarray        # [M2D] float32
    az_weight: np.ndarray      # [N2D] float32
    p_weight: np.ndarray       # [N3D] float32
    z_height: np.ndarray       # [N3D] float32 (stacked-ray heights, updated by sweeps)
    axial_z_sep: float


def make_geometry(seed: int, n2d: int, n_polar: int, z_stacked: int, segments_per_track: float,
                  axial_z_sep: float, assembly_width: float = 21.42) -> RefGeometry:
    """Seeded geometry with the reference's distributions: segments per 2D track
    ~ N(spt, sqrt(spt)) (src/tracks.c:62-65), lengths U(0,1) * width / n
    (src/tracks.c:54), weights U(0,1), stacked rays starting at sep*k (upward)
    or sep*(k+1) (downward, src/tracks.c:126-129)."""
    rng = np.random.default_rng(seed)
    nseg = np.maximum(1, np.rint(rng.normal(segments_per_track, np.sqrt(segments_per_track),
                                            n2d))).astype(np.int64)
    off = np.zeros(n2d + 1, np.int64)
    off[1:] = np.cumsum(nseg)
    seg_len = np.concatenate([(rng.random(n) * assembly_width / n) for n in nseg]).astype(np.float32)
    az = rng.random(n2d).astype(np.float32)
    n3d = n2d * n_polar * z_stacked
    pw = rng.random(n3d).astype(np.float32)
    t = np.arange(n3d)
    k = (t % z_stacked).astype(np.float32)
    j = (t // z_stacked) % n_polar
    sep = np.float32(axial_z_sep)
    z = np.where(j < n_polar // 2, sep * k, sep * (k + np.float32(1))).astype(np.float32)
    return RefGeometry(off, seg_len, az, pw, z, float(axial_z_sep))


@dataclass
class RefProblem:
    """Params / Input in the reference layout over numpy storage."""
    input: Input
    params: Params
    fine_source: np.ndarray
    fine_flux: np.ndarray
    psi_f: np.ndarray
    psi_b: np.ndarray
    tracks: np.ndarray          # Track structs, [N3D]
    _keep: list = field(default_factory=list, repr=False)

    def z_heights(self) -> np.ndarray:
        return np.array([t.z_height for t in self.tracks], dtype=np.float32)


def _struct_array(ctype, n: int) -> tuple[np.ndarray, object]:
    """A zeroed numpy record array with the field offsets and size of the
    ctypes structure `ctype`, and the ctypes array view of the same memory."""
    names = [f[0] for f in ctype._fields_]
    fmt = {C.c_float: "<f4", C.c_long: "<i8", C.c_int: "<i4", C.c_bool: "u1"}
    formats = [fmt.get(f[1], "<u8") for f in ctype._fields_]     # pointers: 8-byte addresses
    offsets = [getattr(ctype, nm).offset for nm in names]
    dt = np.dtype({"names": names, "formats": formats, "offsets": offsets,
                   "itemsize": C.sizeof(ctype)})
    arr = np.zeros(max(1, n), dtype=dt)
    return arr, (ctype * max(1, n)).from_buffer(arr)


def build(hp, geo: RefGeometry, precision: float | None = None) -> RefProblem:
    """Reference-layout problem: sources / cross sections of the HostProblem
    `hp` (one sigma_t row per source, as src/source.c:150-152), 2D tracks and
    stacked rays of `geo`.  The structs are filled through numpy views of
    their memory (millions of tracks at the default sizes)."""
    s = hp.spec
    G, F, NS, P = s.n_groups, s.fai, s.n_sources, s.n_polar
    N2D = len(geo.seg_off) - 1
    Z = len(geo.z_height) // (N2D * P)
    keep = []
    q = hp.fine_source.astype(np.float32, copy=True)
    phi = np.zeros_like(q)
    psi_f = np.zeros(N2D * P * Z * G, np.float32)
    psi_b = np.zeros_like(psi_f)
    sigt_rows = np.ascontiguousarray(hp.sigt.reshape(-1, G)[hp.src_sigt])   # [NS][G]
    xs3 = np.ascontiguousarray(hp.xs.reshape(-1, G, 3))
    sc = np.ascontiguousarray(hp.scatter.reshape(-1, G, G))
    n_xs = xs3.shape[0]
    # row pointer tables: XS[m][g] -> 3 floats, scatter[m][g] -> G floats
    xs_rows = xs3.ctypes.data + 12 * np.arange(n_xs * G, dtype=np.uint64)
    sc_rows = sc.ctypes.data + 4 * G * np.arange(n_xs * G, dtype=np.uint64)
    q_rows = q.ctypes.data + 4 * G * np.arange(NS * F, dtype=np.uint64)
    f_rows = phi.ctypes.data + 4 * G * np.arange(NS * F, dtype=np.uint64)
    src_arr, sources = _struct_array(Source, NS)
    i = np.arange(NS, dtype=np.uint64)
    m = hp.src_xs.astype(np.uint64)
    src_arr["fine_source"] = q_rows.ctypes.data + 8 * F * i
    src_arr["fine_flux"] = f_rows.ctypes.data + 8 * F * i
    src_arr["vol"] = hp.vol
    src_arr["sigT"] = sigt_rows.ctypes.data + 4 * G * i
    src_arr["XS"] = xs_rows.ctypes.data + 8 * G * m
    src_arr["scattering_matrix"] = sc_rows.ctypes.data + 8 * G * m
    seg_arr, segs = _struct_array(Segment, int(geo.seg_off[-1]))
    seg_arr["length"][:len(geo.seg_len)] = geo.seg_len
    t2d_arr, t2d = _struct_array(Track2D, N2D)
    t2d_arr["az_weight"] = geo.az_weight
    t2d_arr["n_segments"] = np.diff(geo.seg_off)
    t2d_arr["segments"] = C.addressof(segs) + C.sizeof(Segment) * geo.seg_off[:-1].astype(np.uint64)
    n3d = N2D * P * Z
    trk_arr, tracks = _struct_array(Track, n3d)
    t = np.arange(n3d, dtype=np.uint64)
    trk_arr["p_weight"] = geo.p_weight
    trk_arr["z_height"] = geo.z_height
    trk_arr["f_psi"] = psi_f.ctypes.data + 4 * G * t
    trk_arr["b_psi"] = psi_b.ctypes.data + 4 * G * t
    rows = C.addressof(tracks) + C.sizeof(Track) * Z * np.arange(N2D * P, dtype=np.uint64)
    tr3 = rows.ctypes.data + 8 * P * np.arange(N2D, dtype=np.uint64)
    keep += [src_arr, seg_arr, t2d_arr, trk_arr]
    leak = (C.c_float * 1)(0.0)
    polar = np.ascontiguousarray(hp.polar_angles, dtype=np.float32)
    table = np.ascontiguousarray(hp.table, dtype=np.float32)
    prm = Params(tracks_2D=C.cast(t2d, C.POINTER(Track2D)),
                 tracks=C.cast(C.c_void_p(tr3.ctypes.data), C.POINTER(C.POINTER(C.POINTER(Track)))),
                 sources=C.cast(sources, C.POINTER(Source)), polar_angles=polar.ctypes.data_as(fp),
                 leakage=C.cast(leak, fp),
                 expTable=Table(values=table.ctypes.data_as(fp), dx=hp.table_dx,
                                maxVal=hp.table_maxval, N=hp.table_n))
    inp = Input()
    inp.cai, inp.fai, inp.axial_exp = s.cai, F, s.axial_exp
    inp.axial_z_sep = geo.axial_z_sep
    inp.n_polar_angles, inp.n_egroups = P, G
    inp.decomp_assemblies_ax = s.decomp_ax
    inp.height = s.height
    inp.precision = s.precision if precision is None else precision
    inp.mype = 1
    inp.ntracks_2D, inp.z_stacked, inp.ntracks = N2D, Z, n3d
    inp.n_source_regions_per_node = NS
    keep += [xs_rows, sc_rows, q_rows, f_rows, sources, sigt_rows, segs, t2d, rows, tr3, leak,
             polar, table, hp, geo, xs3, sc]
    return RefProblem(input=inp, params=prm, fine_source=q, fine_flux=phi, psi_f=psi_f,
                      psi_b=psi_b, tracks=tracks, _keep=keep)
