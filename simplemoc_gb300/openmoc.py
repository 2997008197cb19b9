"""OpenMOC track files (the reference's -d input, src/tracks.c:170-323).

`read` parses a file through the library's bounds-checked reader
(moc_openmoc_probe / moc_openmoc_read); `write` produces the same binary
layout (for tests and for exporting tracks); `to_geometry` turns the 2D tracks
into the reference traversal's input (refabi.RefGeometry), which the drop-in
transport_sweep runs on the GPU.
"""
from __future__ import annotations

import ctypes as C
import struct
from dataclasses import dataclass

import numpy as np

from . import _lib as L


@dataclass
class OpenMOCTracks:
    geometry: bytes             # the geometry string (read back by write only)
    spacing: float
    num_tracks: np.ndarray      # [n_az] int32
    num_x: np.ndarray
    num_y: np.ndarray
    azim_weights: np.ndarray    # [n_az] float64
    track_geometry: np.ndarray  # [N2D, 5] float64: x0, y0, x1, y1, phi
    azim_index: np.ndarray      # [N2D] int32
    seg_off: np.ndarray         # [N2D+1] int64
    seg_len: np.ndarray         # [M] float32 (the reference converts to float)
    material_id: np.ndarray     # [M] int32
    region_id: np.ndarray       # [M] int32

    @property
    def n_azimuthal(self) -> int:
        return int(self.num_tracks.size)

    @property
    def n_tracks_2d(self) -> int:
        return int(self.seg_off.size - 1)

    @property
    def segments_per_track(self) -> int:
        """As the reference recomputes it (src/tracks.c:313): integer mean."""
        return int(self.seg_off[-1]) // max(1, self.n_tracks_2d)


def read(path: str, cmfd: bool = False) -> OpenMOCTracks:
    lib = L._lib()
    p = str(path).encode()
    n_az, nt, ns = C.c_int32(), C.c_int64(), C.c_int64()
    sp = C.c_double()
    L.check(lib.moc_openmoc_probe(p, int(cmfd), C.byref(n_az), C.byref(sp), C.byref(nt),
                                  C.byref(ns)), "moc_openmoc_probe")
    a, n, m = n_az.value, nt.value, ns.value
    out = OpenMOCTracks(
        geometry=b"", spacing=sp.value,
        num_tracks=np.empty(a, np.int32), num_x=np.empty(a, np.int32),
        num_y=np.empty(a, np.int32), azim_weights=np.empty(a, np.float64),
        track_geometry=np.empty((n, 5), np.float64), azim_index=np.empty(n, np.int32),
        seg_off=np.empty(n + 1, np.int64), seg_len=np.empty(m, np.float32),
        material_id=np.empty(m, np.int32), region_id=np.empty(m, np.int32))
    ptr = lambda x: x.ctypes.data if x.size else None
    L.check(lib.moc_openmoc_read(p, int(cmfd), n, m, ptr(out.num_tracks), ptr(out.num_x),
                                 ptr(out.num_y), ptr(out.azim_weights), ptr(out.track_geometry),
                                 ptr(out.azim_index), ptr(out.seg_off), ptr(out.seg_len),
                                 ptr(out.material_id), ptr(out.region_id)), "moc_openmoc_read")
    return out


def write(path: str, t: OpenMOCTracks, cmfd_surfaces: np.ndarray | None = None,
          seg_len64: np.ndarray | None = None) -> None:
    """Writes `t` in the track-file layout.  seg_len64 (float64) replaces the
    float lengths when given; cmfd_surfaces [M, 2] int32 adds the CMFD ids."""
    lens = np.asarray(seg_len64 if seg_len64 is not None else t.seg_len, np.float64)
    with open(path, "wb") as f:
        f.write(struct.pack("=i", len(t.geometry)) + t.geometry)
        f.write(struct.pack("=id", t.n_azimuthal, t.spacing))
        for arr, fmt in ((t.num_tracks, "i"), (t.num_x, "i"), (t.num_y, "i"),
                         (t.azim_weights, "d")):
            f.write(np.asarray(arr, "=" + fmt).tobytes())
        for k in range(t.n_tracks_2d):
            f.write(np.asarray(t.track_geometry[k], "=f8").tobytes())
            a, b = int(t.seg_off[k]), int(t.seg_off[k + 1])
            f.write(struct.pack("=ii", int(t.azim_index[k]), b - a))
            rec = [("len", "=f8"), ("mat", "=i4"), ("reg", "=i4")]
            if cmfd_surfaces is not None:
                rec += [("fwd", "=i4"), ("bwd", "=i4")]
            segs = np.empty(b - a, dtype=np.dtype(rec))
            segs["len"] = lens[a:b]
            segs["mat"] = t.material_id[a:b]
            segs["reg"] = t.region_id[a:b]
            if cmfd_surfaces is not None:
                segs["fwd"] = cmfd_surfaces[a:b, 0]
                segs["bwd"] = cmfd_surfaces[a:b, 1]
            f.write(segs.tobytes())


def synthetic(seed: int, n_azimuthal: int = 4, tracks_per_angle: int = 3,
              segments_per_track: float = 20.0, width: float = 21.42, n_regions: int = 100,
              geometry: bytes = b"synthetic geometry") -> tuple[OpenMOCTracks, np.ndarray]:
    """A seeded track set in the file's terms (float64 lengths returned beside)."""
    rng = np.random.default_rng(seed)
    num = np.full(n_azimuthal, tracks_per_angle, np.int32)
    n2d = int(num.sum())
    nseg = np.maximum(1, np.rint(rng.normal(segments_per_track, np.sqrt(segments_per_track),
                                            n2d))).astype(np.int64)
    off = np.zeros(n2d + 1, np.int64)
    off[1:] = np.cumsum(nseg)
    m = int(off[-1])
    len64 = rng.random(m) * width / np.repeat(nseg, nseg)
    phis = np.pi * (np.arange(n_azimuthal) + 0.5) / n_azimuthal
    geo = np.column_stack([rng.random((n2d, 4)) * width,
                           np.repeat(phis, tracks_per_angle)]).astype(np.float64)
    t = OpenMOCTracks(
        geometry=geometry, spacing=float(width / (tracks_per_angle + 1)), num_tracks=num,
        num_x=rng.integers(1, 5, n_azimuthal).astype(np.int32),
        num_y=rng.integers(1, 5, n_azimuthal).astype(np.int32),
        azim_weights=rng.random(n_azimuthal), track_geometry=geo,
        azim_index=np.repeat(np.arange(n_azimuthal, dtype=np.int32), tracks_per_angle),
        seg_off=off, seg_len=len64.astype(np.float32),
        material_id=rng.integers(0, 8, m).astype(np.int32),
        region_id=rng.integers(0, n_regions, m).astype(np.int32))
    return t, len64


def to_geometry(t: OpenMOCTracks, n_polar: int, z_stacked: int, axial_z_sep: float,
                seed: int = 0, az_weight: str = "uniform"):
    """The reference traversal's input for these 2D tracks: P polar angles and
    Z stacked rays per 2D track, stacked-ray heights as src/tracks.c:126-129.
    az_weight "uniform": seeded U(0,1) per track, as the reference's loader
    does (src/tracks.c:289); "file": the track's azimuthal quadrature weight."""
    from .refabi import RefGeometry
    rng = np.random.default_rng(seed)
    n2d = t.n_tracks_2d
    if az_weight == "file":
        az = t.azim_weights[t.azim_index].astype(np.float32)
    else:
        az = rng.random(n2d).astype(np.float32)
    n3d = n2d * n_polar * z_stacked
    pw = rng.random(n3d).astype(np.float32)
    k = (np.arange(n3d) % z_stacked).astype(np.float32)
    j = (np.arange(n3d) // z_stacked) % n_polar
    sep = np.float32(axial_z_sep)
    z = np.where(j < n_polar // 2, sep * k, sep * (k + np.float32(1))).astype(np.float32)
    return RefGeometry(t.seg_off.astype(np.int64), t.seg_len.astype(np.float32), az, pw, z,
                       float(axial_z_sep))
