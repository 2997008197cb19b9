"""OpenMOC track files (src/tracks.c:170-323): the library's reader against the
reference's own load_OpenMOC_tracks (oracle/_ref, where the reference was
built) on files in the track-file layout, with and without CMFD data, and the
reader's rejection of short or inconsistent files (the reference does not
check them)."""
import struct

import numpy as np
import pytest

import oracle


def _file(tmp_path, seed=3, cmfd=False, **kw):
    from simplemoc_gb300 import openmoc
    t, len64 = openmoc.synthetic(seed, **kw)
    path = tmp_path / f"tracks_{seed}_{int(cmfd)}.bin"
    surf = None
    if cmfd:
        surf = np.random.default_rng(seed).integers(-1, 50, (int(t.seg_off[-1]), 2)).astype(np.int32)
    openmoc.write(path, t, cmfd_surfaces=surf, seg_len64=len64)
    return path, t, len64


@pytest.mark.parametrize("cmfd", [False, True])
def test_reader_round_trip(lib, tmp_path, cmfd):
    from simplemoc_gb300 import openmoc
    path, t, len64 = _file(tmp_path, cmfd=cmfd)
    r = openmoc.read(path, cmfd=cmfd)
    assert r.n_azimuthal == t.n_azimuthal and r.n_tracks_2d == t.n_tracks_2d
    assert r.spacing == t.spacing
    for k in ("num_tracks", "num_x", "num_y", "azim_weights", "track_geometry", "azim_index",
              "seg_off", "material_id", "region_id"):
        assert np.array_equal(getattr(r, k), getattr(t, k)), k
    assert np.array_equal(r.seg_len, len64.astype(np.float32))


@pytest.mark.parametrize("cmfd,seed,n_az,tpa", [(False, 3, 4, 3), (True, 4, 6, 5),
                                                 (False, 5, 1, 1), (True, 6, 8, 2)])
def test_reader_matches_reference_loader(lib, ref, tmp_path, cmfd, seed, n_az, tpa):
    from simplemoc_gb300 import openmoc
    path, t, _ = _file(tmp_path, seed=seed, cmfd=cmfd, n_azimuthal=n_az, tracks_per_angle=tpa)
    mine = openmoc.read(path, cmfd=cmfd)
    theirs = ref.load_openmoc(path, cmfd=cmfd)
    assert theirs["n_tracks_2d"] == mine.n_tracks_2d
    assert theirs["n_azimuthal"] == mine.n_azimuthal
    assert theirs["radial_ray_sep"] == np.float32(mine.spacing)
    assert theirs["segments_per_track"] == mine.segments_per_track
    assert np.array_equal(theirs["n_segments"], np.diff(mine.seg_off))
    assert np.array_equal(theirs["lengths"], mine.seg_len)           # bit for bit
    assert np.array_equal(theirs["source_ids"], mine.region_id.astype(np.int64))


def test_reader_rejects_bad_files(lib, tmp_path):
    from simplemoc_gb300 import MocError, openmoc
    path, t, _ = _file(tmp_path, seed=7)
    data = path.read_bytes()
    bad = tmp_path / "bad.bin"
    # truncated anywhere after the header
    for cut in (3, 30, len(data) // 2, len(data) - 1):
        bad.write_bytes(data[:cut])
        with pytest.raises(MocError):
            openmoc.read(bad)
    # the CMFD flag on a file without CMFD data runs past the end
    with pytest.raises(MocError):
        openmoc.read(path, cmfd=True)
    # trailing bytes are ignored, as the reference ignores them
    bad.write_bytes(data + b"\0" * 8)
    assert openmoc.read(bad).n_tracks_2d == t.n_tracks_2d
    # a negative segment count, a negative track count, an absurd string length
    geo_len = struct.unpack("=i", data[:4])[0]
    hdr = 4 + geo_len + 4 + 8
    n_az = t.n_azimuthal
    first_track = hdr + n_az * (4 * 3 + 8)
    b = bytearray(data)
    b[first_track + 44:first_track + 48] = struct.pack("=i", -5)
    bad.write_bytes(bytes(b))
    with pytest.raises(MocError):
        openmoc.read(bad)
    b = bytearray(data)
    b[hdr:hdr + 4] = struct.pack("=i", -1)
    bad.write_bytes(bytes(b))
    with pytest.raises(MocError):
        openmoc.read(bad)
    b = bytearray(data)
    b[0:4] = struct.pack("=i", 1 << 30)
    bad.write_bytes(bytes(b))
    with pytest.raises(MocError):
        openmoc.read(bad)
    with pytest.raises(MocError):
        openmoc.read(tmp_path / "missing.bin")


def test_geometry_from_track_file(lib, tmp_path):
    from simplemoc_gb300 import openmoc
    path, t, _ = _file(tmp_path, seed=8)
    r = openmoc.read(path)
    g = openmoc.to_geometry(r, n_polar=4, z_stacked=5, axial_z_sep=0.5, seed=1)
    assert np.array_equal(g.seg_off, r.seg_off) and np.array_equal(g.seg_len, r.seg_len)
    assert g.p_weight.size == r.n_tracks_2d * 4 * 5
    gf = openmoc.to_geometry(r, n_polar=4, z_stacked=5, axial_z_sep=0.5, az_weight="file")
    assert np.array_equal(gf.az_weight, r.azim_weights[r.azim_index].astype(np.float32))


def test_reader_rejects_every_truncation_and_survives_corruption(lib, tmp_path):
    """Every proper prefix of a track file is rejected, and files with one
    4-byte field overwritten (counts, ids or parts of doubles) are either read
    or rejected, never read out of bounds."""
    import struct

    from simplemoc_gb300 import MocError, openmoc
    path, t, _ = _file(tmp_path, seed=7, n_azimuthal=3, tracks_per_angle=2)
    data = path.read_bytes()
    bad = tmp_path / "bad.bin"
    for cut in range(len(data)):
        bad.write_bytes(data[:cut])
        with pytest.raises(MocError):
            openmoc.read(bad)
    rng = np.random.default_rng(1)
    values = [-1, 0, 1, 7, 1 << 20, -(1 << 30), (1 << 31) - 1]
    for _ in range(1000):
        b = bytearray(data)
        off = int(rng.integers(0, len(data) - 4))
        b[off:off + 4] = struct.pack("=i", values[int(rng.integers(len(values)))])
        bad.write_bytes(bytes(b))
        try:
            r = openmoc.read(bad)
        except MocError:
            continue
        assert r.seg_off[-1] == r.seg_len.size and np.all(np.diff(r.seg_off) >= 0)
