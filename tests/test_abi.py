"""CPU tests of the C ABI: the library loads, exports every declared symbol,
validates inputs before touching a device, and generates reproducibly."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*"
                            r"([A-Za-z_][A-Za-z0-9_]*)\s*\(", text, flags=re.M)
    return sorted(set(n for n in names if not n.startswith("_")))


def declared_functions_in(header: str):
    text = re.sub(r"/\*.*?\*/", "", (ROOT / "include" / header).read_text(), flags=re.S)
    return re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*"
                      r"([A-Za-z_][A-Za-z0-9_]*)\s*\(", text, flags=re.M)


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_every_declared_symbol(lib):
    from simplemoc_gb300 import _lib as L
    from simplemoc_gb300 import refabi
    refabi.lib()
    # the flat ABI is bound in _lib.SIGNATURES, the reference-signature entry
    # points (include/simplemoc_refabi.h) by simplemoc_gb300.refabi
    ref_names = set(declared_functions_in("simplemoc_refabi.h"))
    missing = []
    for n in declared_functions():
        if n in ref_names:
            if getattr(lib, n).argtypes is None:
                missing.append(n)
        elif n not in L.SIGNATURES:
            missing.append(n)
    assert not missing, missing


def test_status_strings(lib):
    assert lib.moc_status_string(0) == b"ok"
    assert b"argument" in lib.moc_status_string(1)
    assert lib.moc_status_string(999) == b"unknown status"


def test_generator_deterministic_and_thread_independent(lib, monkeypatch):
    import simplemoc_gb300 as sm
    spec = sm.ProblemSpec(n_groups=10, n_sources=100, n_tracks_2d=32, n_polar=4, z_stacked=6,
                          n_seg=20, seed=42)
    a = sm.generate(spec)
    b = sm.generate(spec)
    for k in ("seg_len", "seg_src", "p_weight", "z0", "sigt", "xs", "scatter", "fine_source"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    c = sm.generate(spec.with_(seed=43))
    assert not np.array_equal(a.seg_src, c.seg_src)


def test_generator_distributions(lib):
    """The synthetic inputs follow the stated distributions."""
    import simplemoc_gb300 as sm
    spec = sm.ProblemSpec(n_groups=50, n_sources=2000, n_tracks_2d=64, n_polar=4, z_stacked=10,
                          n_seg=50, seed=1)
    p = sm.generate(spec)
    assert p.seg_len.min() >= 0.05 and p.seg_len.max() < 1.5
    assert abs(p.seg_len.mean() - 0.775) < 0.01
    assert p.seg_src.min() >= 0 and p.seg_src.max() < spec.n_sources
    counts = np.bincount(p.seg_src, minlength=spec.n_sources)
    assert counts.min() > 0.5 * counts.mean()
    assert p.sigt.min() >= 0.1 and p.sigt.max() < 2.0
    S = p.scatter.reshape(8, 50, 50)
    np.testing.assert_allclose(S.sum(axis=2), 0.7, rtol=1e-5)
    X = p.xs.reshape(8, 50, 3)
    assert np.all(X[4:, :, 0] == 0) and X[:4, :, 0].max() < 0.05
    np.testing.assert_allclose(X[:, :, 1], 0.3 * p.sigt.reshape(8, 50), rtol=1e-6)
    np.testing.assert_allclose(X[:, :, 2].sum(axis=1), 1.0, rtol=1e-5)
    assert p.vol.min() >= 0.5 and p.vol.max() < 1.5
    th = (np.arange(4) + 0.5) * np.pi / 4
    np.testing.assert_array_equal(p.polar_angles, th.astype(np.float32))
    # upward stacks start at sep*k, downward at sep*(k+1)
    z = p.z0.reshape(64, 4, 10)
    sep = np.float32(200.0) / np.float32(10)
    np.testing.assert_array_equal(z[0, 0], (sep * np.arange(10, dtype=np.float32)))
    np.testing.assert_array_equal(z[0, 3], (sep * np.arange(1, 11, dtype=np.float32)))


def _create(lib, hp):
    from simplemoc_gb300 import _lib as L
    dims, host = hp.dims(), hp.host()
    h = C.c_void_p()
    return lib.moc_create(C.byref(dims), C.byref(host), 0, C.byref(h)), h


@pytest.mark.parametrize("field,value", [("seg_src", -1), ("seg_src", 10**6), ("src_xs", 9),
                                         ("sigt", 0.0), ("seg_len", np.nan), ("vol", 0.0)])
def test_create_rejects_bad_inputs_before_device(lib, field, value):
    """Index and domain checks run on the host, before any device call."""
    import simplemoc_gb300 as sm
    spec = sm.ProblemSpec(n_groups=8, n_sources=30, n_tracks_2d=4, n_polar=2, z_stacked=3,
                          n_seg=10, seed=3)
    hp = sm.generate(spec)
    arr = getattr(hp, field).copy()
    arr[len(arr) // 2] = value
    setattr(hp, field, arr)
    rc, _ = _create(lib, hp)
    assert rc == 1        # MOC_ERR_ARG


@pytest.mark.parametrize("field,value", [("n_tracks_2d", 1 << 45), ("n_groups", 1 << 30)])
def test_create_rejects_sizes_beyond_64bit_counts(lib, field, value):
    """Dimensions whose array lengths or byte counts would overflow 64-bit
    integers are rejected before any array is read."""
    import simplemoc_gb300 as sm
    spec = sm.ProblemSpec(n_groups=8, n_sources=30, n_tracks_2d=4, n_polar=2, z_stacked=3,
                          n_seg=10, seed=3)
    hp = sm.generate(spec)
    dims, host = hp.dims(), hp.host()
    setattr(dims, field, value)
    h = C.c_void_p()
    assert lib.moc_create(C.byref(dims), C.byref(host), 0, C.byref(h)) == 1    # MOC_ERR_ARG


def test_create_rejects_too_few_fine_intervals(lib):
    import simplemoc_gb300 as sm
    spec = sm.ProblemSpec(n_groups=8, fai=2, n_sources=30, n_tracks_2d=4, n_polar=2,
                          z_stacked=3, n_seg=10, seed=3)
    rc, _ = _create(lib, sm.generate(spec))
    assert rc == 1


def test_create_without_gpu_reports_no_device(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import simplemoc_gb300 as sm
    spec = sm.ProblemSpec(n_groups=8, n_sources=30, n_tracks_2d=4, n_polar=2, z_stacked=3,
                          n_seg=10, seed=3)
    rc, _ = _create(lib, sm.generate(spec))
    assert rc == 7        # MOC_ERR_NO_DEVICE, never a CPU fallback


def test_solver_raises_loudly_without_gpu(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import simplemoc_gb300 as sm
    spec = sm.ProblemSpec(n_groups=8, n_sources=30, n_tracks_2d=4, n_polar=2, z_stacked=3,
                          n_seg=10, seed=3)
    with pytest.raises(sm.MocError):
        sm.Solver(sm.generate(spec))


def test_algorithmic_bytes_of_the_default_problems(lib):
    """The roofline numerator: 20 B per integration (12 B flat), 8 B per
    track-group, 4 B per 3D segment id and 4 B per (2D segment, polar angle)
    length.  The default problem moves 1.3239e12 B per sweep."""
    import simplemoc_gb300 as sm
    d = sm.CONFIGS["default"]
    assert d.n_tracks_3d == 13_107_200 and d.n_seg == 50 and d.n_groups == 100
    ints = d.n_tracks_3d * d.n_seg * d.n_groups
    extra = 8 * d.n_tracks_3d * d.n_groups + 4 * d.n_tracks_3d * d.n_seg \
        + 4 * d.n_tracks_2d * d.n_polar * d.n_seg
    assert d.algorithmic_bytes() == 20 * ints + extra == 1_323_859_968_000
    f = sm.CONFIGS["flat"]
    assert f.axial_exp == 0 and f.algorithmic_bytes() == 12 * ints + extra
