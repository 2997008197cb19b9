"""The reference traversal (src/solver.c:347-523): the oracle's restatement
against the reference's own transport_sweep, and the drop-in build of the
reference driver against libsimplemoc_gb300.so (CPU)."""
import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle

LIBC = C.CDLL(None)
ROOT = Path(__file__).resolve().parent.parent


def _case(axial_exp, seed, n2d=6, n_polar=4, sep=0.5, height=40.0, groups=12, spt=30):
    import simplemoc_gb300 as sm
    from simplemoc_gb300 import refabi
    z = int(height / sep)
    spec = sm.ProblemSpec(n_groups=groups, fai=5, cai=4, height=height, n_sources=60,
                          n_tracks_2d=n2d, n_polar=n_polar, z_stacked=z, n_seg=10,
                          axial_exp=axial_exp, seed=seed)
    hp = sm.generate(spec)
    geo = refabi.make_geometry(seed + 1, n2d, n_polar, z, spt, sep)
    return hp, geo


@pytest.mark.parametrize("axial_exp,seed,n_polar,sep", [(2, 1, 4, 0.5), (0, 2, 4, 0.5),
                                                         (2, 3, 6, 0.25), (2, 4, 2, 1.0)])
def test_oracle_traversal_matches_reference_transport_sweep(port, ref, lib, axial_exp, seed,
                                                            n_polar, sep):
    """Three consecutive sweeps under the same srand seeds: sub-segment count,
    stacked-ray heights, angular and scalar fluxes are bit-identical."""
    hp, geo = _case(axial_exp, seed, n_polar=n_polar, sep=sep)
    rg = oracle.make_refgeo(geo)
    op = oracle.make_problem(hp)
    st_r, st_o = oracle.fresh_state(hp), oracle.fresh_state(hp)
    z_r, z_o = geo.z_height.copy(), geo.z_height.copy()
    for sweep in range(3):
        LIBC.srand(100 + seed * 10 + sweep)
        n_r = ref.transport_sweep(hp, st_r, rg, z_r)
        LIBC.srand(100 + seed * 10 + sweep)
        n_o = port.ref_sweep(op, rg, st_o["fine_source"], st_o["fine_flux"], st_o["psi_f"], z_o)
        assert n_r == n_o > 0
        assert np.array_equal(z_r, z_o)
        assert np.array_equal(st_r["psi_f"], st_o["psi_f"])
        assert np.array_equal(st_r["fine_flux"], st_o["fine_flux"])


@pytest.mark.parametrize("case", [
    # one 2D track of one segment, one stacked ray per polar angle, one group
    dict(axial_exp=2, seed=21, n2d=1, n_polar=2, sep=40.0, groups=1, spt=1),
    # two stacked rays per polar angle along a 200-segment 2D track
    dict(axial_exp=2, seed=22, n2d=1, n_polar=2, sep=20.0, groups=3, spt=200),
    # 400 stacked rays, 8 polar angles, flat source
    dict(axial_exp=0, seed=23, n2d=3, n_polar=8, sep=0.1, groups=5, spt=5),
    dict(axial_exp=2, seed=24, n2d=2, n_polar=4, sep=0.5, groups=128, spt=40),
])
def test_oracle_traversal_matches_reference_at_edge_sizes(port, ref, lib, case):
    hp, geo = _case(**case)
    rg = oracle.make_refgeo(geo)
    op = oracle.make_problem(hp)
    st_r, st_o = oracle.fresh_state(hp), oracle.fresh_state(hp)
    z_r, z_o = geo.z_height.copy(), geo.z_height.copy()
    for sweep in range(3):
        LIBC.srand(500 + sweep)
        n_r = ref.transport_sweep(hp, st_r, rg, z_r)
        LIBC.srand(500 + sweep)
        n_o = port.ref_sweep(op, rg, st_o["fine_source"], st_o["fine_flux"], st_o["psi_f"], z_o)
        assert n_r == n_o > 0
        assert np.array_equal(z_r, z_o)
        assert np.array_equal(st_r["psi_f"], st_o["psi_f"])
        assert np.array_equal(st_r["fine_flux"], st_o["fine_flux"])


def test_traversal_with_given_ids_equals_libc_draws(port, lib):
    """ids[] in traversal order reproduce the rand() draws exactly."""
    hp, geo = _case(2, 9)
    rg = oracle.make_refgeo(geo)
    op = oracle.make_problem(hp)
    a, b = oracle.fresh_state(hp), oracle.fresh_state(hp)
    za, zb = geo.z_height.copy(), geo.z_height.copy()
    LIBC.srand(77)
    n = port.ref_sweep(op, rg, a["fine_source"], a["fine_flux"], a["psi_f"], za)
    LIBC.srand(77)
    ids = np.array([LIBC.rand() % hp.spec.n_sources for _ in range(n)], dtype=np.int32)
    m = port.ref_sweep(op, rg, b["fine_source"], b["fine_flux"], b["psi_f"], zb, ids)
    assert n == m
    assert np.array_equal(a["psi_f"], b["psi_f"]) and np.array_equal(za, zb)


def test_reference_driver_links_against_the_library(tmp_path, lib):
    """src/main.c, io.c, init.c, tracks.c, source.c, utils.c of the reference link
    against libsimplemoc_gb300.so in place of solver.o, unchanged, and the
    driver runs to its summary; without a GPU every solver call reports
    MOC_ERR_NO_DEVICE through moc_ref_status and keff is NaN (no CPU fallback)."""
    src = oracle.ref_src()
    if src is None or not (src / "main.c").exists():
        pytest.skip("reference sources not mounted")
    libdir = ROOT / "simplemoc_gb300"
    exe = tmp_path / "SimpleMOC_gpu"
    files = [str(src / f) for f in ("main.c", "io.c", "init.c", "tracks.c", "source.c", "utils.c")]
    subprocess.run(["gcc", "-std=gnu99", "-O1", f"-I{src}", *files, f"-L{libdir}",
                    "-lsimplemoc_gb300", f"-Wl,-rpath,{libdir}", "-lm", "-o", str(exe)],
                   check=True, capture_output=True)
    # a tiny problem in the reference's input-file format (src/io.c:198-270)
    vals = ["1", "1", "2", "3", "2", "2.0", "4.0", "4", "2", "4", "0", "1", "5", "21.42", "40.0",
            "0.01", "20", "0"]
    inp = tmp_path / "tiny.in"
    inp.write_text("".join(f"{v} - value\n" for v in vals))
    import torch
    res = subprocess.run([str(exe), "-i", str(inp)], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stderr
    assert "keff =" in res.stdout
    if not torch.cuda.is_available():
        assert "keff = nan" in res.stdout or "keff = -nan" in res.stdout
