"""Generates the golden fixtures of tests/golden/ from the reference itself.

    python tests/golden/make_golden.py

Runs the reference's own compiled solver (oracle/_ref/libref_harness.so, built
from the mounted reference sources by oracle/Makefile) over small seeded
problems and stores inputs and outputs in compressed .npz files:

  * after one transport sweep: fine_flux, psi_f
  * after N power iterations (sweep, renormalize_flux, update_sources,
    compute_keff as src/main.c:57-92): fine_flux, fine_source, psi_f, psi_b,
    and the (keff, residual) history

The reference has no tests, fixtures or golden vectors of its own, so these
files pin the CPU restatement (oracle/moc_oracle.c) to the reference's objects.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
import simplemoc_gb300 as sm  # noqa: E402

HERE = Path(__file__).resolve().parent

CASES = {
    # quadratic source, groups a multiple of 4
    "quad_g12": sm.ProblemSpec(n_groups=12, fai=5, cai=4, height=200.0, n_sources=40,
                               n_tracks_2d=6, n_polar=4, z_stacked=5, n_seg=50, seed=101),
    # quadratic source, ragged groups (padding path), three fine intervals, 6 polar
    "quad_g7_f3": sm.ProblemSpec(n_groups=7, fai=3, cai=3, height=90.0, n_sources=30,
                                 n_tracks_2d=5, n_polar=6, z_stacked=4, n_seg=37, seed=202),
    # flat source (axial_exp 0, attenuate_FSR_fluxes)
    "flat_g10": sm.ProblemSpec(n_groups=10, fai=4, cai=2, height=120.0, n_sources=24,
                               n_tracks_2d=4, n_polar=2, z_stacked=6, n_seg=20, axial_exp=0,
                               seed=303),
}
ITERS = 3

INPUT_KEYS = ["seg_len", "seg_src", "az_weight", "p_weight", "z0", "polar_angles", "src_sigt",
              "src_xs", "vol", "sigt", "xs", "scatter", "fine_source", "table"]


def make(name: str, spec: sm.ProblemSpec) -> Path:
    hp = sm.generate(spec)
    ref = oracle.Reference()
    st = oracle.fresh_state(hp)
    ref.iterate(hp, st, 1, sweep_only=True)
    sweep1 = {"sweep1_fine_flux": st["fine_flux"].copy(), "sweep1_psi_f": st["psi_f"].copy()}
    st = oracle.fresh_state(hp)
    hist = ref.iterate(hp, st, ITERS)
    spec_fields = {f"spec_{k}": np.asarray(v) for k, v in spec.__dict__.items()}
    out = HERE / f"{name}.npz"
    np.savez_compressed(
        out, **{k: getattr(hp, k) for k in INPUT_KEYS},
        table_dx=np.float32(hp.table_dx), table_maxval=np.float32(hp.table_maxval),
        table_n=np.int32(hp.table_n), **spec_fields, **sweep1,
        iters=np.int32(ITERS), hist=np.asarray(hist, dtype=np.float64),
        **{f"final_{k}": v for k, v in st.items()})
    return out


if __name__ == "__main__":
    oracle.build(reference=True)
    for n, s in CASES.items():
        p = make(n, s)
        print(p, p.stat().st_size, "bytes")
