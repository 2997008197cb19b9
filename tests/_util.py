"""Shared helpers for the test-suite."""
from __future__ import annotations

from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
GOLDEN_CASES = sorted(p.stem for p in GOLDEN.glob("*.npz"))


def load_golden(name: str):
    """(HostProblem, fixture dict) for tests/golden/<name>.npz."""
    import simplemoc_gb300 as sm
    z = dict(np.load(GOLDEN / f"{name}.npz"))
    fields = {k[5:]: z[k].item() for k in z if k.startswith("spec_")}
    spec = sm.ProblemSpec(**fields)
    hp = sm.HostProblem(
        spec=spec, seg_len=z["seg_len"], seg_src=z["seg_src"], az_weight=z["az_weight"],
        p_weight=z["p_weight"], z0=z["z0"], polar_angles=z["polar_angles"],
        src_sigt=z["src_sigt"], src_xs=z["src_xs"], vol=z["vol"], sigt=z["sigt"], xs=z["xs"],
        scatter=z["scatter"], fine_source=z["fine_source"], fine_flux=None, psi_f=None,
        psi_b=None, table=z["table"], table_dx=float(z["table_dx"]),
        table_maxval=float(z["table_maxval"]), table_n=int(z["table_n"]))
    return hp, z


def rel_err(a, b) -> float:
    """Normwise max relative error max|a-b| / max|b|."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.abs(b).max()
    return float(np.abs(a - b).max() / (den if den > 0 else 1.0))


def elem_rel_err(a, b, floor_frac: float = 1e-3) -> float:
    """Max per-element relative error over elements with |b| >= floor_frac*max|b|."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    m = np.abs(b) >= floor_frac * np.abs(b).max()
    if not m.any():
        return 0.0
    return float((np.abs(a - b)[m] / np.abs(b)[m]).max())
