"""Python binding of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and the CPU-baseline legs of bench.py may
import this package; the product never does.  Two libraries:

  port       oracle/_build/libmoc_oracle.so: the C restatement (moc_oracle.c)
  reference  oracle/_ref/libref_harness.so: the reference's own solver objects
             driven over the same explicit segment streams (built only where the
             reference sources are mounted)

Problems are passed duck-typed: any object with the array attributes of
simplemoc_gb300.problem.HostProblem (numpy, C-contiguous).
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
PORT_LIB = HERE / "_build" / "libmoc_oracle.so"
# the same restatement built with the reference's timing flags (-Ofast
# -ffast-math -ftree-vectorize -fopenmp): the timed CPU baseline, never a checker
PORT_FAST_LIB = HERE / "_build" / "libmoc_oracle_fast.so"
REF_LIB = HERE / "_ref" / "libref_harness.so"


def ref_src() -> Path | None:
    """The reference's src/ directory, as the oracle Makefile locates it
    (SIMPLEMOC_REF_SRC overrides), or None where it is absent."""
    try:
        out = subprocess.run(["make", "-s", "-C", str(HERE), "print-ref-src"], check=True,
                             capture_output=True, text=True).stdout.strip()
    except (OSError, subprocess.CalledProcessError):
        return None
    p = Path(out) if out else None
    return p if p is not None and (p / "solver.c").exists() else None


f32p = C.POINTER(C.c_float)
f64p = C.POINTER(C.c_double)
i32p = C.POINTER(C.c_int32)
i64p = C.POINTER(C.c_int64)


class OracleProblem(C.Structure):
    _fields_ = [
        ("G", C.c_int32), ("F", C.c_int32), ("cai", C.c_int32), ("decomp_ax", C.c_int32),
        ("height", C.c_float), ("axial_exp", C.c_int32), ("NS", C.c_int64), ("N2D", C.c_int64),
        ("P", C.c_int32), ("Z", C.c_int32), ("S", C.c_int32),
        ("seg_len", f32p), ("seg_src", i32p), ("az_weight", f32p), ("p_weight", f32p),
        ("z0", f32p), ("polar_angles", f32p), ("src_sigt", i32p), ("src_xs", i32p),
        ("vol", f32p), ("sigt", f32p), ("xs", f32p), ("scatter", f32p), ("table", f32p),
        ("table_n", C.c_int32), ("table_dx", C.c_float), ("table_maxval", C.c_float),
    ]


class OracleRefGeo(C.Structure):
    _fields_ = [("N2D", C.c_int64), ("seg_off", i64p), ("seg_len", f32p), ("az_weight", f32p),
                ("p_weight", f32p), ("axial_z_sep", C.c_float)]


def make_refgeo(geo) -> OracleRefGeo:
    """oracle_refgeo over a simplemoc_gb300.refabi.RefGeometry (duck-typed)."""
    g = OracleRefGeo(N2D=len(geo.seg_off) - 1, seg_off=_p(geo.seg_off, C.c_int64),
                     seg_len=_p(geo.seg_len, C.c_float), az_weight=_p(geo.az_weight, C.c_float),
                     p_weight=_p(geo.p_weight, C.c_float), axial_z_sep=geo.axial_z_sep)
    g._keep = geo
    return g


def build(reference: bool | None = None) -> None:
    """make -C oracle port [ref]; `ref` only where the reference sources exist."""
    targets = ["port"]
    src = ref_src()
    if reference is None:
        reference = src is not None
    if reference and src is not None:
        targets.append("ref")
    subprocess.run(["make", "-s", "-C", str(HERE), *targets, "port-fast"], check=True,
                   capture_output=True)


def timing_flags() -> str:
    """The compiler flags of the timing build (oracle/Makefile TFLAGS)."""
    try:
        return subprocess.run(["make", "-s", "-C", str(HERE), "print-timing-flags"], check=True,
                              capture_output=True, text=True).stdout.strip()
    except (OSError, subprocess.CalledProcessError):
        return "unknown"


def _p(a, t):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(t))


def make_problem(hp) -> OracleProblem:
    s = hp.spec
    op = OracleProblem(
        G=s.n_groups, F=s.fai, cai=s.cai, decomp_ax=s.decomp_ax, height=s.height,
        axial_exp=s.axial_exp, NS=s.n_sources, N2D=s.n_tracks_2d, P=s.n_polar, Z=s.z_stacked,
        S=s.n_seg, seg_len=_p(hp.seg_len, C.c_float), seg_src=_p(hp.seg_src, C.c_int32),
        az_weight=_p(hp.az_weight, C.c_float), p_weight=_p(hp.p_weight, C.c_float),
        z0=_p(hp.z0, C.c_float), polar_angles=_p(hp.polar_angles, C.c_float),
        src_sigt=_p(hp.src_sigt, C.c_int32), src_xs=_p(hp.src_xs, C.c_int32),
        vol=_p(hp.vol, C.c_float), sigt=_p(hp.sigt, C.c_float), xs=_p(hp.xs, C.c_float),
        scatter=_p(hp.scatter, C.c_float), table=_p(hp.table, C.c_float),
        table_n=hp.table_n, table_dx=hp.table_dx, table_maxval=hp.table_maxval)
    op._keep = hp          # arrays must outlive the struct
    return op


class Port:
    """The C restatement (moc_oracle.c)."""

    def __init__(self, path: Path = PORT_LIB, fast: bool = False):
        """fast: the build with the reference's timing flags (for timing only:
        its fast-math results are not the reference's bit for bit)."""
        if fast:
            path = PORT_FAST_LIB
        if not path.exists():
            build(reference=False)
        lib = C.CDLL(str(path))
        P = C.POINTER(OracleProblem)
        sig = {
            "oracle_exp_table_size": (C.c_int32, [C.c_float, C.c_float]),
            "oracle_build_exp_table": (None, [C.c_float, C.c_float, f32p, f32p, f32p,
                                              C.POINTER(C.c_int32)]),
            "oracle_interpolate": (C.c_float, [f32p, C.c_float, C.c_float, C.c_float]),
            "oracle_pairwise_sum": (C.c_float, [f32p, C.c_int64]),
            "oracle_sweep": (C.c_int64, [P, f32p, f32p, f32p]),
            "oracle_sweep_tracks": (None, [P, f32p, i64p, C.c_int64, f32p, f32p, f32p]),
            "oracle_sweep_omp": (C.c_int64, [P, f32p, f32p, f32p, C.c_int]),
            "oracle_omp_max_threads": (C.c_int, []),
            "oracle_renormalize": (None, [P, f32p, f32p, f32p]),
            "oracle_update_sources": (C.c_float, [P, f32p, f32p, C.c_float]),
            "oracle_compute_keff": (C.c_float, [P, f32p, C.c_float]),
            "oracle_sweep64": (C.c_int64, [P, f64p, f64p, f64p]),
            "oracle_renormalize64": (None, [P, f64p, f64p, f64p]),
            "oracle_update_sources64": (C.c_double, [P, f64p, f64p, C.c_double]),
            "oracle_compute_keff64": (C.c_double, [P, f64p, C.c_double]),
            "oracle_ref_sweep": (C.c_int64, [P, C.POINTER(OracleRefGeo), f32p, f32p, f32p, f32p,
                                             i32p]),
            "oracle_adjoint64": (None, [P, f64p, f64p, f64p, f64p, f64p, f64p]),
        }
        for n, (r, a) in sig.items():
            fn = getattr(lib, n)
            fn.restype = r
            fn.argtypes = a
        self.lib = lib

    def exp_table(self, precision: float, maxval: float = 10.0):
        n = self.lib.oracle_exp_table_size(precision, maxval)
        vals = np.empty(2 * n, dtype=np.float32)
        dx, mv, nn = C.c_float(), C.c_float(), C.c_int32()
        self.lib.oracle_build_exp_table(precision, maxval, _p(vals, C.c_float), C.byref(dx),
                                        C.byref(mv), C.byref(nn))
        return vals, dx.value, mv.value, nn.value

    def sweep(self, op, q, phi, psi_f) -> int:
        f = C.c_float
        return self.lib.oracle_sweep(C.byref(op), _p(q, f), _p(phi, f), _p(psi_f, f))

    def sweep_omp(self, op, q, phi, psi_f, nthreads: int = 0) -> int:
        f = C.c_float
        return self.lib.oracle_sweep_omp(C.byref(op), _p(q, f), _p(phi, f), _p(psi_f, f),
                                         nthreads)

    def sweep_tracks(self, op, q, tracks, psi_in, phi=None):
        G = op.G
        tracks = np.ascontiguousarray(tracks, dtype=np.int64)
        out = np.empty(len(tracks) * G, dtype=np.float32)
        f = C.c_float
        self.lib.oracle_sweep_tracks(C.byref(op), _p(q, f), _p(tracks, C.c_int64), len(tracks),
                                     _p(psi_in, f), _p(out, f), _p(phi, f))
        return out

    def ref_sweep(self, op, rg, q, phi, psi_f, z_height, ids=None) -> int:
        """The reference traversal (oracle_ref_sweep); ids None = libc rand()."""
        f = C.c_float
        return self.lib.oracle_ref_sweep(C.byref(op), C.byref(rg), _p(q, f), _p(phi, f),
                                         _p(psi_f, f), _p(z_height, f), _p(ids, C.c_int32))

    def renormalize(self, op, phi, psi_f, psi_b) -> None:
        f = C.c_float
        self.lib.oracle_renormalize(C.byref(op), _p(phi, f), _p(psi_f, f), _p(psi_b, f))

    def update_sources(self, op, phi, q, keff: float) -> float:
        f = C.c_float
        return self.lib.oracle_update_sources(C.byref(op), _p(phi, f), _p(q, f), keff)

    def compute_keff(self, op, phi, leakage: float = 0.0) -> float:
        return self.lib.oracle_compute_keff(C.byref(op), _p(phi, C.c_float), leakage)

    def sweep64(self, op, q, phi, psi_f) -> int:
        d = C.c_double
        return self.lib.oracle_sweep64(C.byref(op), _p(q, d), _p(phi, d), _p(psi_f, d))

    def adjoint64(self, op, q, dphi, psi_in=None):
        """(dq, dsigt, dpsi_in) of one FP64 sweep for dL/dphi (all float64)."""
        d = C.c_double
        G = op.G
        nr = op.NS * op.F
        n3d = op.N2D * op.P * op.Z
        n_sigt = op._keep.sigt.size // G
        dq = np.zeros(nr * G, np.float64)
        ds = np.zeros(n_sigt * G, np.float64)
        dp = np.zeros(n3d * G, np.float64)
        self.lib.oracle_adjoint64(C.byref(op), _p(q, d), _p(psi_in, d), _p(dphi, d), _p(dq, d),
                                  _p(ds, d), _p(dp, d))
        return dq, ds, dp

    def renormalize64(self, op, phi, psi_f, psi_b) -> None:
        d = C.c_double
        self.lib.oracle_renormalize64(C.byref(op), _p(phi, d), _p(psi_f, d), _p(psi_b, d))

    def update_sources64(self, op, phi, q, keff: float) -> float:
        d = C.c_double
        return self.lib.oracle_update_sources64(C.byref(op), _p(phi, d), _p(q, d), keff)

    def compute_keff64(self, op, phi, leakage: float = 0.0) -> float:
        return self.lib.oracle_compute_keff64(C.byref(op), _p(phi, C.c_double), leakage)

    # -- a whole power iteration (src/main.c:57-92) ---------------------------
    def iterate(self, hp, state: dict, n_iters: int, keff: float = 1.0, threads: int = 1):
        """state: dict with fine_source, fine_flux, psi_f, psi_b (float32, updated)."""
        op = make_problem(hp)
        hist = []
        for _ in range(n_iters):
            if threads == 1:
                self.sweep(op, state["fine_source"], state["fine_flux"], state["psi_f"])
            else:
                self.sweep_omp(op, state["fine_source"], state["fine_flux"], state["psi_f"],
                               threads)
            self.renormalize(op, state["fine_flux"], state["psi_f"], state["psi_b"])
            res = self.update_sources(op, state["fine_flux"], state["fine_source"], keff)
            keff = self.compute_keff(op, state["fine_flux"], 0.0)
            hist.append((float(keff), float(res)))
        return hist

    def iterate64(self, hp, state: dict, n_iters: int, keff: float = 1.0):
        op = make_problem(hp)
        hist = []
        for _ in range(n_iters):
            self.sweep64(op, state["fine_source"], state["fine_flux"], state["psi_f"])
            self.renormalize64(op, state["fine_flux"], state["psi_f"], state["psi_b"])
            res = self.update_sources64(op, state["fine_flux"], state["fine_source"], keff)
            keff = self.compute_keff64(op, state["fine_flux"], 0.0)
            hist.append((float(keff), float(res)))
        return hist


class Reference:
    """The reference's own compiled solver (oracle/_ref), if it was built here."""

    def __init__(self, path: Path = REF_LIB):
        if not path.exists():
            raise FileNotFoundError(f"{path} not built (needs the reference sources)")
        lib = C.CDLL(str(path))
        P = C.POINTER(OracleProblem)
        sig = {
            "refh_setup": (C.c_int, [P, C.c_float, f32p, f32p, f32p, f32p]),
            "refh_sweep": (C.c_long, []),
            "refh_renormalize": (None, []),
            "refh_update_sources": (C.c_float, [C.c_float]),
            "refh_compute_keff": (C.c_float, []),
            "refh_table": (C.c_int, [C.c_float, f32p, C.c_int, f32p, f32p]),
            "refh_teardown": (None, []),
        }
        for n, (r, a) in sig.items():
            fn = getattr(lib, n)
            fn.restype = r
            fn.argtypes = a
        self.lib = lib

    @staticmethod
    def available() -> bool:
        return REF_LIB.exists()

    def exp_table(self, precision: float):
        cap = 1 << 20
        vals = np.empty(2 * cap, dtype=np.float32)
        dx, mv = C.c_float(), C.c_float()
        n = self.lib.refh_table(precision, _p(vals, C.c_float), cap, C.byref(dx), C.byref(mv))
        return vals[:2 * n].copy(), dx.value, mv.value, n

    def transport_sweep(self, hp, state: dict, rg, z_height) -> int:
        """The reference's own transport_sweep (serial build: libc rand() ids,
        seeded by the caller's srand) over a reference-style geometry."""
        op = make_problem(hp)
        f = C.c_float
        self.lib.refh_setup_ref.argtypes = [C.POINTER(OracleRefGeo), f32p, C.c_float]
        self.lib.refh_transport_sweep.restype = C.c_long
        self.lib.refh_transport_sweep.argtypes = [f32p]
        self.lib.refh_setup(C.byref(op), hp.spec.precision, _p(state["fine_source"], f),
                            _p(state["fine_flux"], f), _p(state["psi_f"], f),
                            _p(state["psi_b"], f))
        try:
            self.lib.refh_setup_ref(C.byref(rg), _p(z_height, f), rg.axial_z_sep)
            return int(self.lib.refh_transport_sweep(_p(z_height, f)))
        finally:
            self.lib.refh_teardown()

    def load_openmoc(self, path, cmfd: bool = False, cap_tracks: int = 1 << 16,
                     cap_segs: int = 1 << 22) -> dict:
        """The reference's own load_OpenMOC_tracks on `path`: per 2D track its
        segment count, per segment the float length and region id, and the
        reader's metadata (n_azimuthal, radial_ray_sep, segments_per_track)."""
        fn = self.lib.refh_load_openmoc
        fn.restype = C.c_long
        fn.argtypes = [C.c_char_p, C.c_int, C.c_long, C.c_long, C.POINTER(C.c_int),
                       C.POINTER(C.c_float), C.POINTER(C.c_long), C.c_void_p, C.c_void_p,
                       C.c_void_p]
        nseg = np.zeros(cap_tracks, np.int64)
        lens = np.zeros(cap_segs, np.float32)
        ids = np.zeros(cap_segs, np.int64)
        n_az, sep, spt = C.c_int(), C.c_float(), C.c_long()
        n = fn(str(path).encode(), int(cmfd), cap_tracks, cap_segs, C.byref(n_az), C.byref(sep),
               C.byref(spt), nseg.ctypes.data, lens.ctypes.data, ids.ctypes.data)
        if n < 0:
            raise ValueError("track file larger than the harness buffers")
        m = int(nseg[:n].sum())
        return {"n_tracks_2d": int(n), "n_segments": nseg[:n].copy(), "lengths": lens[:m].copy(),
                "source_ids": ids[:m].copy(), "n_azimuthal": n_az.value,
                "radial_ray_sep": sep.value, "segments_per_track": spt.value}

    def iterate(self, hp, state: dict, n_iters: int, keff: float = 1.0, sweep_only=False):
        op = make_problem(hp)
        f = C.c_float
        self.lib.refh_setup(C.byref(op), hp.spec.precision, _p(state["fine_source"], f),
                            _p(state["fine_flux"], f), _p(state["psi_f"], f),
                            _p(state["psi_b"], f))
        hist = []
        try:
            for _ in range(n_iters):
                self.lib.refh_sweep()
                if sweep_only:
                    continue
                self.lib.refh_renormalize()
                res = self.lib.refh_update_sources(keff)
                keff = self.lib.refh_compute_keff()
                hist.append((float(keff), float(res)))
        finally:
            self.lib.refh_teardown()
        return hist


def fresh_state(hp, dtype=np.float32) -> dict:
    s = hp.spec
    nf, nt = s.n_fsr * s.n_groups, s.n_tracks_3d * s.n_groups
    st = {
        "fine_source": hp.fine_source.astype(dtype, copy=True),
        "fine_flux": (np.zeros(nf, dtype) if hp.fine_flux is None
                      else hp.fine_flux.astype(dtype, copy=True)),
        "psi_f": np.zeros(nt, dtype) if hp.psi_f is None else hp.psi_f.astype(dtype, copy=True),
        "psi_b": np.zeros(nt, dtype) if hp.psi_b is None else hp.psi_b.astype(dtype, copy=True),
    }
    return st
