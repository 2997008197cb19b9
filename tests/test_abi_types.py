"""CPU test: the ctypes binding agrees with include/simplemoc_gb300.h.

Every declared function has, in simplemoc_gb300._lib.SIGNATURES, the same
number of parameters with the same scalar widths (pointers as pointers), and
the same return type; the struct mirrors (moc_dims, moc_host, moc_gen_params)
have the header's fields, in order, with the header's types.  A mismatch here
is an ABI bug that no GPU test would show until a value is misread.
"""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "simplemoc_gb300.h"

SCALARS = {"int": "i32", "int32_t": "i32", "int64_t": "i64", "uint64_t": "u64",
           "float": "f32", "double": "f64", "void": "void"}


def _text():
    return re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)


def _c_kind(decl: str) -> str:
    """'const float *x' -> 'ptr'; 'int64_t n' -> 'i64'; 'int' -> 'i32'."""
    if "*" in decl:
        return "ptr"
    words = [w for w in re.findall(r"[A-Za-z_][A-Za-z0-9_]*", decl) if w != "const"]
    return SCALARS[words[0]]


def _ctype_kind(t) -> str:
    if t is None:
        return "void"
    if t in (C.c_void_p, C.c_char_p) or isinstance(t, type(C.POINTER(C.c_int))):
        return "ptr"
    if t in (C.c_int, C.c_int32):
        return "i32"
    if t is C.c_int64:
        return "i64"
    if t is C.c_uint64:
        return "u64"
    if t is C.c_float:
        return "f32"
    if t is C.c_double:
        return "f64"
    raise AssertionError(f"unexpected ctypes type {t!r}")


def _prototypes():
    out = {}
    for m in re.finditer(r"^\s*((?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**)\s*"
                         r"([A-Za-z_][A-Za-z0-9_]*)\s*\(([^;{]*?)\)\s*;", _text(), flags=re.M | re.S):
        ret, name, params = m.group(1), m.group(2), m.group(3).strip()
        kinds = [] if params in ("", "void") else [_c_kind(p) for p in params.split(",")]
        out[name] = (_c_kind(ret), kinds)
    return out


def test_every_signature_matches_the_header():
    from simplemoc_gb300 import _lib as L
    protos = _prototypes()
    assert len(protos) >= 40
    bad = []
    for name, (ret, kinds) in protos.items():
        assert name in L.SIGNATURES, name
        res, args = L.SIGNATURES[name]
        got = (_ctype_kind(res), [_ctype_kind(a) for a in args])
        if got != (ret, kinds):
            bad.append((name, (ret, kinds), got))
    assert not bad, bad


def _struct_fields(name: str):
    m = re.search(r"typedef\s+struct\s+" + name + r"\s*\{(.*?)\}\s*" + name + r"\s*;", _text(),
                  flags=re.S)
    assert m, name
    fields = []
    for stmt in m.group(1).split(";"):
        stmt = stmt.strip()
        if not stmt:
            continue
        # 'float len_lo, len_hi' declares two fields of one type
        head, *rest = [s.strip() for s in stmt.split(",")]
        base = re.match(r"((?:const\s+)?[A-Za-z_][A-Za-z0-9_]*)\s*(\**)\s*([A-Za-z_][A-Za-z0-9_]*)$",
                        head)
        assert base, stmt
        t, star, fname = base.groups()
        scalar = SCALARS[t.replace("const ", "").strip()]
        fields.append((fname, "ptr" if star else scalar))
        for r in rest:
            r_star, r_name = re.match(r"(\**)\s*([A-Za-z_][A-Za-z0-9_]*)$", r).groups()
            fields.append((r_name, "ptr" if r_star else scalar))
    return fields


@pytest.mark.parametrize("cname,pyname", [("moc_dims", "MocDims"), ("moc_host", "MocHost"),
                                          ("moc_gen_params", "MocGenParams")])
def test_struct_mirrors_match_the_header(cname, pyname):
    from simplemoc_gb300 import _lib as L
    want = _struct_fields(cname)
    got = [(n, _ctype_kind(t)) for n, t in getattr(L, pyname)._fields_]
    assert got == want


# ---- the drop-in header (include/simplemoc_refabi.h) -------------------------

REF_HEADER = ROOT / "include" / "simplemoc_refabi.h"
REF_STRUCTS = {"moc_ref_input": "Input", "moc_ref_segment": "Segment",
               "moc_ref_track2d": "Track2D", "moc_ref_track": "Track",
               "moc_ref_source": "Source", "moc_ref_table": "Table",
               "moc_ref_params": "Params", "moc_ref_commgrid": "CommGrid"}
REF_SCALARS = dict(SCALARS, long="i64", bool="bool")


def _ref_text():
    text = re.sub(r"/\*.*?\*/", "", REF_HEADER.read_text(), flags=re.S)
    # the serial build's layout: drop the OpenMP build's extra fields
    return re.sub(r"#ifdef SIMPLEMOC_REF_OPENMP.*?#endif", "", text, flags=re.S)


def _ref_kind(t: str, star: str) -> str:
    if star:
        return "ptr"
    return f"struct:{t}" if t in REF_STRUCTS else REF_SCALARS[t]


def _ref_ctype_kind(t) -> str:
    for cname, pyname in REF_STRUCTS.items():
        if getattr(t, "__name__", None) == pyname and issubclass(t, C.Structure):
            return f"struct:{cname}"
    if t is C.c_bool:
        return "bool"
    if t is C.c_long:
        return "i64"
    return _ctype_kind(t)


@pytest.mark.parametrize("cname", sorted(REF_STRUCTS))
def test_reference_struct_mirrors_match_the_drop_in_header(cname):
    from simplemoc_gb300 import refabi
    m = re.search(r"typedef\s+struct\s+" + cname + r"\s*\{(.*?)\}\s*" + cname + r"\s*;",
                  _ref_text(), flags=re.S)
    assert m, cname
    want = []
    for stmt in m.group(1).split(";"):
        stmt = stmt.strip()
        if not stmt:
            continue
        head, *rest = [s.strip() for s in stmt.split(",")]
        t, star, name = re.match(r"([A-Za-z_][A-Za-z0-9_]*)\s*(\**)\s*([A-Za-z_][A-Za-z0-9_]*)$",
                                 head).groups()
        want.append((name, _ref_kind(t, star)))
        for r in rest:
            r_star, r_name = re.match(r"(\**)\s*([A-Za-z_][A-Za-z0-9_]*)$", r).groups()
            want.append((r_name, _ref_kind(t, r_star)))
    py = getattr(refabi, REF_STRUCTS[cname])
    got = [(n, _ref_ctype_kind(t)) for n, t in py._fields_]
    assert got == want


def test_reference_entry_points_match_the_drop_in_header(lib):
    from simplemoc_gb300 import refabi
    lb = refabi.lib()
    bad, seen = [], 0
    for m in re.finditer(r"^\s*([A-Za-z_][A-Za-z0-9_]*\s*\**)\s*([A-Za-z_][A-Za-z0-9_]*)\s*"
                         r"\(([^;{]*?)\)\s*;", _ref_text(), flags=re.M | re.S):
        ret, name, params = m.group(1).strip(), m.group(2), m.group(3).strip()
        kinds = []
        if params not in ("", "void"):
            for p in params.split(","):
                t, star = re.match(r"\s*(?:const\s+)?([A-Za-z_][A-Za-z0-9_]*)\s*(\**)", p).groups()
                kinds.append(_ref_kind(t, star))
        r_t, r_star = re.match(r"([A-Za-z_][A-Za-z0-9_]*)\s*(\**)", ret).groups()
        want = (_ref_kind(r_t, r_star), kinds)
        fn = getattr(lb, name)
        got = (_ref_ctype_kind(fn.restype), [_ref_ctype_kind(a) for a in fn.argtypes])
        seen += 1
        if got != want:
            bad.append((name, want, got))
    assert seen == 11 and not bad, (seen, bad)
