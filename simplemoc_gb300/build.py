"""Builds libsimplemoc_gb300.so in-tree for sm_103a (nvcc + g++, no cmake).

    python -m simplemoc_gb300.build        # or __graft_entry__.build()

Translation units compile in parallel; objects go to simplemoc_gb300/_build/,
the shared library to simplemoc_gb300/libsimplemoc_gb300.so.  Host code is
compiled with -ffp-contract=off so that float expressions that restate the
reference (tables, segment lengths, coefficient products) round exactly as the
reference's do.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libsimplemoc_gb300.so"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

CU_SOURCES = ["moc_api.cu", "moc_sweep.cu", "moc_post.cu", "moc_refabi.cu", "moc_batch.cu",
              "moc_update_tc.cu", "moc_determ.cu", "moc_update_adj.cu"]
CPP_SOURCES = ["moc_host.cpp", "moc_openmoc.cpp", "moc_libc_rand.cpp"]


def _nvcc() -> str:
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cand = Path(cuda) / "bin" / "nvcc"
    return str(cand) if cand.exists() else (shutil.which("nvcc") or "nvcc")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.h")) + list((ROOT / "include").glob("*.h"))
    inc = [f"-I{ROOT / 'include'}", f"-I{CSRC}"]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        obj = BUILD / (src + ".o")
        objs.append(obj)
        if _stale(obj, [CSRC / src] + headers):
            jobs.append([_nvcc(), ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler",
                         "-fPIC,-ffp-contract=off,-fopenmp", *inc, "-c", str(CSRC / src),
                         "-o", str(obj)])
    for src in CPP_SOURCES:
        obj = BUILD / (src + ".o")
        objs.append(obj)
        if _stale(obj, [CSRC / src] + headers):
            jobs.append(["g++", "-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fopenmp",
                         *inc, "-c", str(CSRC / src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for cmd in jobs:
            if verbose:
                print(" ".join(cmd), flush=True)
        list(ex.map(_run, jobs))
    if jobs or _stale(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp")
        # -Bsymbolic: calls inside the library bind to its own definitions even when
        # another loaded object exports the same reference entry-point names
        _run([_nvcc(), ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-Xcompiler", "-fopenmp",
              "-Xlinker", "-Bsymbolic", "-lgomp", "-ldl"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
