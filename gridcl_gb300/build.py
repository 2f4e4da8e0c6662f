"""Builds the in-tree CUDA library ``gridcl_gb300/libtlgeom.so`` for sm_103a.

Translation units compile in parallel with nvcc (one ``-gencode``, ``-lineinfo``) and link
into one shared library with the CUDA runtime linked statically. Run
``python -m gridcl_gb300.build``; ``__graft_entry__.build()`` calls :func:`build`.
"""

from __future__ import annotations

import concurrent.futures
import os
import pathlib
import shutil
import subprocess
import sys

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parent
CSRC = HERE / "csrc"
OUT_DIR = HERE / "_build"
LIB = HERE / "libtlgeom.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["api.cu", "coop.cu", "csr.cu", "eval_df.cu", "eval_f32.cu", "eval_f64.cu", "eval_pair.cu", "eval_pair_meas.cu", "measure.cu", "order.cpp",
           "pullback.cu", "refcell.cpp", "sumfact.cu", "sumfact_df.cu", "sumfact_fn.cu", "tc.cu", "umma.cu", "vjp_f64.cu", "vjp_split.cu", "vjp_surface.cu"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return exe


def _compile(src: pathlib.Path, obj: pathlib.Path, extra) -> None:
    cmd = [nvcc(), *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
           "-I", str(ROOT / "include"), "-c", str(src), "-o", str(obj), *extra]
    if src.suffix == ".cpp":
        cmd = [nvcc(), "-x", "c++", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
               "-I", str(ROOT / "include"), "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip():
        sys.stderr.write(r.stderr)


def build(verbose_ptxas: bool = False, force: bool = False) -> pathlib.Path:
    OUT_DIR.mkdir(exist_ok=True)
    deps = sorted(CSRC.glob("*")) + [ROOT / "include" / "tlgeom.h"]
    newest = max(p.stat().st_mtime for p in deps)
    if LIB.exists() and not force and LIB.stat().st_mtime > newest and not verbose_ptxas:
        return LIB
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    objs = []
    jobs = []
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        for name in SOURCES:
            src = CSRC / name
            obj = OUT_DIR / (name + ".o")
            objs.append(obj)
            jobs.append(ex.submit(_compile, src, obj, extra))
        for j in jobs:
            j.result()
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-cudart", "static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose_ptxas="-v" in sys.argv, force="-f" in sys.argv))
