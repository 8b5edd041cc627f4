"""Build the CPU oracle (and, where the reference sources are mounted, the
reference's own C implementation of the path).

TEST INFRASTRUCTURE ONLY: the libraries built here are checkers for the CUDA
path (tests/, __graft_entry__.smoke(), bench.py's cpu_baseline and reference
legs).  Nothing in the product library links or loads them.

* ``oracle/_build/liboracle.so`` -- ``oracle/oracle.c`` and
  ``oracle/kmer_oracle.c`` (this project's own restatements), ``gcc -O3
  -fopenmp``.
* ``oracle/_ref/sw_align_ref.so`` -- ``clustkit/csrc/sw_align.c`` compiled
  straight from the reference checkout (read in place, never copied), with the
  reference's own build line (clustkit/csrc/sw_align.c:10) minus
  ``-march=native``.  Built only when the reference checkout exists.
* ``oracle/_ref/kmer_score_ref.so`` -- ``clustkit/csrc/kmer_score.c``, the
  reference's C k-mer scorer (Phase A, top-K, Phase B, diagonal hints), for
  the golden vectors of the search path's candidate stage.
* ``oracle/_ref/sw_cupy_ref.cubin`` -- the reference's CuPy SW kernel
  (the ``_SW_ALIGN_KERNEL_CODE`` string, clustkit/pairwise.py:1215-1402, read
  from the checkout with ``ast``, never imported), compiled by nvcc for
  sm_103a from a temporary file outside the repository; only the device
  binary is written.  It is the "reference's CuPy path" baseline timed by
  bench.py through oracle/cupy_ref.py (CuPy itself is not installed).
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
# Root of the clustkit reference checkout: the CLUSTKIT_REFERENCE environment
# variable, else the location where the build container mounts it.  This
# recipe and tests/golden/make_golden.py (which takes it from here) are the
# only readers; nothing at run time needs the checkout, and without it the
# reference-built checkers are simply not produced.
REF_ROOT = Path(os.environ.get("CLUSTKIT_REFERENCE", "/root/reference"))
REF_SRC = REF_ROOT / "clustkit" / "csrc" / "sw_align.c"

CFLAGS = ["-O3", "-fopenmp", "-shared", "-fPIC", "-std=c11"]


def _needs(out: Path, src: Path) -> bool:
    return not out.exists() or out.stat().st_mtime < src.stat().st_mtime


def build_oracle(verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    srcs = [HERE / "oracle.c", HERE / "kmer_oracle.c"]
    out = BUILD / "liboracle.so"
    if any(_needs(out, src) for src in srcs):
        cmd = ["gcc", *CFLAGS, "-o", str(out), *map(str, srcs)]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        subprocess.run(cmd, check=True)
    return out


def build_reference(verbose: bool = False) -> Path | None:
    """Compile the reference's sw_align.c into oracle/_ref/ if the checkout is present."""
    if not REF_SRC.exists():
        return None
    REF_OUT.mkdir(exist_ok=True)
    out = REF_OUT / "sw_align_ref.so"
    if _needs(out, REF_SRC):
        cmd = ["gcc", "-O3", "-fopenmp", "-shared", "-fPIC", "-o", str(out), str(REF_SRC)]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        subprocess.run(cmd, check=True)
    return out


def build_reference_kmer_scorer(verbose: bool = False) -> Path | None:
    """Compile the reference's C k-mer scorer (clustkit/csrc/kmer_score.c) into oracle/_ref/."""
    src = REF_SRC.parent / "kmer_score.c"
    if not src.exists():
        return None
    REF_OUT.mkdir(exist_ok=True)
    out = REF_OUT / "kmer_score_ref.so"
    if _needs(out, src):
        cmd = ["gcc", "-O3", "-fopenmp", "-shared", "-fPIC", "-o", str(out), str(src)]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        subprocess.run(cmd, check=True)
    return out


def build_reference_cupy_kernel(verbose: bool = False) -> Path | None:
    """Compile the reference's CuPy kernel string into oracle/_ref/sw_cupy_ref.cubin."""
    import ast
    import tempfile
    py = REF_SRC.parent.parent / "pairwise.py"
    if not py.exists():
        return None
    REF_OUT.mkdir(exist_ok=True)
    out = REF_OUT / "sw_cupy_ref.cubin"
    if out.exists() and out.stat().st_mtime >= py.stat().st_mtime:
        return out
    code = None
    for node in ast.parse(py.read_text()).body:
        if isinstance(node, ast.Assign) and any(getattr(t, "id", None) == "_SW_ALIGN_KERNEL_CODE"
                                                for t in node.targets):
            code = node.value.value
    if code is None:
        return None
    with tempfile.TemporaryDirectory() as td:
        src = Path(td) / "sw_cupy_ref.cu"
        src.write_text(code)
        cmd = ["nvcc", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-o", str(out), str(src)]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        subprocess.run(cmd, check=True)
    return out


def main() -> None:
    print(build_oracle(verbose=True))
    print(build_reference(verbose=True))
    print(build_reference_cupy_kernel(verbose=True))
    print(build_reference_kmer_scorer(verbose=True))


if __name__ == "__main__":
    main()
