"""Build the GB300 transport library in-tree (nvcc, sm_103a).

Produces ``openmc_gb300/_lib/libopenmc_gb300.so`` from the sources in
``openmc_gb300/csrc``.  Translation units compile in parallel; device code is
built for ``sm_103a`` only with ``-fmad=false`` so that every floating-point
multiply and add rounds separately, as in the reference's C++ expressions;
the transport build that FP32-table mode runs (namespace l2f) fuses them.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_lib"
LIB = OUT / "libopenmc_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code rounds every multiply and add separately too (no FMA contraction
# on the Arm host), as the reference's expressions and the oracle do
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off"]
EXACT = ["-fmad=false"]
SOURCES = ["h5lite.cpp", "host_model.cpp", "capi.cpp", "capi_model.cpp", "capi_offpath.cpp", "transport_dispatch.cpp", "xsbench.cu",
           "mlp.cu"]
# transport.cu is built once per maximum coordinate depth (namespaces l2, l4)
# with separately rounded multiplies and adds, and once for FP32-table mode at
# depth 2 with multiply-adds fused (l2f)
VARIANTS = [("transport.cu", "transport_l2", ["-DOMC_MAXL=2", "-DOMC_NS=l2", *EXACT]),
            ("transport.cu", "transport_l4", ["-DOMC_MAXL=4", "-DOMC_NS=l4", *EXACT]),
            ("transport.cu", "transport_l2f", ["-DOMC_MAXL=2", "-DOMC_NS=l2f", "-fmad=true",
                                               # FP32-table collisions wait on memory, not
                                               # the FP64 pipe: three CTAs per SM
                                               "-DOMC_MINB_COLL=3"])]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found")
    return exe


def _compile(src: Path, obj: Path, extra):
    cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stderr


def build(force: bool = False, verbose: bool = False, extra=()) -> Path:
    units = [(CSRC / s, Path(s).stem, list(EXACT)) for s in SOURCES if (CSRC / s).exists()]
    units += [(CSRC / s, stem, flags) for s, stem, flags in VARIANTS]
    srcs = [u[0] for u in units]
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh"))
    newest = max(p.stat().st_mtime for p in srcs + headers)
    if LIB.exists() and not force and LIB.stat().st_mtime >= newest:
        return LIB
    OUT.mkdir(parents=True, exist_ok=True)
    objs = [OUT / (stem + ".o") for _, stem, _ in units]
    with cf.ThreadPoolExecutor(max_workers=min(8, len(units))) as ex:
        futs = [ex.submit(_compile, src, o, list(flags) + list(extra))
                for (src, _, flags), o in zip(units, objs)]
        for f in futs:
            msg = f.result()
            if verbose and msg:
                print(msg)
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    for o in objs:
        o.unlink(missing_ok=True)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True))
