"""In-tree build of libfsph.so for sm_103a (nvcc directly, no cmake).

    python -m fltk_sph_ice_gb300.build                  # or __graft_entry__.build()
    python -m fltk_sph_ice_gb300.build --debug-bounds   # the bounds-checking debug library

Translation units compile in parallel into ``_build/*.o`` and link into
``_build/libfsph.so``; a unit is recompiled only when it or a header changed.
``--debug-bounds`` builds ``_build/debug_bounds/libfsph.so`` with
FSPH_DEBUG_BOUNDS=1: every neighbour slot, cell row and list count the passes
read is checked before use and a failed check is reported in
``fsph_step_stats.bounds_bits`` (load it with FSPH_LIBRARY=<path>).
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
OUT_DEBUG_BOUNDS = os.path.join(OUT, "debug_bounds")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no contraction of a * b + c into fused multiply-adds (gcc does it by default where the ISA has
# them, as on Arm), so host arithmetic -- parameter derivation, grid geometry -- rounds the same on every host
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _headers_mtime() -> float:
    hs = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))
    return max((os.path.getmtime(h) for h in hs), default=0.0)


def _compile(src: str, obj: str, extra: list[str], verbose: bool) -> None:
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr.strip():
        print(r.stderr, file=sys.stderr)


def build(verbose: bool = False, force: bool = False, extra: list[str] | None = None,
          debug_bounds: bool = False) -> str:
    out = OUT_DEBUG_BOUNDS if debug_bounds else OUT
    os.makedirs(out, exist_ok=True)
    extra = list(extra or []) + (["-DFSPH_DEBUG_BOUNDS=1"] if debug_bounds else [])
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    hdr = _headers_mtime()
    jobs = []
    objs = []
    for s in srcs:
        o = os.path.join(out, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if force or not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), hdr):
            jobs.append((s, o))
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for f in [ex.submit(_compile, s, o, extra, verbose) for s, o in jobs]:
            f.result()
    lib = os.path.join(out, "libfsph.so")
    if jobs or not os.path.exists(lib):
        cmd = [nvcc(), *ARCH, "-shared", "-o", lib, *objs, "-lcudart"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return lib


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv, debug_bounds="--debug-bounds" in sys.argv))
