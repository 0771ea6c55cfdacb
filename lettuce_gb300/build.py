"""In-tree build of ``liblettuce_gb300.so`` (the CUDA C-ABI library).

``python -m lettuce_gb300.build`` compiles every translation unit under
``csrc/`` for sm_103a with nvcc, in parallel (one object per stencil x
population storage for the generic step kernel), and links them into
``lettuce_gb300/_build/liblettuce_gb300.so``. Sources whose hash is
unchanged since the last build are not recompiled.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import json
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT_DIR = os.path.join(PKG, "_build")
LIB_NAME = "liblettuce_gb300.so"
LIB_PATH = os.path.join(OUT_DIR, LIB_NAME)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                     "-I", INCLUDE, "-I", CSRC]

STEP_STENCILS = ["d1q3", "d2q9", "d3q15", "d3q19", "d3q27"]
# stencils whose units are split into grids without boundaries and, with
# boundaries, the pulling and the other patterns (their instantiations take
# the longest to compile)
SPLIT_STENCILS = ("d3q19", "d3q27")
N_STORAGES = 4
# per-unit flags: the initialisation / enstrophy unit rounds every product
# and sum on its own (no fused multiply-add), in lettuce's evaluation order
UNIT_FLAGS = {"lgb_init.cu": ["-fmad=false"]}


def nvcc_path() -> str:
    cand = shutil.which("nvcc")
    if cand:
        return cand
    for home in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if home and os.path.exists(os.path.join(home, "bin", "nvcc")):
            return os.path.join(home, "bin", "nvcc")
    raise RuntimeError("nvcc not found (set CUDA_HOME or put nvcc on PATH)")


def _units():
    """(object name, source, extra flags) for every translation unit"""
    units = []
    for st in STEP_STENCILS:
        parts = [("_p0", ["-DLGB_MASK_PART=0"]), ("_p1", ["-DLGB_MASK_PART=1"]),
                 ("_p3", ["-DLGB_MASK_PART=3"])] if st in SPLIT_STENCILS else [("", [])]
        for s in range(N_STORAGES):
            for tag, part in parts:
                units.append((f"step_{st}_s{s}{tag}.o", f"lgb_step_{st}.cu",
                              [f"-DLGB_STORAGE_ID={s}"] + part))
                # forced BGK, regularized, Smagorinsky and MRT: their own objects
                units.append((f"stepx_{st}_s{s}{tag}.o", f"lgb_step_{st}.cu",
                              [f"-DLGB_STORAGE_ID={s}", "-DLGB_EXT_COLLISIONS=1"] + part))
    for src in sorted(os.listdir(CSRC)):
        if src.endswith(".cu") and not src.startswith("lgb_step_"):
            units.append((src[:-3] + ".o", src, UNIT_FLAGS.get(src, [])))
    return units


def _headers_digest() -> str:
    h = hashlib.sha256()
    for d in (CSRC, INCLUDE):
        for name in sorted(os.listdir(d)):
            if name.endswith((".cuh", ".h")):
                with open(os.path.join(d, name), "rb") as fh:
                    h.update(name.encode() + fh.read())
    return h.hexdigest()


def _unit_key(src: str, flags, hdr: str) -> str:
    h = hashlib.sha256()
    with open(os.path.join(CSRC, src), "rb") as fh:
        h.update(fh.read())
    h.update(" ".join(NVCC_FLAGS + list(flags)).encode())
    h.update(hdr.encode())
    return h.hexdigest()


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compile and link the library; returns its path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = nvcc_path()
    stamp_path = os.path.join(OUT_DIR, "stamps.json")
    try:
        with open(stamp_path) as fh:
            stamps = json.load(fh)
    except (OSError, ValueError):
        stamps = {}
    hdr = _headers_digest()
    units = _units()
    todo = []
    for obj, src, flags in units:
        key = _unit_key(src, flags, hdr)
        if stamps.get(obj) != key or not os.path.exists(os.path.join(OUT_DIR, obj)):
            todo.append((obj, src, flags, key))

    def compile_one(item):
        obj, src, flags, key = item
        cmd = [nvcc] + NVCC_FLAGS + list(flags) + ["-c", os.path.join(CSRC, src),
                                                   "-o", os.path.join(OUT_DIR, obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src} {flags}:\n{r.stderr[-4000:]}")
        if verbose:
            print(f"[lettuce_gb300] built {obj}", file=sys.stderr)
        return obj, key

    # longest first, so the last units to finish are short ones
    cost = {"d3q27": 0, "d3q19": 1, "batched": 2, "abi": 3, "d3q15": 4}
    todo.sort(key=lambda it: min([v for k, v in cost.items() if k in it[0]] + [9]))
    jobs = jobs or max(1, os.cpu_count() or 1)
    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
            for obj, key in ex.map(compile_one, todo):
                stamps[obj] = key
                with open(stamp_path, "w") as fh:
                    json.dump(stamps, fh)
    objs = [os.path.join(OUT_DIR, u[0]) for u in units]
    need_link = bool(todo) or not os.path.exists(LIB_PATH)
    if need_link:
        tmp = LIB_PATH + ".tmp"
        cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose=True))
