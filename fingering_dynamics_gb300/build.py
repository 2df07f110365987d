"""Build ``libfdlbm.so`` in-tree with nvcc for sm_103a.

Each translation unit is compiled separately and in parallel; the FP64 /
reference-order units get ``-fmad=false`` (the reference's arithmetic
without contraction), the others keep FMA contraction.  The shared library
lands in ``fingering_dynamics_gb300/_lib/``.

    python -m fingering_dynamics_gb300.build [--force] [--verbose] [--out DIR] [--define NAME=VALUE ...]

--out / --define build another copy of the library with compile-time options
(e.g. FD_TMA_NS_16=6) into DIR; point FDLBM_LIBRARY at DIR/libfdlbm.so to
load it instead of the in-tree build.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import fcntl
import hashlib
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT, "libfdlbm.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
          "-I", os.path.join(REPO, "include")]
# translation unit -> extra flags
UNITS = {
    "fd_capi.cu": [],
    "fd_ref.cu": ["-fmad=false"],
    "fd_fused_f64.cu": ["-fmad=false"],
    "fd_fused_f32.cu": [],
    "fd_fused_dev.cu": [],
    "fd_fused_tma.cu": [],
    "fd_noalloc.cu": [],
    "fd_diag.cu": [],
    "fd_batch.cu": [],
    "fd_host_step.cu": [],
    "sg_kernels.cu": [],
    "sg_tcgen05.cu": [],
}


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _sources_digest(extra: list[str]) -> str:
    h = hashlib.sha256()
    for root in (CSRC, os.path.join(REPO, "include")):
        for name in sorted(os.listdir(root)):
            if name.endswith((".cu", ".cuh", ".h")):
                with open(os.path.join(root, name), "rb") as fh:
                    h.update(name.encode() + fh.read())
    h.update(" ".join(ARCH + COMMON + extra).encode())
    return h.hexdigest()


def _up_to_date(lib_path: str, stamp: str, digest: str) -> bool:
    if not (os.path.exists(lib_path) and os.path.exists(stamp)):
        return False
    with open(stamp) as fh:
        return fh.read().strip() == digest


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False, out: str | None = None,
          defines: tuple[str, ...] = ()) -> str:
    """Compile and link when the sources changed.  Concurrent callers (one per
    rank of a multi-GPU run) serialise on a lock file; the later ones find the
    library already built.  `out` / `defines`: another build directory and
    extra -D options (see the module docstring)."""
    out = os.path.abspath(out) if out else OUT
    lib_path = os.path.join(out, "libfdlbm.so")
    os.makedirs(out, exist_ok=True)
    extra = (["-Xptxas", "-v"] if ptxas_info else []) + [f"-D{d}" for d in defines]
    digest = _sources_digest(extra)
    stamp = os.path.join(out, "libfdlbm.sha256")
    if not force and _up_to_date(lib_path, stamp, digest):
        return lib_path
    with open(os.path.join(out, ".build.lock"), "w") as lock:
        fcntl.flock(lock, fcntl.LOCK_EX)
        try:
            if not force and _up_to_date(lib_path, stamp, digest):
                return lib_path
            return _compile_and_link(digest, stamp, extra, verbose, out)
        finally:
            fcntl.flock(lock, fcntl.LOCK_UN)


def _compile_and_link(digest: str, stamp: str, extra: list, verbose: bool, out: str) -> str:
    cc = nvcc()
    objs = []
    lib_path = os.path.join(out, "libfdlbm.so")

    def compile_one(name):
        obj = os.path.join(out, name.replace(".cu", ".o"))
        cmd = [cc, *ARCH, *COMMON, *UNITS[name], *extra, "-c", os.path.join(CSRC, name), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {name}:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return obj, (r.stdout + r.stderr)

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        for obj, log in ex.map(compile_one, list(UNITS)):
            objs.append(obj)
            if verbose and log.strip():
                print(log, file=sys.stderr)
    tmp = lib_path + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib_path)
    with open(stamp, "w") as fh:
        fh.write(digest)
    return lib_path


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--ptxas-info", action="store_true")
    ap.add_argument("--out", default=None, help="build directory (default: the in-tree fingering_dynamics_gb300/_lib)")
    ap.add_argument("--define", action="append", default=[], help="extra preprocessor definition NAME=VALUE")
    a = ap.parse_args()
    print(build(force=a.force, verbose=a.verbose or a.ptxas_info, ptxas_info=a.ptxas_info, out=a.out,
                defines=tuple(a.define)))
