"""Builds the CUDA library libocpx_gb300.so in-tree for sm_103a with nvcc.

Translation units are compiled in parallel; the compositional flash kernels are
compiled once per component capacity (4, 6, 8, 10, 12 EoS components), each
kernel in a translation unit of its own (FLASH_PARTS), so that the large ones
compile side by side.  An object is rebuilt only when its source or a header
it includes (directly or not) is newer than it.  Objects go to
opencaeporox_gb300/_build/, the library next to this file.
Parity builds use --fmad=false: the reference is compiled without FMA
contraction, and the black-oil and assembly arithmetic is then bit-identical.
The host code is compiled with -ffp-contract=off for the same reason: GCC
contracts a*b + c into one fused operation by default where the target has
one (aarch64 does, baseline x86-64 does not), and the host sums of the C ABI
(the wells' rows, for one) must round the same on both.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libocpx_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NCM_CAPS = (4, 6, 8, 10, 12)
FLASH_PARTS = 9  # plain + dispatch, budgeted, fused, round, cooperative, SM-exclusive cooperative, post,
                 # the consumers of recomputed flash derivatives, the split cells with lane refill


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libocpx_gb300.so")


def common_flags():
    return ARCH + ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-Xcompiler", "-ffp-contract=off",
                   "-I" + os.path.join(REPO, "include"), "-I" + CSRC, "-diag-suppress", "177"]


def units():
    out = [("k_fim.cu", [], "k_fim.o"), ("ocpx_capi.cu", [], "ocpx_capi.o"), ("k_probe.cu", [], "k_probe.o"),
           ("k_noalloc.cu", [], "k_noalloc.o"), ("k_nrctl.cu", [], "k_nrctl.o"),
           ("k_linsolve.cu", [], "k_linsolve.o"), ("k_wells.cu", [], "k_wells.o")]
    for c in NCM_CAPS:
        for part in range(FLASH_PARTS):
            out.append(("k_flash_comp.cu", [f"-DOCPX_NCM={c}", f"-DOCPX_FLASH_PART={part}"],
                        f"k_flash_comp_{c}_{part}.o"))
    return out


_INCLUDE = re.compile(r'^\s*#\s*include\s+"([^"]+)"', re.M)


def _header_path(name):
    for d in (CSRC, os.path.join(REPO, "include")):
        p = os.path.join(d, name)
        if os.path.exists(p):
            return p
    return None


def _deps_mtime(src, seen=None):
    """Newest modification time of src and of every project header it
    includes, directly or through other headers (and of this script)."""
    seen = set() if seen is None else seen
    if src in seen:
        return 0.0
    seen.add(src)
    m = os.path.getmtime(src)
    with open(src, errors="replace") as f:
        for name in _INCLUDE.findall(f.read()):
            h = _header_path(name)
            if h:
                m = max(m, _deps_mtime(h, seen))
    return max(m, os.path.getmtime(__file__))


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile (if anything changed) and return the library path."""
    os.makedirs(BUILD, exist_ok=True)
    jobs = []
    for src, extra, obj in units():
        o = os.path.join(BUILD, obj)
        if not force and os.path.exists(o) and os.path.getmtime(o) >= _deps_mtime(os.path.join(CSRC, src)):
            continue
        jobs.append([nvcc_path()] + common_flags() + extra + ["-c", os.path.join(CSRC, src), "-o", o])
    objs = [os.path.join(BUILD, o) for _, _, o in units()]
    if not jobs and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(o) for o in objs):
        return LIB
    nvcc = nvcc_path()

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    # the longest compilations first
    jobs.sort(key=lambda c: "k_flash_comp" not in c[-3])
    workers = max(1, min(len(jobs), max(2, os.cpu_count() or 2)))
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose and (r.stdout or r.stderr):
                print(r.stdout + r.stderr, file=sys.stderr)
            if r.returncode != 0:
                raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
