"""Builds the oracle (test infrastructure, never part of the product).

* ``build()``: the C restatement ocpx_oracle.c -> oracle/_build/liboracle.so
  (cc -O3 -ffp-contract=off -fopenmp; no FMA contraction, like a baseline
  x86-64 build of the reference; -O3 vectorizes loops without reordering any
  sum, so its results equal an -O2 build's).
* ``build_reference_if_present()``: where the reference sources exist (the
  directory in OCPX_REFERENCE_DIR, else the checkout this recipe reads by
  default), the reference itself via oracle/ref/Makefile into oracle/_ref/
  (used to regenerate the golden fixtures).  This recipe is the one place
  that names the checkout's default location.
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "liboracle.so")
REF = os.environ.get("OCPX_REFERENCE_DIR", "/root/reference")


VARIANTS = {
    # the restatement itself
    "exact": ("ocpx_oracle.c", LIB),
    # the same code with every transcendental result moved by one ulp (ulp_nudge.c):
    # measures the reference algorithm's sensitivity to libm rounding
    "ulp": ("ulp_nudge.c", os.path.join(OUT, "liboracle_ulp.so")),
}


def build(force: bool = False, variant: str = "exact") -> str:
    os.makedirs(OUT, exist_ok=True)
    main, lib = VARIANTS[variant]
    src = [os.path.join(HERE, main)]
    deps = [os.path.join(HERE, f) for f in ("ocpx_oracle.c", "ocpx_oracle.h", main)]
    if not force and os.path.exists(lib) and os.path.getmtime(lib) >= max(os.path.getmtime(d) for d in deps):
        return lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        raise RuntimeError("no C compiler for the oracle")
    tmp = lib + ".tmp"
    cmd = [cc, "-O3", "-g0", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-shared", "-fPIC",
           "-I", HERE, "-o", tmp] + src + ["-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    os.replace(tmp, lib)
    return lib


def build_reference_if_present() -> str | None:
    if not os.path.isdir(os.path.join(REF, "src")):
        return None
    r = subprocess.run(["make", "-C", os.path.join(HERE, "ref"), "-j8", f"REF={REF}"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference oracle build failed:\n" + r.stdout[-2000:] + r.stderr[-2000:])
    return os.path.join(HERE, "_ref", "ocp_ref_dump")


def build_binding() -> str:
    """The reference-side binding of the GPU library compiled against the
    reference's headers (oracle/ref/Makefile, target gpu_binding); needs the
    library built and the reference's sources."""
    r = subprocess.run(["make", "-C", os.path.join(HERE, "ref"), "-j8", "gpu_binding", f"REF={REF}"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("binding build failed:\n" + r.stdout[-2000:] + r.stderr[-2000:])
    return os.path.join(HERE, "_ref", "ocp_gpu_binding")


if __name__ == "__main__":
    print(build(force=True))
    print(build_reference_if_present())
