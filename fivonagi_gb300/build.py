"""Build libfivonagi.so in-tree with nvcc for sm_103a.

Translation units, compiled in parallel:
  fv_step.cu (exact)  --fmad=false: no FMA contraction, bit-identical to the oracle
  fv_step.cu (fast)   --fmad=true : contracted FMAs, checked against the FP32 tolerance
  fv_api.cu           the C ABI of one simulation (host code, control-block kernels)
  fv_batch.cu         the C ABI of batches
  fv_noalloc.cu       one step attempt with no device allocation
  fv_adjoint.cu       the adjoint (its forward runs the step kernels above)
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "lib")
OBJ_DIR = os.path.join(HERE, "lib", "obj")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code is built without FMA contraction too (gcc contracts a*b+c by
# default on aarch64): the init hooks and parameter set-up must round like
# the oracle does.
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "-Xptxas", "-v", "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise FileNotFoundError("nvcc not found")


def _units():
    step = os.path.join(CSRC, "fv_step.cu")
    return [
        ("fv_step_exact.o", step, ["-DFV_VARIANT_EXACT=1", "--fmad=false"]),
        ("fv_step_fast.o", step, ["-DFV_VARIANT_EXACT=0", "--fmad=true"]),
        ("fv_api.o", os.path.join(CSRC, "fv_api.cu"), []),
        ("fv_batch.o", os.path.join(CSRC, "fv_batch.cu"), []),
        ("fv_noalloc.o", os.path.join(CSRC, "fv_noalloc.cu"), []),
        ("fv_adjoint.o", os.path.join(CSRC, "fv_adjoint.cu"), []),
    ]


def build(verbose: bool = False) -> str:
    """Compile and link; returns the library path. Raises on failure."""
    os.makedirs(OBJ_DIR, exist_ok=True)
    exe = nvcc()
    procs = []
    for obj, src, extra in _units():
        out = os.path.join(OBJ_DIR, obj)
        cmd = [exe, *ARCH, *COMMON, *extra, "-c", src, "-o", out]
        log = open(out + ".log", "w")
        procs.append((obj, cmd, subprocess.Popen(cmd, stdout=log, stderr=subprocess.STDOUT), out + ".log"))
    failed = []
    for obj, cmd, p, logp in procs:
        rc = p.wait()
        if rc != 0 or verbose:
            with open(logp) as f:
                text = f.read()
            if rc != 0:
                failed.append(f"{' '.join(cmd)}\n{text}")
            elif verbose:
                sys.stdout.write(text)
    if failed:
        raise RuntimeError("nvcc failed:\n" + "\n".join(failed))
    lib = os.path.join(LIB_DIR, "libfivonagi.so")
    objs = [os.path.join(OBJ_DIR, u[0]) for u in _units()]
    subprocess.run([exe, *ARCH, "-shared", "-o", lib, *objs, "-lcudart_static", "-lrt", "-lpthread", "-ldl"],
                   check=True)
    return lib


def ptxas_report() -> str:
    """Register/spill/shared-memory lines of the last build."""
    lines = []
    for obj, _, _ in _units():
        logp = os.path.join(OBJ_DIR, obj + ".log")
        if os.path.exists(logp):
            with open(logp) as f:
                for ln in f:
                    if "registers" in ln or "spill" in ln or "Compiling entry" in ln:
                        lines.append(f"{obj}: {ln.rstrip()}")
    return "\n".join(lines)


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
    print(ptxas_report())
