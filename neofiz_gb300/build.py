"""In-tree build of libneofiz_gpu.so for sm_103a.

Translation units are compiled in parallel with nvcc and linked into one shared object in
neofiz_gb300/_build. Flags that matter for correctness:
  --fmad=false              no multiply-add contraction in device code, so every expression
                            rounds where the reference's Java does;
  -Xcompiler -ffp-contract=off   the same for the host-side set-up arithmetic (lumped mass,
                            node slots, initial step), which matters on the aarch64 host.
k_batch_comp.cu alone (the compensated batch form, which has no bit-level twin) is built with
float contraction, fast float division/square root and denormal flushing instead.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBRARY = os.path.join(BUILD, "libneofiz_gpu.so")
SOURCES = ["api.cu", "api_batch.cu", "k_step.cu", "k_contact.cu", "k_scan.cu", "k_mixed.cu",
           "k_batch.cu", "k_batch_comp.cu", "k_adjoint.cu", "k_film.cu", "noalloc.cu",
           "k_peak.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-prec-div=true",
              "-prec-sqrt=true", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
              "-Xptxas", "-O3"]


# The compensated batch form has no bit-level twin; its translation unit is built for speed
# (float multiply-add contraction, fast float division and square root, denormals flushed).
FAST_FLOAT_SOURCES = {"k_batch_comp.cu"}
FAST_FLOAT_FLAGS = ["--fmad=true", "-prec-div=false", "-prec-sqrt=false", "-ftz=true"]


def flags_for(src: str):
    if src not in FAST_FLOAT_SOURCES:
        return NVCC_FLAGS
    strict = ("--fmad=false", "-prec-div=true", "-prec-sqrt=true")
    return [f for f in NVCC_FLAGS if f not in strict] + FAST_FLOAT_FLAGS


# The host-side set-up library (the defect field's deterministic arithmetic), plain C.
HOST_LIBRARY = os.path.join(BUILD, "libneofiz_host.so")
HOST_SOURCES = ["defect_field.c"]
HOST_FLAGS = ["-O2", "-std=gnu11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
              "-pthread", "-fvisibility=hidden"]


def build_host(force: bool = False) -> str:
    """Compiles libneofiz_host.so with contraction off (no fused multiply-add contraction, so
    the field is the same on every host)."""
    os.makedirs(BUILD, exist_ok=True)
    deps = [os.path.join(CSRC, f) for f in HOST_SOURCES]
    deps += [os.path.join(CSRC, "nf_math.h"), os.path.join(CSRC, "nf_math_tables.h")]
    if not force and os.path.exists(HOST_LIBRARY):
        t = os.path.getmtime(HOST_LIBRARY)
        if all(os.path.getmtime(d) <= t for d in deps):
            return HOST_LIBRARY
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        raise RuntimeError("no C compiler (gcc) found for libneofiz_host.so")
    tmp = f"{HOST_LIBRARY}.{os.getpid()}.tmp"
    cmd = [cc, *HOST_FLAGS, *[os.path.join(CSRC, f) for f in HOST_SOURCES], "-o", tmp, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"gcc failed on the host library:\n{r.stderr}")
    os.replace(tmp, HOST_LIBRARY)
    return HOST_LIBRARY


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _deps():
    out = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    out.append(os.path.join(HERE, "..", "include", "neofiz.h"))
    return out


def build(force: bool = False, verbose: bool = False, extra=()) -> str:
    os.makedirs(BUILD, exist_ok=True)
    build_host(force)
    if not force and os.path.exists(LIBRARY):
        t = os.path.getmtime(LIBRARY)
        if all(os.path.getmtime(d) <= t for d in _deps()):
            return LIBRARY
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        cmd = [cc, *ARCH, *flags_for(src), *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIBRARY + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIBRARY)
    return LIBRARY


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True,
                extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else []))
