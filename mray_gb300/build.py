"""Builds the CUDA library ``mray_gb300/libmraygb.so`` in-tree for sm_103a.

Each translation unit is compiled by nvcc in parallel and the objects are linked into one shared library with
the CUDA runtime linked statically.  ``mese.cu`` and ``coding.cu`` are compiled without FMA contraction so
that the FP32 MESE algebra and the quantizer round exactly as the reference's separately rounded operations;
the marching kernels keep contraction on.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(HERE, "libmraygb.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include"),
          "--expt-relaxed-constexpr"]

# (source, extra flags)
SOURCES = [
    ("generate.cu", []),
    ("reconstruct.cu", []),
    ("scan.cu", []),
    ("compact_noalloc.cu", []),
    ("particles.cu", []),
    ("adjoint.cu", []),
    ("mese.cu", ["--fmad=false"]),
    ("mese_f64.cu", []),
    ("mese_ff.cu", []),
    ("coding.cu", ["--fmad=false"]),
    ("quant_curve.cu", ["--fmad=false"]),
    ("uncertainty.cu", ["--fmad=false"]),
    ("reference.cu", []),
    ("scattering.cu", []),
    ("lz4_block.cpp", []),
    ("arith_coder.cpp", ["-Xcompiler", "-ffp-contract=off"]),
    ("moment_file.cpp", []),
    ("libm_trig_host.cpp", []),
    ("fp32_rate.cu", []),
    ("api.cpp", ["-x", "cu"]),
]

# The sinf / cosf exception table (csrc/libm_trig_core.h): generated by running the host C library over every float
# of [-pi, pi], then linked into the library as a read-only blob.
TRIG_GEN_SRC = os.path.join(CSRC, "libm_trig_gen.cpp")
TRIG_GEN = os.path.join(BUILD_DIR, "libm_trig_gen")
TRIG_TABLE = os.path.join(BUILD_DIR, "libm_trig_table.bin")
TRIG_ASM = os.path.join(BUILD_DIR, "libm_trig_table.S")
TRIG_OBJ = os.path.join(BUILD_DIR, "libm_trig_table.o")


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build mray_gb300")


def _compile(src: str, extra: list[str], verbose: bool) -> str:
    obj = os.path.join(BUILD_DIR, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose:
        sys.stderr.write(r.stderr)
    return obj


def _host_cxx() -> str:
    for cand in (os.environ.get("CXX"), shutil.which("g++"), shutil.which("c++")):
        if cand:
            return cand
    raise RuntimeError("no host C++ compiler found (g++)")


def _run(cmd: list[str], what: str) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{what} failed:\n{r.stdout}\n{r.stderr}")


def _trig_table() -> str:
    """Compile and run the table generator; assemble the table into an object file."""
    _run([_host_cxx(), "-O2", "-std=c++17", "-ffp-contract=off", "-pthread", TRIG_GEN_SRC, "-o", TRIG_GEN],
         "compiling libm_trig_gen")
    _run([TRIG_GEN, TRIG_TABLE], "generating the sinf / cosf table")
    with open(TRIG_ASM, "w") as f:
        f.write("\t.section .rodata.mraygb_libm_trig,\"a\"\n"
                "\t.balign 16\n"
                "\t.globl mraygb_libm_trig_table_begin\n"
                "\t.hidden mraygb_libm_trig_table_begin\n"
                "mraygb_libm_trig_table_begin:\n"
                f"\t.incbin \"{TRIG_TABLE}\"\n"
                "\t.globl mraygb_libm_trig_table_end\n"
                "\t.hidden mraygb_libm_trig_table_end\n"
                "mraygb_libm_trig_table_end:\n"
                "\t.section .note.GNU-stack,\"\",%progbits\n")
    cc = os.environ.get("CC") or shutil.which("gcc") or "cc"
    _run([cc, "-c", TRIG_ASM, "-o", TRIG_OBJ], "assembling the sinf / cosf table")
    return TRIG_OBJ


def _stale() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [
        os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile (if stale) and return the path of libmraygb.so."""
    if not force and not _stale():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES) + 1) as ex:
        table = ex.submit(_trig_table)
        objs = list(ex.map(lambda s: _compile(s[0], s[1], verbose), SOURCES))
        objs.append(table.result())
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs, "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
