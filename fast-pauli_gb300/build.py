"""Build recipe of the GB300 Pauli engine (no cmake; nvcc + g++ directly).

Products (in-tree, git-ignored):
  fast-pauli_gb300/fast_pauli/libfpg.so            -- CUDA kernels + C ABI (include/fpg.h)
  fast-pauli_gb300/fast_pauli/_fast_pauli*.so      -- Python module over the C++ host API

Translation units compile in parallel; sm_103a only.
"""

from __future__ import annotations

import os
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor

PKG_ROOT = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG_ROOT)
CSRC = os.path.join(PKG_ROOT, "csrc")
CPP_INC = os.path.join(PKG_ROOT, "cpp", "include")
ABI_INC = os.path.join(REPO, "include")
OUT_DIR = os.path.join(PKG_ROOT, "fast_pauli")
OBJ_DIR = os.path.join(PKG_ROOT, "_build")
LIB = os.path.join(OUT_DIR, "libfpg.so")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["k_expect.cu", "k_expect_wht.cu", "k_apply.cu", "k_contract.cu", "k_contract_tc.cu", "k_noalloc.cu",
              "batch.cu", "k_expect_pair.cu", "k_expect_tile.cu", "k_expect_marg.cu", "k_square.cu", "k_product.cu", "k_df64.cu",
              "k_peak.cu"]
CPP_SOURCES = ["capi.cpp", "server.cpp"]


def _cuda_include() -> str:
    return os.path.join(CUDA_HOME, "include")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    if os.environ.get("FPG_BUILD_VERBOSE"):
        sys.stderr.write(r.stdout + r.stderr)


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _headers() -> list[str]:
    hs = []
    for d in (CSRC, CPP_INC, ABI_INC):
        for f in os.listdir(d):
            if f.endswith((".h", ".hpp", ".cuh")):
                hs.append(os.path.join(d, f))
    return hs


def build_lib(force: bool = False, verbose_ptxas: bool = False) -> str:
    os.makedirs(OBJ_DIR, exist_ok=True)
    hdrs = _headers()
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        if not os.path.exists(s):
            continue
        o = os.path.join(OBJ_DIR, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-I", CSRC, "-I", ABI_INC, "-c", s, "-o", o]
            if verbose_ptxas:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ_DIR, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-pthread", "-Wall", "-Wextra", "-I", CSRC, "-I", ABI_INC,
                         "-I", _cuda_include(), "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        list(ex.map(_run, jobs))
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + f".tmp{os.getpid()}"
        _run([NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart", "-Xcompiler", "-pthread"])
        os.replace(tmp, LIB)
    return LIB


def build_module(force: bool = False) -> str:
    """pybind11 module fast_pauli._fast_pauli (pybind11 headers bundled with torch)."""
    import torch  # only for the location of its bundled pybind11 headers

    torch_inc = os.path.join(os.path.dirname(torch.__file__), "include")
    py_inc = sysconfig.get_paths()["include"]
    suffix = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    target = os.path.join(OUT_DIR, "_fast_pauli" + suffix)
    src = os.path.join(PKG_ROOT, "cpp", "src", "module.cpp")
    if not os.path.exists(src):
        return ""
    if force or _stale(target, [src, LIB] + _headers()):
        tmp = target + f".tmp{os.getpid()}"
        _run(["g++", "-O2", "-std=c++20", "-fPIC", "-shared", "-fvisibility=hidden",
              "-I", CPP_INC, "-I", ABI_INC, "-I", _cuda_include(), "-I", torch_inc, "-I", py_inc,
              src, "-o", tmp, "-L", OUT_DIR, "-lfpg", "-Wl,-rpath,$ORIGIN",
              "-L", os.path.join(CUDA_HOME, "lib64"), "-lcudart"])
        os.replace(tmp, target)
    return target


def build(force: bool = False) -> None:
    build_lib(force)
    build_module(force)


if __name__ == "__main__":
    build(force="--force" in sys.argv)
    print("built", LIB)
