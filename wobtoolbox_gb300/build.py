"""Builds the engine's shared library in-tree: wobtoolbox_gb300/_lib/libwob_gb300.so.

CUDA units are compiled by nvcc for sm_103a only, in parallel; the host scene builder by the host
C++ compiler. Walk kernels are built with -fmad=false and host code with -ffp-contract=off: every
formula on the walk is evaluated in plain IEEE single precision (fused multiply-adds only where the
source writes fmaf), which is what makes the engine's paths reproducible on the CPU.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
BUILD = os.path.join(HERE, "_build", platform.machine())  # objects per host architecture
LIB = os.path.join(OUT, "libwob_gb300.so")
FMA_OUT = os.path.join(OUT, "fma")
FMA_LIB = os.path.join(FMA_OUT, "libwob_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["capi.cu", "kernels_dispatch.cu", "k2_generic_domain.cu", "k2_generic_boundary.cu", "k3_generic_domain.cu",
              "k3_generic_boundary.cu", "k2_fast.cu", "k3_fast.cu", "k_batch.cu", "k_cv.cu",
              "k2_multi_rhs.cu", "k3_multi_rhs.cu", "mlp.cu", "scene_build_gpu.cu",
              "k_vpl.cu", "k_wos.cu", "k_sl.cu", "k_cv_tables.cu", "mlp_train.cu", "k_probe.cu", "k_fwd_wave.cu", "k_sample.cu"]
# Units outside the bit-exact walk, compiled with FMA contraction: the control-variate tables
# (checked against a float64 restatement with a tolerance, not path for path) and the fused
# training step (checked against float64 autograd with a tolerance).
CONTRACTED_SOURCES = {"k_cv_tables.cu", "mlp_train.cu"}
CPP_SOURCES = ["scene_build.cpp"]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


APPS = os.path.join(HERE, "apps")
# app -> (source under apps/, WOB_APP_DIM, links the CUDA runtime for device buffers)
APP_BINARIES = {
    "general_2d": ("general.cpp", 2, False),
    "general_3d": ("general.cpp", 3, False),
    "potential_flow_vpl": ("potential_flow_vpl.cpp", 2, True),
    "poisson_equation": ("poisson_equation.cpp", 2, False),
    "boundary_estimate": ("boundary_estimate.cpp", 2, True),
    "simple_wob_and_wos": ("simple_wob_and_wos.cpp", 2, True),
}


def app_path(name: str) -> str:
    return os.path.join(OUT, name)


def _deps() -> list[str]:
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(INCLUDE, "wob_capi.h"))
    files.append(os.path.abspath(__file__))
    return files


def build_apps(force: bool = False) -> list[str]:
    """The JSON apps (apps/*.cpp, one executable per reference app), linked against the library."""
    cxx = os.environ.get("CXX", "g++")
    deps = [os.path.join(APPS, f) for f in os.listdir(APPS)] + [os.path.join(INCLUDE, "wob_gb300.hpp"),
                                                                 os.path.join(INCLUDE, "wob_capi.h"), LIB]
    jobs, outs = [], []
    cuda = os.path.dirname(os.path.dirname(nvcc_path()))
    for name, (src, dim, cudart) in APP_BINARIES.items():
        out = app_path(name)
        outs.append(out)
        extra = ["-I", os.path.join(cuda, "include"), "-L", os.path.join(cuda, "lib64"), "-lcudart",
                 "-Wl,-rpath," + os.path.join(cuda, "lib64")] if cudart else []
        if force or _stale(out, deps):
            jobs.append([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-fopenmp", "-Wall", f"-DWOB_APP_DIM={dim}",
                         "-I", INCLUDE, os.path.join(APPS, src), "-o", out + ".tmp", "-L", OUT,
                         "-lwob_gb300", "-Wl,-rpath,$ORIGIN"] + extra)
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for j, proc in zip(jobs, ex.map(lambda j: subprocess.run(j, capture_output=True, text=True), jobs)):
            if proc.returncode != 0:
                raise RuntimeError("build failed:\n" + " ".join(j) + "\n" + proc.stdout + proc.stderr)
            os.replace(j[j.index("-o") + 1], j[j.index("-o") + 1][:-4])
    return outs


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + proc.stdout + proc.stderr)


def cu_flags(extra: list[str] | None = None, contract: bool = False) -> list[str]:
    return ARCH + ["-O3", "-std=c++17", "-lineinfo", "-fmad=true" if contract else "-fmad=false",
                   "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", INCLUDE] + (extra or [])


def _obj_stale(obj: str, src: str, headers: list[str]) -> bool:
    """An object is rebuilt when it is missing or older than its source, a header or this file."""
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in [src] + headers)


def build(verbose: bool = False, force: bool = False, ptxas_info: bool = False, fma: bool = False) -> str:
    """Compiles the library if any source changed; returns its path. fma=True builds the
    measurement variant into _lib/fma/ instead: every CUDA unit with FMA contraction (-fmad=true),
    host code unchanged, no apps -- its paths are not bit-identical to the oracle's; it exists to
    measure what the bit-exact build costs (bench.py --workload fmad)."""
    out_dir, build_dir, lib_path = (FMA_OUT, BUILD + "_fma", FMA_LIB) if fma else (OUT, BUILD, LIB)
    os.makedirs(out_dir, exist_ok=True)
    os.makedirs(build_dir, exist_ok=True)
    deps = _deps()
    if not force and not ptxas_info and not _stale(lib_path, deps):
        if not fma:
            build_apps()
        return lib_path
    nvcc = nvcc_path()
    cxx = os.environ.get("CXX", "g++")
    jobs = []
    objs = []
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp", ".h"))]
    headers += [os.path.join(INCLUDE, "wob_capi.h"), os.path.abspath(__file__)]
    for src in CU_SOURCES:
        obj = os.path.join(build_dir, src.replace(".cu", ".o"))
        objs.append(obj)
        if not (force or ptxas_info) and not _obj_stale(obj, os.path.join(CSRC, src), headers):
            continue
        extra = ["-Xptxas", "-v"] if ptxas_info else []
        jobs.append([nvcc] + cu_flags(extra, contract=fma or src in CONTRACTED_SOURCES) +
                    ["-c", os.path.join(CSRC, src), "-o", obj])
    for src in CPP_SOURCES:
        obj = os.path.join(build_dir, src.replace(".cpp", ".o"))
        objs.append(obj)
        if not force and not _obj_stale(obj, os.path.join(CSRC, src), headers):
            continue
        jobs.append([cxx, "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-c",
                     os.path.join(CSRC, src), "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        futs = [ex.submit(subprocess.run, j, capture_output=True, text=True) for j in jobs]
        for j, f in zip(jobs, futs):
            proc = f.result()
            if proc.returncode != 0:
                raise RuntimeError("build failed:\n" + " ".join(j) + "\n" + proc.stdout + proc.stderr)
            if verbose or ptxas_info:
                sys.stderr.write(proc.stderr)
    tmp = lib_path + ".tmp"
    _run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-Xcompiler", "-fPIC"])
    os.replace(tmp, lib_path)
    if not fma:
        build_apps(force=True)
    return lib_path


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv, ptxas_info="--ptxas" in sys.argv, fma="--fma" in sys.argv))
