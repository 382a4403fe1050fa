"""Build ``libvxg.so`` (the CUDA kernels + C ABI) in-tree for sm_103a, and
``libvxg_symbolic.so`` (the host symbolic analysis, plain C++).

Plain nvcc, one translation unit per source compiled in parallel, then one
link; the host planner is one g++ call. No torch, no cmake. Outputs:
``voltax_gb300/_lib/libvxg.so`` and ``voltax_gb300/_lib/libvxg_symbolic.so``.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "csrc"
OUT = HERE / "_lib"
INCLUDE = HERE.parent / "include"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["stamp.cu", "factor.cu", "solve.cu", "newton.cu", "capi.cu", "fused.cu",
           "factor_static.cu", "mlp.cu", "gemm_tc.cu",
           *[f"fused_{t}_{n}.cu" for t in ("f32", "f64") for n in (64, 128, 256, 512)],
           "fused_warp_f32.cu", "fused_warp_f64.cu"]


def nvcc() -> str:
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    path = Path(cuda) / "bin" / "nvcc"
    return str(path) if path.exists() else "nvcc"


def flags(extra=()) -> list[str]:
    return [*ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
            "--expt-relaxed-constexpr", f"-I{INCLUDE}", f"-I{SRC}", *extra]


def _compile(name: str, extra) -> Path:
    src = SRC / name
    obj = OUT / (src.stem + ".o")
    deps = [src, *SRC.glob("*.cuh"), INCLUDE / "vxg.h"]
    if obj.exists() and obj.stat().st_mtime > max(d.stat().st_mtime for d in deps):
        return obj
    cmd = [nvcc(), *flags(extra), "-c", str(src), "-o", str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {name}:\n{res.stdout}\n{res.stderr}")
    return obj


def build_symbolic(verbose: bool = False) -> Path:
    """The host planner library (no CUDA): rebuilt when its sources change."""
    OUT.mkdir(exist_ok=True)
    lib = OUT / "libvxg_symbolic.so"
    src = SRC / "symbolic.cpp"
    deps = [src, INCLUDE / "vxg_symbolic.h"]
    if lib.exists() and lib.stat().st_mtime > max(d.stat().st_mtime for d in deps):
        return lib
    tmp = OUT / f".libvxg_symbolic.{os.getpid()}.so"
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-shared", "-fPIC", "-pthread",
           f"-I{INCLUDE}", str(src), "-o", str(tmp)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"g++ failed on symbolic.cpp:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, lib)  # atomic: a concurrent loader never sees a partial file
    if verbose:
        print(lib)
    return lib


def build_xla(verbose: bool = False) -> Path | None:
    """The XLA FFI shim (libvxg_xla.so), only where jax exposes its FFI
    headers (jax.ffi.include_dir()); None elsewhere, or when that build
    fails (the shim is optional: nothing else depends on it)."""
    try:
        from jax import ffi
        include = ffi.include_dir()
    except Exception:
        return None
    lib = OUT / "libvxg_xla.so"
    src = SRC / "vxg_xla.cc"
    if lib.exists() and lib.stat().st_mtime > src.stat().st_mtime:
        return lib
    cuda = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-shared", "-fPIC",
           f"-I{include}", f"-I{INCLUDE}", f"-I{cuda / 'include'}", str(src), "-o", str(lib),
           f"-L{OUT}", "-lvxg", f"-Wl,-rpath,{OUT}"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        print(f"libvxg_xla.so not built (g++ failed):\n{res.stderr[-2000:]}", file=sys.stderr)
        return None
    if verbose:
        print(lib)
    return lib


def build(verbose: bool = False, extra=()) -> Path:
    build_symbolic(verbose)
    OUT.mkdir(exist_ok=True)
    lib = OUT / "libvxg.so"
    sources = [s for s in SOURCES if (SRC / s).exists()]
    with cf.ThreadPoolExecutor(max_workers=len(sources)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), sources))
    if not lib.exists() or lib.stat().st_mtime < max(o.stat().st_mtime for o in objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(lib), *map(str, objs), "-lcudart"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    if verbose:
        print(lib)
    build_xla(verbose)
    return lib


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
