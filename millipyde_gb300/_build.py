"""In-tree build of the CUDA library and the CPython extension.

Produces, next to this file:
  libmillipyde_gb300.so          the C-ABI library (CUDA kernels for sm_103a,
                                 cudart linked statically)
  _millipyde<EXT_SUFFIX>         the CPython extension (C), linked against it

No setuptools, no cmake: nvcc and gcc are invoked directly, translation units
compile in parallel, and nothing is rebuilt when outputs are newer than every
source.  The reference built one setuptools extension with hipcc
(setup.py:48-66); this build targets sm_103a only.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")

CU_SOURCES = ["mp_vh_c3.cu", "mp_vc_c3.cu", "mp_vc_c3_lo.cu", "mp_vc_c3_mid.cu", "mp_vh_c1.cu", "mp_vh_c4.cu", "mp_vc_c4.cu", "mp_vb_c3.cu", "mp_vb_c1.cu", "mp_vb_c4.cu", "mp_vd_c3.cu", "mp_vd_c1.cu", "mp_vd_c4.cu", "mp_stream_c3.cu", "mp_stream_grey3.cu",
              "mp_stream_c1.cu", "mp_runtime.cu", "mp_kernels.cu", "mp_stream.cu", "mp_rot.cu", "mp_vh.cu",
              "mp_ops.cu", "mp_grad.cu", "mp_noalloc.cu", "mp_legacy.cu", "mp_fuse.cu", "mp_fuse_c1.cu",
              "mp_fuse_c3.cu"]
C_SOURCES = ["py_module.c", "py_objects.c", "py_compose.c"]
HEADERS = ["mp_internal.cuh", "mp_stream.cuh", "mp_vh.cuh", "mp_fuse.cuh", "py_common.h"]

LIB_NAME = "libmillipyde_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build millipyde_gb300")


def ext_path() -> str:
    return os.path.join(PKG, "_millipyde" + sysconfig.get_config_var("EXT_SUFFIX"))


def lib_path() -> str:
    return os.path.join(PKG, LIB_NAME)


def _newest(paths) -> float:
    return max(os.path.getmtime(p) for p in paths if os.path.exists(p))


def _stale(out: str, deps) -> bool:
    return not os.path.exists(out) or os.path.getmtime(out) < _newest(deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n  %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r


def build(force: bool = False, verbose: bool = False) -> None:
    """Compile the library and the extension if sources changed."""
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "millipyde_gb300.h")]
    nvcc = _nvcc()
    cu_flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                       "-Xcompiler", "-Wall", "-I" + INCLUDE]
    objs, jobs = [], []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc] + cu_flags + ["-c", s, "-o", o])
    if jobs:
        with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            for r in ex.map(_run, jobs):
                if verbose and (r.stdout or r.stderr):
                    print(r.stdout + r.stderr)
    lib = lib_path()
    if force or jobs or _stale(lib, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", lib] + objs)

    ext = ext_path()
    c_srcs = [os.path.join(CSRC, c) for c in C_SOURCES]
    if force or _stale(ext, c_srcs + headers + [lib]):
        import numpy
        cc = os.environ.get("CC", "gcc")
        inc = [sysconfig.get_paths()["include"], numpy.get_include(), INCLUDE]
        cmd = [cc, "-O2", "-fPIC", "-shared", "-std=c11", "-Wall", "-Wno-missing-field-initializers"]
        cmd += ["-I" + i for i in inc] + c_srcs
        cmd += ["-L" + PKG, "-l:" + LIB_NAME, "-Wl,-rpath,$ORIGIN", "-o", ext]
        r = _run(cmd)
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print("built", lib_path(), ext_path())
