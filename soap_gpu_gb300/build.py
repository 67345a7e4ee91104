"""Build recipe for libsoapgb (sm_103a) and the drop-in executables.

Everything is compiled in-tree with nvcc directly (no cmake, no torch extension):

* ``soap_gpu_gb300/lib/libsoapgb.so`` -- the C-ABI library (``include/soapgb.h``);
* ``soap_gpu_gb300/bin/{SOAP_initialize, SOAP_integration, SOAP_integration_solar,
  SOAP_resolution, BIS_FIT2}`` -- argv/file compatible replacements of the
  reference's executables, linked against the library.

Translation units compile in parallel; a unit is rebuilt when it or a header is
newer than its object.  Host code is compiled with ``-ffp-contract=off`` so x86 and
Arm hosts round identically.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
TOOLS = os.path.join(CSRC, "tools")
OBJ = os.path.join(PKG, "_obj")
LIBDIR = os.path.join(PKG, "lib")
BINDIR = os.path.join(PKG, "bin")
LIB = os.path.join(LIBDIR, "libsoapgb.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
TOOL_NAMES = ["SOAP_initialize", "SOAP_integration", "SOAP_integration_solar", "SOAP_resolution", "BIS_FIT2"]


def _nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsoapgb")
    return cand


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + [os.path.join(ROOT, "include", "soapgb.h")]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("build failed: %s\n%s" % (" ".join(cmd), p.stdout))
    return p.stdout


def build(verbose: bool = False, force: bool = False, jobs: int = 0) -> str:
    nvcc = _nvcc()
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(BINDIR, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    hdrs = _headers()
    common = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                     "-I", os.path.join(ROOT, "include")]
    jobs = jobs or min(8, os.cpu_count() or 4)

    def compile_one(src):
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        if force or _stale(obj, [src] + hdrs):
            out = _run([nvcc] + common + ["-c", src, "-o", obj])
            if verbose and out.strip():
                print(out)
        return obj

    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(compile_one, srcs))
    if force or _stale(LIB, objs):
        tmp = LIB + ".tmp.%d" % os.getpid()
        _run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart", "-lpthread"])
        os.replace(tmp, LIB)

    def link_tool(name):
        src = os.path.join(TOOLS, name.replace("_solar", "") + ".cpp") if name != "SOAP_integration_solar" \
            else os.path.join(TOOLS, "SOAP_integration.cpp")
        exe = os.path.join(BINDIR, name)
        deps = [src, LIB, os.path.join(TOOLS, "tool_common.h"), os.path.join(ROOT, "include", "soapgb.h")]
        if force or _stale(exe, deps):
            flags = ["-DSOAPGB_SOLAR=1"] if name == "SOAP_integration_solar" else []
            _run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "include")] + flags +
                 [src, "-o", exe, "-L", LIBDIR, "-lsoapgb", "-Wl,-rpath,$ORIGIN/../lib"])
        return exe

    if os.path.isdir(TOOLS):
        with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
            list(ex.map(link_tool, TOOL_NAMES))
    build_torch_ops(verbose=verbose)
    return LIB


def _torch_ops_registered() -> bool:
    """torch.ops.soapgb is registered in this process (torch imported and the operator
    library loaded)."""
    if "torch" not in sys.modules:
        return False
    try:
        sys.modules["torch"].ops.soapgb.synchronize
        return True
    except (AttributeError, RuntimeError):
        return False


TORCH_SRC = os.path.join(CSRC, "torch", "soapgb_torch.cpp")
TORCH_OPS = os.path.join(LIBDIR, "soapgb_torch.so")


def build_torch_ops(verbose: bool = False) -> str:
    """The torch operators over libsoapgb (csrc/torch/soapgb_torch.cpp: torch.ops.soapgb.*)
    as lib/soapgb_torch.so, through torch.utils.cpp_extension (a C++ source linked
    against libsoapgb and the CUDA runtime; no device code)."""
    deps = [TORCH_SRC, LIB, os.path.join(ROOT, "include", "soapgb.h")]
    if not _stale(TORCH_OPS, deps):
        return TORCH_OPS
    if _torch_ops_registered():
        # cpp_extension.load also loads what it builds, and torch takes an operator
        # namespace once per process: a process that holds the operators already builds
        # the new copy in a child process
        _run([sys.executable, "-c", "import sys; sys.path.insert(0, %r); "
              "from soap_gpu_gb300.build import build_torch_ops; build_torch_ops()" % ROOT])
        return TORCH_OPS
    import torch.utils.cpp_extension as ce
    bdir = os.path.join(OBJ, "torch_ops")
    os.makedirs(bdir, exist_ok=True)
    ce.load(name="soapgb_torch", sources=[TORCH_SRC], extra_include_paths=[os.path.join(ROOT, "include")],
            extra_cflags=["-O2"], extra_ldflags=["-L" + LIBDIR, "-lsoapgb", "-Wl,-rpath," + LIBDIR],
            with_cuda=True, build_directory=bdir, is_python_module=False, verbose=verbose)
    built = os.path.join(bdir, "soapgb_torch.so")
    tmp = TORCH_OPS + ".tmp.%d" % os.getpid()
    shutil.copyfile(built, tmp)
    os.replace(tmp, TORCH_OPS)
    return TORCH_OPS


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
    print(LIB)
