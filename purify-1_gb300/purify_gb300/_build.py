"""Builds the native library ``lib/libpurify_gb300.so`` in-tree.

CUDA sources are compiled by nvcc for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``); host sources by g++.  Objects
are rebuilt when a source or any header under ``csrc/`` or ``include/`` is
newer.  Translation units compile in parallel.
"""
import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))  # purify-1_gb300/
REPO_ROOT = os.path.dirname(PKG_ROOT)
CSRC = os.path.join(PKG_ROOT, "csrc")
INCLUDE = os.path.join(REPO_ROOT, "include")
BUILD_DIR = os.path.join(PKG_ROOT, "_build")
LIB_DIR = os.path.join(PKG_ROOT, "lib")
LIB_PATH = os.path.join(LIB_DIR, "libpurify_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home():
    env = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if env and os.path.isdir(env):
        return env
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return "/usr/local/cuda"


def _newest_header_mtime():
    hdrs = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh"))
    hdrs += glob.glob(os.path.join(INCLUDE, "*.h")) + glob.glob(os.path.join(INCLUDE, "**", "*.h"),
                                                               recursive=True)
    return max([os.path.getmtime(h) for h in hdrs] + [0.0])


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stderr


def build(verbose=False, jobs=None):
    """Compiles and links the library; returns its path."""
    home = cuda_home()
    nvcc = os.path.join(home, "bin", "nvcc")
    if not os.path.exists(nvcc):
        nvcc = shutil.which("nvcc") or "nvcc"
    cuinc = os.path.join(home, "include")
    culib = None
    for cand in ("lib64", "lib", os.path.join("targets", "sbsa-linux", "lib"),
                 os.path.join("targets", "x86_64-linux", "lib")):
        p = os.path.join(home, cand)
        if os.path.exists(os.path.join(p, "libcudart.so")) or os.path.exists(
                os.path.join(p, "libcufft.so")):
            culib = p
            break
    culib = culib or os.path.join(home, "lib64")
    os.makedirs(BUILD_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    hdr_time = _newest_header_mtime()
    cmds, objs = [], []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp"))):
        obj = os.path.join(BUILD_DIR, os.path.basename(src) + ".o")
        objs.append(obj)
        if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), hdr_time):
            continue
        if src.endswith(".cu"):
            cmd = [nvcc, "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC",
                   "-I", CSRC, "-I", INCLUDE, "-c", src, "-o", obj]
            if verbose:
                cmd.insert(4, "-Xptxas=-v")
        else:
            cmd = ["g++", "-std=c++17", "-O3", "-fPIC", "-fopenmp", "-Wall", "-Wno-unused-function",
                   "-I", CSRC, "-I", INCLUDE, "-I", cuinc, "-c", src, "-o", obj]
        cmds.append(cmd)
    if cmds:
        with ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
            for msg in ex.map(_compile, cmds):
                if verbose and msg:
                    sys.stderr.write(msg)
    lib_time = os.path.getmtime(LIB_PATH) if os.path.exists(LIB_PATH) else -1
    if cmds or lib_time < max(os.path.getmtime(o) for o in objs):
        tmp = LIB_PATH + ".tmp"
        link = ["g++", "-shared", "-o", tmp, *objs, "-L", culib, "-Wl,-rpath," + culib,
                "-lcufft", "-lcudart", "-fopenmp"]
        _compile(link)
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
