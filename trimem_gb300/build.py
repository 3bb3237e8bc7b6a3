"""In-tree build of the native parts.

* ``libtrimem_gpu.so``: the CUDA kernels and the C ABI declared in
  ``include/trimem_gpu.h`` (nvcc, sm_103a only).
* ``core`` (``core.cpython-*.so``): the pybind11 module that mirrors the
  reference's ``trimem.core`` API on top of the C ABI.  pybind11 headers come
  from torch's include directory; the module links the C ABI library with an
  ``$ORIGIN`` rpath.

Objects go to ``trimem_gb300/_build/<machine>``; a target is rebuilt when a
source or a header is newer than it, or when it was built for another
machine architecture.
"""
import concurrent.futures as cf
import glob
import os
import platform
import subprocess
import sys
import sysconfig

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build", platform.machine())
LIB = os.path.join(PKG, "libtrimem_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC]
# The flip sweep's accept decisions are checked bit for bit against a CPU
# port; without FMA contraction both round every operation the same way.
PER_FILE = {"flips.cu": ["-fmad=false"]}


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def module_path():
    return os.path.join(PKG, "core" + sysconfig.get_config_var("EXT_SUFFIX"))


def _stale_arch(path):
    """True when the shared object at `path` was built for another machine."""
    if not os.path.exists(path):
        return False
    with open(path, "rb") as fh:
        head = fh.read(20)
    if head[:4] != b"\x7fELF":
        return True
    mach = int.from_bytes(head[18:20], "little")
    want = {"x86_64": 62, "aarch64": 183}.get(platform.machine())
    return want is not None and mach != want


def build(verbose=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    for target in (LIB, module_path()):
        if _stale_arch(target):
            os.remove(target)
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    nvcc = _nvcc()
    objs = []
    todo = []
    for src in sources:
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if _newer(obj, [src] + headers):
            todo.append([nvcc] + NVCC_FLAGS + PER_FILE.get(os.path.basename(src), []) + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, max(1, os.cpu_count() or 1))) as ex:
        for f in [ex.submit(_run, c, verbose) for c in todo]:
            f.result()
    if _newer(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"], verbose)
    mod = module_path()
    src = os.path.join(CSRC, "core_py.cpp")
    if _newer(mod, [src, LIB] + headers):
        import torch  # only for its bundled pybind11 headers

        tinc = os.path.join(os.path.dirname(torch.__file__), "include")
        pyinc = sysconfig.get_paths()["include"]
        cxx = os.environ.get("CXX", "g++")
        _run([cxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-fvisibility=hidden", "-I", pyinc, "-I", tinc,
              "-I", INCLUDE, src, "-o", mod, "-L", PKG, "-ltrimem_gpu", "-Wl,-rpath,$ORIGIN"], verbose)
    return LIB, mod


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
