"""In-tree build of the adfwi_gb300 CUDA library (``lib/libadfwi_gb300.so``) for sm_103a.

Every ``csrc/*.cu`` translation unit is compiled in parallel with nvcc into an object
file under ``_build/`` and linked into one shared library with a plain C ABI
(declared in ``include/adfwi_gb300.h``). No cmake, no torch extension machinery:
the Python host code binds the library with ctypes.
"""
import concurrent.futures
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
LIBNAME = "libadfwi_gb300.so"
BUILD = os.path.join(ROOT, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "--expt-relaxed-constexpr"]


# Extra nvcc arguments for tuning builds (for example -DADFWI_VEC_GROUPS=2); build(force=True)
# after changing them.
EXTRA = os.environ.get("ADFWI_NVCC_EXTRA", "").split()


def nvcc_path():
    cand = shutil.which("nvcc")
    if cand:
        return cand
    for base in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if base and os.path.exists(os.path.join(base, "bin", "nvcc")):
            return os.path.join(base, "bin", "nvcc")
    raise RuntimeError("nvcc not found: the adfwi_gb300 CUDA library cannot be built")


def library_path():
    return os.path.join(LIBDIR, LIBNAME)


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)) + [
        os.path.join(ROOT, "include", "adfwi_gb300.h")]


def _stale(out, inputs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(i) > t for i in inputs)


def build(force=False, verbose=False):
    """Compile and link the library if any source is newer than it. Returns its path."""
    nvcc = nvcc_path()
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    deps = _deps()
    srcs = _sources()
    objs = [os.path.join(BUILD, os.path.basename(s)[:-3] + ".o") for s in srcs]
    jobs = [(s, o) for s, o in zip(srcs, objs) if force or _stale(o, deps)]

    def compile_one(job):
        src, obj = job
        cmd = [nvcc, *ARCH, *FLAGS, *EXTRA, "-I", os.path.join(ROOT, "include"), "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
        if verbose:
            print(" ".join(cmd))
        return obj

    if jobs:
        with concurrent.futures.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 1)) as ex:
            list(ex.map(compile_one, jobs))
    lib = library_path()
    if force or jobs or _stale(lib, objs):
        tmp = lib + ".tmp"
        cmd = [nvcc, *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
        os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(verbose=True))
