"""In-tree build of the CUDA library libpwa_gb300.so for sm_103a.

Every translation unit in csrc/ is compiled by nvcc in parallel and linked
into rootpwa_gb300/libpwa_gb300.so next to this file.  Objects go to
rootpwa_gb300/_build/.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpwa_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no FMA contraction, so that it rounds the same on x86-64 and
# aarch64 hosts (gcc contracts a*b+c by default on aarch64)
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", INCLUDE, "-I", CSRC]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _headers_mtime():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return max(os.path.getmtime(h) for h in hs)


def _compile(src, ptxas_verbose=False):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if (os.path.exists(obj) and os.path.getmtime(obj) >= os.path.getmtime(src)
            and os.path.getmtime(obj) >= _headers_mtime()):
        return obj, ""
    cmd = [_nvcc()] + ARCH + FLAGS + (["-Xptxas", "-v"] if ptxas_verbose else []) + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    return obj, r.stdout + r.stderr


def build(force=False, ptxas_verbose=False, verbose=False):
    """Compile and link libpwa_gb300.so; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    if force:
        for f in os.listdir(BUILD):
            os.remove(os.path.join(BUILD, f))
    srcs = sources()
    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        results = list(ex.map(lambda s: _compile(s, ptxas_verbose), srcs))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            if log:
                sys.stdout.write(log)
    if (not os.path.exists(LIB) or force
            or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs)):
        cmd = [_nvcc()] + ARCH + ["-shared", "-cudart", "shared", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    return LIB


LIB_DEBUG = os.path.join(HERE, "libpwa_gb300_debug.so")
BUILD_DEBUG = os.path.join(HERE, "_build_debug")
# translation units rebuilt with the shared-memory bounds checks compiled in
DEBUG_SOURCES = ("fdf_kernels.cu", "fdf_fused.cu", "fdf_narrow.cu")


def build_debug():
    """libpwa_gb300_debug.so: the release objects, except the FdF kernels,
    which are compiled with -DPWA_DEBUG_CHECKS (every shared-memory access
    checked against its region; a failed check sets a device error flag and
    skips the access).  Loaded instead of the release library when the
    environment has PWA_GB300_DEBUG=1."""
    build()
    os.makedirs(BUILD_DEBUG, exist_ok=True)
    objs = []
    todo = []
    for src in sources():
        name = os.path.basename(src)
        if name in DEBUG_SOURCES:
            obj = os.path.join(BUILD_DEBUG, name + ".o")
            if not (os.path.exists(obj) and os.path.getmtime(obj) >= os.path.getmtime(src)
                    and os.path.getmtime(obj) >= _headers_mtime()):
                todo.append((src, obj))
            objs.append(obj)
        else:
            objs.append(os.path.join(BUILD, name + ".o"))

    def comp(job):
        src, obj = job
        cmd = [_nvcc()] + ARCH + FLAGS + ["-DPWA_DEBUG_CHECKS", "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))

    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, len(todo))) as ex:
        list(ex.map(comp, todo))
    if not os.path.exists(LIB_DEBUG) or any(os.path.getmtime(o) > os.path.getmtime(LIB_DEBUG) for o in objs):
        cmd = [_nvcc()] + ARCH + ["-shared", "-cudart", "shared", "-o", LIB_DEBUG] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    return LIB_DEBUG


if __name__ == "__main__":
    build(force="--force" in sys.argv, ptxas_verbose="-v" in sys.argv, verbose=True)
    print(LIB)
