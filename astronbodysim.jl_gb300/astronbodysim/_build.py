"""Build recipe of libnbody_gb300.so (sm_103a), run in place.

Each .cu under csrc/ compiles to an object in parallel with one -gencode
(compute_103a / sm_103a), then the objects link into a shared library next to
the sources.  Files named in FP64_STRICT build with -fmad=false so FP64
products and sums round separately, as the reference's Julia expressions do.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(ROOT, "csrc")
REPO = os.path.dirname(ROOT)
INCLUDE = os.path.join(REPO, "include")
BUILD = os.path.join(CSRC, "_build")
LIB = os.path.join(CSRC, "libnbody_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC]
FP64_STRICT = {"nb_force_fp64.cu", "nb_integrate.cu"}


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(force=False, verbose=False, ptxas_v=False):
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    jobs = []
    objs = []
    for f in sources():
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f[:-3] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            flags = list(COMMON) + ARCH
            if f in FP64_STRICT:
                flags += ["-fmad=false"]
            # extra -D tuning definitions (launch-shape experiments)
            flags += os.environ.get("NBODY_GB300_NVCC_DEFS", "").split()
            if ptxas_v:
                flags += ["-Xptxas", "-v"]
            jobs.append([nvcc] + flags + ["-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
        for cmd, r in zip(jobs, results):
            if verbose or ptxas_v:
                print(r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError("nvcc failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        cmd = [nvcc, "-shared"] + ARCH + ["-o", tmp] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build_library(force="--force" in sys.argv, verbose=True, ptxas_v="-v" in sys.argv))
