"""Build recipe for libblis_gb300.so (sm_103a only).

Every CUDA translation unit under csrc/ is compiled with
`nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo` in parallel,
then linked into blis_gb300/libblis_gb300.so against the shared CUDA
runtime.  The library is loaded in-tree by blis_gb300/_lib.py.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libblis_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def headers():
    inc = os.path.join(os.path.dirname(HERE), "include")
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(inc, f) for f in os.listdir(inc) if f.endswith(".h")]
    return hs


def _compile(src, verbose_ptxas=False):
    obj = os.path.join(OBJ, os.path.basename(src) + ".o")
    dep_time = max(os.path.getmtime(h) for h in headers() + [src])
    if os.path.exists(obj) and os.path.getmtime(obj) >= dep_time and not verbose_ptxas:
        return obj, ""
    cmd = [nvcc()] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                             "-Xcompiler", "-fvisibility=default", "-c", src, "-o", obj]
    if verbose_ptxas:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return obj, r.stderr


def build(force=False, verbose_ptxas=False, jobs=None):
    os.makedirs(OBJ, exist_ok=True)
    if force:
        for f in os.listdir(OBJ):
            os.remove(os.path.join(OBJ, f))
    srcs = sources()
    jobs = jobs or min(len(srcs), max(2, os.cpu_count() or 2))
    with cf.ThreadPoolExecutor(jobs) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose_ptxas), srcs))
    objs = [o for o, _ in results]
    log = "".join(l for _, l in results)
    newest = max(os.path.getmtime(o) for o in objs)
    if force or verbose_ptxas or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "shared", "-o", tmp] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
        os.replace(tmp, LIB)
    return LIB, log


if __name__ == "__main__":
    import sys
    lib, log = build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv)
    print(log)
    print(lib)
