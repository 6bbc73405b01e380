"""In-tree build of libmandoct_gb300.so for sm_103a with nvcc (no cmake, no torch
extension machinery): each .cu under csrc/ compiles to an object in parallel, then
one shared library is linked next to this file.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB_NAME = "libmandoct_gb300.so"
LIB_PATH = os.path.join(HERE, LIB_NAME)
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path():
    p = shutil.which("nvcc")
    if p:
        return p
    for c in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _compile(nvcc, src, extra):
    obj = os.path.join(OBJ, os.path.basename(src)[:-3] + ".o")
    cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include"),
           *extra, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    return obj, r.returncode, r.stdout + r.stderr, " ".join(cmd)


def build(verbose=False, extra=(), force=False):
    """Compile every CUDA source and link the shared library; returns its path."""
    nvcc = nvcc_path()
    os.makedirs(OBJ, exist_ok=True)
    srcs = sources()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    newest = max([os.path.getmtime(s) for s in srcs + headers] +
                 [os.path.getmtime(os.path.join(ROOT, "include", "mandoct_gb300.h"))])
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= newest and not extra:
        return LIB_PATH
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(nvcc, s, list(extra)), srcs))
    failed = [r for r in results if r[1] != 0]
    for obj, rc, out, cmd in results:
        if verbose or rc != 0:
            sys.stderr.write(f"$ {cmd}\n{out}")
    if failed:
        raise RuntimeError(f"nvcc failed for {[os.path.basename(f[0]) for f in failed]}")
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-cudart", "shared", "-o", tmp, *[r[0] for r in results]]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else (),
                force="--force" in sys.argv))
