"""Build recipe of libnfft3_gb300.so (nvcc, sm_103a only, in-tree).

Every translation unit is compiled in parallel with
``-gencode arch=compute_103a,code=sm_103a`` and linked with cuFFT into
``nfft_gb300/libnfft3_gb300.so``.  Objects go to ``nfft_gb300/_build/``.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libnfft3_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=default",
          "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith(".cu") or f.endswith(".cpp"))


def _obj(src):
    return os.path.join(BUILD, os.path.basename(src) + ".o")


def _deps_mtime():
    return max(os.path.getmtime(os.path.join(CSRC, f)) for f in os.listdir(CSRC)
               if f.endswith((".cuh", ".h"))) if os.path.isdir(CSRC) else 0.0


def _compile(src, extra):
    out = _obj(src)
    cmd = [NVCC] + ARCH + COMMON + extra + ["-c", src, "-o", out]
    if src.endswith(".cpp"):
        cmd = [NVCC] + COMMON + extra + ["-x", "c++", "-c", src, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return out, r.stderr


def build(force=False, verbose=False, ptxas_v=False, jobs=None):
    """Compile and link; returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    inc = os.path.join(ROOT, "include")
    hdr = max([_deps_mtime()] + [os.path.getmtime(os.path.join(inc, f)) for f in os.listdir(inc)])
    extra = ["-Xptxas", "-v"] if ptxas_v else []
    todo = [s for s in srcs if force or ptxas_v or not os.path.exists(_obj(s))
            or os.path.getmtime(_obj(s)) < max(os.path.getmtime(s), hdr)]
    logs = []
    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            for out, err in ex.map(lambda s: _compile(s, extra), todo):
                logs.append(err)
    objs = [_obj(s) for s in srcs]
    if todo or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        tmp = LIB + ".tmp"
        cmd = [NVCC] + ARCH + ["-shared", "-Xlinker", "-Bsymbolic", "-o", tmp] + objs + ["-lcufft", "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s" % (r.stdout, r.stderr))
        os.replace(tmp, LIB)
    if verbose:
        for l in logs:
            if l.strip():
                sys.stderr.write(l)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_v="--ptxas-v" in sys.argv)
    print(LIB)
