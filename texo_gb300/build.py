"""Builds the engine's CUDA library in-tree for sm_103a (GB300).

Every translation unit under texo_gb300/csrc is compiled by nvcc in parallel
with `-gencode arch=compute_103a,code=sm_103a`, then linked into
texo_gb300/_build/libtexo_gp.so. Host code is compiled with
-ffp-contract=off so that the host arithmetic that must match the CPU
restatement bit for bit is never fused.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libtexo_gp.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
INCLUDE = os.path.join(os.path.dirname(HERE), "include")


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".cu", ".cpp")))


def headers():
    hs = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".cuh", ".h"))]
    return hs + [os.path.join(INCLUDE, "texo_gp.h")]


def _obj(src):
    return os.path.join(OUT, os.path.basename(src) + ".o")


def _compile(src, verbose=False, ptxas_v=False):
    cmd = [nvcc(), "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC,-ffp-contract=off",
           "-I", INCLUDE, "-c", src, "-o", _obj(src)]
    if src.endswith(".cpp"):
        cmd = [nvcc(), "-std=c++17", "-O3", "-x", "c++", "-Xcompiler", "-fPIC,-ffp-contract=off",
               "-I", INCLUDE, "-c", src, "-o", _obj(src)]
    if ptxas_v and src.endswith(".cu"):
        cmd.insert(1, "-Xptxas=-v")
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    return r.stderr


def needs_build():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(f) > t for f in sources() + headers())


def build(force=False, verbose=False, ptxas_v=False):
    if not force and not needs_build():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    srcs = sources()
    hdr_t = max(os.path.getmtime(h) for h in headers())
    todo = [s for s in srcs if force or ptxas_v or not os.path.exists(_obj(s))
            or os.path.getmtime(_obj(s)) < max(os.path.getmtime(s), hdr_t)]
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(todo), os.cpu_count() or 4))) as ex:
        logs = list(ex.map(lambda s: _compile(s, verbose, ptxas_v), todo))
    if ptxas_v:
        for s, log in zip(todo, logs):
            print("==", os.path.basename(s), "==\n" + log)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc(), "-shared", *ARCH, "-o", tmp] + [_obj(s) for s in srcs]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force=True, verbose=True, ptxas_v="-v" in sys.argv))
