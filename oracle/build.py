"""Build recipe for the parity oracle (TEST INFRASTRUCTURE ONLY).

Compiles oracle/texo_oracle.cpp, auction_oracle.cpp and routability_oracle.cpp into oracle/_build/libtexo_oracle.so with
g++ -O3 -ffp-contract=off (no fused multiply-add, matching Rust semantics).
The seeded synthetic-netlist generator of the engine (texo_gb300/csrc/synth.cpp,
plain host C++) is compiled in as well, so the benchmark's reference arm builds
its inputs without loading the engine library. Only the test suite, the smoke
check and the benchmark's CPU-baseline and reference legs load the result.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libtexo_oracle.so")
SRC = [os.path.join(HERE, "texo_oracle.cpp"), os.path.join(HERE, "auction_oracle.cpp"),
       os.path.join(HERE, "routability_oracle.cpp"),
       os.path.join(HERE, "..", "texo_gb300", "csrc", "synth.cpp")]
DEPS = SRC + [os.path.join(HERE, "texo_oracle.h"),
              os.path.join(HERE, "..", "include", "texo_gp.h")]


def needs_build():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(d) > t for d in DEPS)


def build(force=False, verbose=False):
    if not force and not needs_build():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
           "-pthread", "-Wall", "-Wno-unused-function", "-o", tmp] + SRC
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
