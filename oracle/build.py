"""Build recipe for the CPU oracle (test infrastructure only).

Compiles topo_oracle.c with gcc + OpenMP into oracle/_build/libtopo_oracle.so.
Portable C11: no x86 intrinsics, no -march=native, so it builds identically
on the x86 development container and on the aarch64 GPU host.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libtopo_oracle.so")


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "topo_oracle.c")
    hdr = os.path.join(HERE, "topo_oracle.h")
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-fopenmp", "-fno-fast-math",
           "-ffp-contract=off", src, "-o", tmp, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
