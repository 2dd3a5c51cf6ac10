"""Build the oracle's C helpers (test infrastructure) with gcc.

``oracle/_build/liboracle.so`` holds the C restatement of the reference's
heap Dijkstra; it is compiled on whichever machine runs the tests or the CPU
baseline (x86 here, aarch64 on the GPU host) with the same flags.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "liboracle.so")
SRC = [os.path.join(HERE, "csrc", "heap_dijkstra.c")]


def build() -> str:
    os.makedirs(OUT, exist_ok=True)
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(s) for s in SRC):
        return LIB
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-o", LIB, *SRC, "-lm"]
    subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    print(build())
