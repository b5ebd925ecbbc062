"""Build recipe for the CPU oracle (test infrastructure, not the product).

Compiles oracle/ss_oracle.cpp into oracle/_build/libss_oracle.so with g++
(OpenMP over particles).  Portable flags only: the same recipe runs on the
x86_64 development host and on the aarch64 GPU host.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "ss_oracle.cpp")
OUT_DIR = os.path.join(HERE, "_build")
OUT = os.path.join(OUT_DIR, "libss_oracle.so")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    hdr = os.path.join(HERE, "..", "include", "streamsculptor_gb300.h")
    if (not force and os.path.exists(OUT)
            and os.path.getmtime(OUT) >= max(os.path.getmtime(SRC), os.path.getmtime(hdr))):
        return OUT
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared",
           "-ffp-contract=off", "-o", OUT + ".tmp", SRC]
    subprocess.check_call(cmd)
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
