"""Build the CPU oracle shared libraries (test infrastructure, not the product).

Two builds of oracle/xnb_oracle.cpp:
  * liboracle_parity.so  -- -O2 -ffp-contract=off, no OpenMP: the bit-exact checker;
  * liboracle_omp.so     -- -O3 -fopenmp -ffp-contract=off: the timed CPU baseline
    (OpenMP over cells as in the reference; contraction stays off so both builds
    give identical numbers).

Both land in oracle/_build/ (git-ignored). Usable on x86_64 and aarch64 hosts.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(HERE, "xnb_oracle.cpp")
    jobs = [
        ("liboracle_parity.so", ["-O2", "-ffp-contract=off"]),
        ("liboracle_omp.so", ["-O3", "-fopenmp", "-ffp-contract=off"]),
    ]
    procs = []
    for name, flags in jobs:
        dst = os.path.join(OUT, name)
        if os.path.exists(dst) and os.path.getmtime(dst) >= max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "xnb_oracle.h")),
            os.path.getmtime(os.path.join(HERE, "xnb_snap_oracle.h"))
        ):
            continue
        cmd = ["g++", "-std=c++17", "-shared", "-fPIC", *flags, src, "-o", dst + ".tmp"]
        if verbose:
            print(" ".join(cmd))
        procs.append((subprocess.Popen(cmd), dst))
    for p, dst in procs:
        if p.wait() != 0:
            raise RuntimeError("oracle build failed: %s" % dst)
        os.replace(dst + ".tmp", dst)
    return OUT


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
