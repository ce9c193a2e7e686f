"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``oracle/mdft_oracle.c`` into ``oracle/_build/libmdft_oracle.so``
with OpenMP.  ``-ffp-contract=off`` keeps the oracle's rounding identical on
x86_64 and aarch64 hosts (GCC contracts a*b+c into FMA by default on Arm).

The Mini-MDFT reference itself cannot be compiled here: its hot path is
header-only C++ on top of Kokkos >= 4.4 and kokkos-fft >= 0.2.1 (FFTW/cuFFT),
none of which is present, so no ``oracle/_ref`` build exists.
"""
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "mdft_oracle.c")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libmdft_oracle.so")


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = [SRC, os.path.join(HERE, "mdft_oracle.h")]
    stamp = os.path.join(OUT_DIR, "HOST")
    if not (os.path.exists(stamp) and open(stamp).read().strip() == platform.machine()):
        force = True
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps)):
        return LIB
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-std=gnu11", "-o", LIB + ".tmp", SRC, "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    with open(stamp, "w") as f:
        f.write(platform.machine())
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
