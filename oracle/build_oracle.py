"""Build recipe for the oracle's C helpers (test infrastructure and the
benchmark's CPU baseline only): oracle/_build/libcsr_bicgstab.so, an OpenMP
complex128 CSR SpMV + BiCGSTAB.  Portable flags only (the same source builds
on x86-64 and aarch64 hosts)."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build", "libcsr_bicgstab.so")


def build():
    src = os.path.join(HERE, "csr_bicgstab.c")
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    if os.path.exists(OUT) and os.path.getmtime(OUT) > max(os.path.getmtime(src), os.path.getmtime(__file__)):
        return OUT
    subprocess.run(["gcc", "-O3", "-fopenmp", "-shared", "-fPIC", "-std=c11", src, "-o", OUT, "-lm"], check=True)
    return OUT


if __name__ == "__main__":
    print(build())
