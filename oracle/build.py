"""Build recipe for the oracle's C restatement (test infrastructure only).

    python oracle/build.py      ->  oracle/_build/libkmc_oracle.so

``-ffp-contract=off`` keeps every a*b+c as two rounded operations, as in the
reference's Python/numpy arithmetic (gcc fuses them by default on aarch64).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build", "libkmc_oracle.so")


def build(force=False):
    src = os.path.join(HERE, "kmc_oracle.c")
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= os.path.getmtime(src):
        return OUT
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    tmp = OUT + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-shared", "-fPIC",
           "-o", tmp, src, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
