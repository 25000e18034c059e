"""Builds oracle/liboracle_contract.so (the float64 CPU contractor used only
as the tests' oracle and the benchmark's CPU baseline).  gcc + OpenMP."""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "contract_oracle.c")
LIB = os.path.join(HERE, "liboracle_contract.so")


def build():
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["gcc", "-O3", "-fopenmp", "-shared", "-fPIC", "-std=c99", SRC, "-o", LIB + ".tmp", "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build())
    sys.exit(0)
