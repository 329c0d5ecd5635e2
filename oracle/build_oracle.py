"""Builds the oracle's C core (oracle_core.c) into oracle/lib/liborc.so with gcc + OpenMP.

Test infrastructure only: the timed CPU baseline and a second checker."""
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "oracle_core.c"
LIB = HERE / "lib" / "liborc.so"


def build() -> Path:
    LIB.parent.mkdir(exist_ok=True)
    if LIB.exists() and LIB.stat().st_mtime > SRC.stat().st_mtime:
        return LIB
    cmd = ["gcc", "-O3", "-fopenmp", "-shared", "-fPIC", "-std=c11", "-o", str(LIB), str(SRC), "-lm"]
    subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    print(build())
