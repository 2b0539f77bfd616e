"""ORACLE (test infrastructure only): compile the C restatements with gcc.

Output: oracle/_build/liboracle.so.  -ffp-contract=off keeps the host compiler
from fusing multiply-adds (gcc fuses by default on aarch64), so x86 and Arm
builds round identically.
"""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = [HERE / "march.c"]
OUT = HERE / "_build" / "liboracle.so"


def build() -> Path:
    OUT.parent.mkdir(exist_ok=True)
    if OUT.exists() and all(OUT.stat().st_mtime >= s.stat().st_mtime for s in SRC):
        return OUT
    cmd = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           *map(str, SRC), "-o", str(OUT), "-lm"]
    subprocess.run(cmd, check=True)
    return OUT


if __name__ == "__main__":
    print(build())
