"""Build recipe of the CPU oracle (test infrastructure only).

Compiles ``oracle/rz_oracle.cpp`` -- the C++ restatement of rusterize's burn
path -- into ``oracle/_build/librz_oracle.so`` with IEEE-exact flags
(``-O2 -ffp-contract=off``, no fast-math).  The reference itself is Rust and
cannot be compiled here (no cargo/rustc), so there is no ``oracle/_ref``.
"""

from __future__ import annotations

import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "rz_oracle.cpp"
OUT = HERE / "_build" / "librz_oracle.so"
FLAGS = ["-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared"]


def build(force: bool = False) -> Path:
    if not force and OUT.exists() and OUT.stat().st_mtime >= SRC.stat().st_mtime:
        return OUT
    OUT.parent.mkdir(parents=True, exist_ok=True)
    cmd = ["g++", *FLAGS, str(SRC), "-o", str(OUT)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + res.stdout + res.stderr)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
