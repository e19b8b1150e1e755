"""Build recipe for the oracle library (test infrastructure only; see asph_oracle.h).

Compiles oracle/asph_oracle.c with gcc into oracle/libasph_oracle.so. Floating-point contraction is
disabled so that the FP32 variant performs exactly the operations written in the source.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "asph_oracle.c")
DEPS = [SRC, os.path.join(HERE, "oracle_body.h"), os.path.join(HERE, "refine_body.h"), os.path.join(HERE, "asph_oracle.h")]
LIB = os.path.join(HERE, "libasph_oracle.so")


def needs_build() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(d) > t for d in DEPS)


def build(force: bool = False) -> str:
    if force or needs_build():
        cmd = [
            os.environ.get("CC", "gcc"),
            "-O2",
            "-std=c11",
            "-fopenmp",
            "-ffp-contract=off",
            "-fno-fast-math",
            "-fPIC",
            "-shared",
            "-Wall",
            "-Wno-unused-function",
            "-o",
            LIB + ".tmp",
            SRC,
            "-lm",
        ]
        subprocess.run(cmd, check=True)
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
