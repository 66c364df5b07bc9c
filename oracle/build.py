"""Builds the C oracle (oracle/pt_oracle.c + pt_oracle_bh.inc) into oracle/_build/liboracle.so.

Test infrastructure only. The flags matter: -ffp-contract=off keeps every f32
multiply and add separately rounded, as Rust evaluates them (rustc never
contracts a*b+c into an FMA); -fno-fast-math keeps IEEE semantics; OpenMP gives
the multi-threaded restatement of particular's rayon methods that the CPU
baseline times.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SRC = os.path.join(HERE, "pt_oracle.c")
DEPS = [SRC, os.path.join(HERE, "pt_oracle_bh.inc")]

CFLAGS = ["-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
          "-fopenmp", "-Wall", "-Wno-unknown-pragmas"]


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in DEPS)):
        return LIB
    cc = os.environ.get("CC", "gcc")
    tmp = LIB + ".tmp"
    subprocess.check_call([cc, *CFLAGS, SRC, "-o", tmp, "-lm"])
    os.replace(tmp, LIB)
    return LIB


CEILING_SRC = os.path.join(HERE, "learned_ceiling.c")
CEILING_BIN = os.path.join(OUT_DIR, "learned_ceiling")


def build_ceiling(force=False):
    """The FP64 model of the group walk that bounds learned corrections
    (learned_ceiling.c; a program, not part of the library)."""
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(CEILING_BIN) and os.path.getmtime(CEILING_BIN) >= os.path.getmtime(CEILING_SRC):
        return CEILING_BIN
    cc = os.environ.get("CC", "gcc")
    tmp = CEILING_BIN + ".tmp"
    subprocess.check_call([cc, "-O3", "-std=c11", "-fopenmp", "-Wall", "-Wno-unknown-pragmas", CEILING_SRC,
                           "-o", tmp, "-lm"])
    os.replace(tmp, CEILING_BIN)
    return CEILING_BIN


if __name__ == "__main__":
    build_ceiling(force=True)
    print(build(force=True))
