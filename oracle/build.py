"""Build recipe of the CPU oracle (test infrastructure): compiles oracle.c and gen.c
into oracle/_build/liboracle.so with gcc.  Floating-point contraction is disabled so
Float32 arithmetic rounds once per operation, as Julia does."""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build", "liboracle.so")
SRCS = [os.path.join(HERE, "oracle.c"), os.path.join(HERE, "gen.c")]
FLAGS = ["-O2", "-fPIC", "-shared", "-std=gnu11", "-ffp-contract=off", "-fno-fast-math"]


def build(force: bool = False) -> str:
    if not force and os.path.exists(OUT):
        newest = max(os.path.getmtime(s) for s in SRCS)
        if os.path.getmtime(OUT) >= newest:
            return OUT
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    cc = os.environ.get("CC", "gcc")
    tmp = OUT + ".tmp%d" % os.getpid()
    cmd = [cc] + FLAGS + ["-fopenmp", "-o", tmp] + SRCS + ["-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:  # a toolchain without OpenMP still builds the serial oracle
        cmd = [cc] + FLAGS + ["-o", tmp] + SRCS + ["-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stderr)
            raise RuntimeError("oracle build failed: " + " ".join(cmd))
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
