"""Build recipe for the oracle shared library (test infrastructure only).

Compiles ``msod_oracle.c`` twice -- FP32 (the reference's rp=4) and FP64
(rp=8) -- into ``oracle/libmsod_oracle.so``.  ``-ffp-contract=off`` keeps
Fortran's separate multiply and add roundings on every host architecture, and
``-fopenmp`` enables the all-cores CPU baseline (the serial path is the
faithful single-core restatement).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libmsod_oracle.so")
SRC = os.path.join(HERE, "msod_oracle.c")

CFLAGS = ["-O3", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-std=gnu11", "-Wall"]


def build(force=False, verbose=False):
    """Compile the oracle if its library is missing or older than its source."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    bdir = os.path.join(HERE, "_build")
    os.makedirs(bdir, exist_ok=True)
    objs = []
    procs = []
    for real, sfx in (("float", "_f32"), ("double", "_f64")):
        obj = os.path.join(bdir, "msod_oracle%s.o" % sfx)
        cmd = ["gcc", *CFLAGS, "-DORC_REAL=%s" % real, "-DORC_SFX=%s" % sfx,
               "-DORC_IS_FLOAT=%d" % (real == "float"), "-c", SRC, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        procs.append(subprocess.Popen(cmd))
        objs.append(obj)
    for p in procs:
        if p.wait() != 0:
            raise RuntimeError("oracle compile failed")
    tmp = LIB + ".tmp"
    subprocess.check_call(["gcc", "-shared", "-fopenmp", "-o", tmp, *objs, "-lm"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
