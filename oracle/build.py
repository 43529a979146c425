"""Builds the CPU oracle (test infrastructure only) into oracle/_build/.

liboracle.so holds two compilations of lbm_oracle.c: REAL=float (orc32_*,
the ref-literal FP32 stepper) and REAL=double (orc64_*, the FP64 oracle).
FMA contraction is switched off so the operation order is the GLSL's.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(HERE, "lbm_oracle.c")
    adj = os.path.join(HERE, "adjoint_oracle.c")
    so = os.path.join(OUT, "liboracle.so")
    if os.path.exists(so) and os.path.getmtime(so) > max(os.path.getmtime(src), os.path.getmtime(adj)):
        return so
    flags = ["-O2", "-std=c11", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-fopenmp"]
    objs = []
    for tag, defs in (("32", ["-DREAL=float", "-DORC(n)=orc32_##n"]), ("64", ["-DREAL=double", "-DORC(n)=orc64_##n"])):
        obj = os.path.join(OUT, f"oracle{tag}.o")
        cmd = ["gcc", *flags, *defs, "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        subprocess.check_call(cmd)
        objs.append(obj)
    obj = os.path.join(OUT, "adjoint64.o")
    subprocess.check_call(["gcc", *flags, "-c", adj, "-o", obj])
    objs.append(obj)
    tmp = so + ".tmp"
    subprocess.check_call(["gcc", "-shared", "-fopenmp", "-o", tmp, *objs, "-lm"])
    os.replace(tmp, so)
    return so


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
