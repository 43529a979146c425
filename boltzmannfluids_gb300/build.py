"""In-tree build of the sm_103a shared library libbfgb300.so.

Each .cu translation unit is compiled by nvcc in parallel (one per velocity
set, plus the auxiliary kernels and the C ABI) and linked into one shared
object next to this file.  No cmake, no torch extension machinery: the
library exports a plain C ABI (include/bf_lbm.h).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libbfgb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["lbm_q9.cu", "lbm_q15.cu", "lbm_q19.cu", "lbm_q27.cu", "lbm_aux.cu", "bf_abi.cu", "bf_noalloc.cu", "lbm_adjoint.cu",
           "marching_cubes.cu", "voxelize.cu", "render3d.cu"]


# the step kernels of each (velocity set, storage) pair: one generated
# translation unit each, so that the heaviest templates compile in parallel
STEP_UNITS = [(q, st) for q in (9, 15, 19, 27) for st in range(5)]


def _generated_units():
    gen = os.path.join(BUILD, "gen")
    os.makedirs(gen, exist_ok=True)
    out = []
    for q, st in STEP_UNITS:
        path = os.path.join(gen, f"step_q{q}_s{st}.cu")
        text = ("// generated by boltzmannfluids_gb300/build.py: step kernels of one velocity set and storage\n"
                f'#include "{os.path.join(CSRC, "lbm_kernels.cuh")}"\n'
                f"namespace bf {{\nBF_INSTANTIATE_STEP({q}, {st})\n}}\n")
        if not os.path.exists(path) or open(path).read() != text:
            with open(path, "w") as f:
                f.write(text)
        out.append(path)
    return out


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libbfgb300.so")


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(HERE, "..", "include", "bf_lbm.h"))
    return max(os.path.getmtime(f) for f in files)


def build(verbose=False, force=False):
    """Compiles every kernel for sm_103a and links libbfgb300.so; returns its path."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    # -ffp-contract=off for the host side: the launch constants must be the
    # same roundings as the oracle's on x86 and on Arm (where GCC would fuse)
    flags = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
             "-Xptxas", "-v" if verbose else "-O3",
             "--expt-relaxed-constexpr", *ARCH]
    # tuning: extra -D definitions (e.g. BF_STEP_BLOCK, BF_FAST_MIN_BLOCKS)
    flags += [f for f in os.environ.get("BF_NVCC_DEFINES", "").split() if f.startswith("-D")]

    def compile_one(src):
        path = src if os.path.isabs(src) else os.path.join(CSRC, src)
        obj = os.path.join(BUILD, os.path.splitext(os.path.basename(src))[0] + ".o")
        cmd = [nvcc(), *flags, "-c", path, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        return obj, r.stderr

    units = SOURCES + _generated_units()
    with cf.ThreadPoolExecutor(max_workers=min(len(units), max(4, (os.cpu_count() or 4)))) as ex:
        results = list(ex.map(compile_one, units))
    if verbose:
        for obj, err in results:
            print(obj)
            print(err)
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared", *ARCH, "-o", tmp, *[o for o, _ in results], "-lcudart"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
