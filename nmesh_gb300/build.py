"""Build the native library nmesh_gb300/_build/libnmg.so in-tree with nvcc
for sm_103a (GB300).  Host C++ is compiled with -ffp-contract=off so that
the mesh geometry is bitwise identical on x86-64 and aarch64 hosts."""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libnmg.so")
SOURCES = ["nmg.cu", "stage_eo.cu", "stage_tc.cu", "stage_gather.cu", "stage_fv.cu", "stage_fv_fast.cu",
           "grhd.cu", "grhd_evolve.cu", "noalloc.cu", "mesh.cpp", "ckpt.cpp"]
# per-file extra flags: the finite-volume kernel rounds every product and sum
# separately, in the reference's order (no FMA contraction)
EXTRA_FLAGS = {"stage_fv.cu": ["-fmad=false"], "grhd.cu": ["-fmad=false"]}
HEADERS = ["mesh.h", "stage.cuh", "ctx.h", "weno.cuh", "grhd.cuh", "tc_build.h", "tc_device.cuh",os.path.join("..", "..", "include", "nmg.h")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                     "-Xcompiler", "-fPIC,-ffp-contract=off", "-Xptxas", "-v"]


def _nvcc():
    for cand in ("nvcc", "/usr/local/cuda/bin/nvcc"):
        try:
            subprocess.run([cand, "--version"], check=True, capture_output=True)
            return cand
        except (OSError, subprocess.CalledProcessError):
            continue
    raise RuntimeError("nvcc not found")


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, s) for s in SOURCES + HEADERS] + [__file__]
    return any(os.path.getmtime(p) > t for p in deps)


def build(force=False, verbose=False):
    """Compile (if stale) and return the path of libnmg.so."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        cmd = [nvcc] + NVCC_FLAGS + EXTRA_FLAGS.get(src, []) + \
            ["-c", os.path.join(CSRC, src), "-o", obj]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{res.stderr}")
        log = os.path.join(BUILD, src + ".ptxas.txt")
        with open(log, "w") as fp:
            fp.write(res.stderr)
        if verbose:
            sys.stdout.write(res.stderr)
        return obj

    with ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    subprocess.run(cmd, check=True, capture_output=not verbose)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
