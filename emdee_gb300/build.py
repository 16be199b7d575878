"""Builds the GB300 EmDee library in-tree: emdee_gb300/lib/libemdee.so.

Every translation unit is compiled for sm_103a only, in parallel.  The FP64
units (neighbor lists, FP64 forces, phase-space updates) and the host units are
compiled without FMA contraction so their FP64 arithmetic rounds like the
reference's statements.

    python -m emdee_gb300.build [--force]
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "lib", "libemdee.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
          "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]
# source -> extra flags
UNITS = {
    "api.cpp": [],
    "models.cpp": [],
    "neighbor.cu": ["-fmad=false"],
    "pair_fp64.cu": ["-fmad=false"],
    "motion.cu": ["-fmad=false"],
    "pair_mixed.cu": [],
    "bodies.cu": ["-fmad=false"],
    "ewald.cu": ["-fmad=false"],
    "verlet.cu": ["-fmad=false"],
    "replicas.cu": ["-fmad=false"],
    "bonded.cu": ["-fmad=false"],
    "surrogate.cu": [],
}
HEADERS = ["system.hpp", "pairmath.cuh", "tile.cuh", "f32x2.cuh", "ffkick.cuh", "fpconv.h", "reduce.cuh", "rigid.cuh", "bodies.cuh", os.path.join("..", "..", "include", "emdee.h")]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, flags, force):
    obj = os.path.join(OBJ, src + ".o")
    deps = [os.path.join(CSRC, src)] + [os.path.join(CSRC, h) for h in HEADERS]
    if not force and not _stale(obj, deps):
        return obj, None
    extra = os.environ.get("EMDEE_NVCC_FLAGS", "").split()   # tuning defines, e.g. -DPAIR_MIN_BLOCKS=6
    cmd = [NVCC] + ARCH + COMMON + flags + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
    if src.endswith(".cpp"):
        cmd = [NVCC] + COMMON + ["-x", "c++", "-c", os.path.join(CSRC, src), "-o", obj]
        cmd = [c for c in cmd if c not in ("-lineinfo", "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj, (r.stdout + r.stderr).strip() or None


def build(force=False, verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        futs = {ex.submit(_compile, s, f, force): s for s, f in UNITS.items()}
        objs = []
        for fu in cf.as_completed(futs):
            obj, log = fu.result()
            objs.append(obj)
            if log and verbose:
                print("[%s]\n%s" % (futs[fu], log))
    objs.sort()
    if force or _stale(LIB, objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-Xlinker", "-Bsymbolic"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s" % (r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
