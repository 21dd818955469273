"""Build libcylpic.so in-tree with nvcc for sm_103a.

The FP64 parity kernels (fields, FP64 push, particle boundaries) are
compiled with --fmad=false so every operation rounds once, as in the
reference build; host code is compiled with -ffp-contract=off for the same
reason (GCC contracts to FMA by default on aarch64).  The mixed-precision
push is compiled with contraction on.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcylpic.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
          "--expt-relaxed-constexpr"]

# Tile shapes of the mixed push (the order of TILE_SHAPES in push_mixed.cuh):
# push_mixed.cu is compiled once per shape.
TILE_SHAPES = ((16, 8), (8, 16), (8, 8), (16, 4), (8, 4))

# (source, extra flags, object name)
SOURCES = [
    ("capi.cu", ["--fmad=false"], "capi"),
    ("fields.cu", ["--fmad=false"], "fields"),
    ("push_fp64.cu", ["--fmad=false"], "push_fp64"),
    ("particles.cu", ["--fmad=false"], "particles"),
    ("charge.cu", ["--fmad=false"], "charge"),
    ("loader.cu", ["--fmad=false"], "loader"),
    ("ionise.cu", ["--fmad=false"], "ionise"),
] + [
    ("push_mixed.cu", ["--fmad=true", f"-DCYL_TILE_X={tx}", f"-DCYL_TILE_Y={ty}", f"-DCYL_TILE_NS=t{tx}x{ty}",
                       f"-DCYL_TILE_FNS=push_mixed_fns_{tx}x{ty}"], f"push_mixed_{tx}x{ty}")
    for tx, ty in TILE_SHAPES
] + [
    ("fields_fp32.cu", ["--fmad=true"], "fields_fp32"),
    ("mixed_particles.cu", ["--fmad=true"], "mixed_particles"),
    ("host_deck.cpp", [], "host_deck"),
    ("server.cpp", [], "server"),
    ("sdf_io.cpp", [], "sdf_io"),
]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src, extra, name, verbose):
    obj = os.path.join(OUT_DIR, name + ".o")
    path = os.path.join(CSRC, src)
    if src.endswith(".cpp"):
        cmd = [nvcc(), "-x", "c++", "-O2", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-pthread",
               "-c", path, "-o", obj]
    else:
        cmd = [nvcc()] + ARCH + COMMON + extra + ["-c", path, "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, "..", "include", "cylpic.h"))
    deps.append(os.path.join(HERE, "..", "include", "cyl_math.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force=False, verbose=False):
    """Compile every CUDA/C++ source and link libcylpic.so; returns its path."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda a: _compile(a[0], a[1], a[2], verbose), SOURCES))
    objs = [o for o, _ in results]
    if verbose:
        for (_, _, name), (_, log) in zip(SOURCES, results):
            sys.stderr.write(f"== {name}\n{log}")
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart", "-Xcompiler", "-pthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
