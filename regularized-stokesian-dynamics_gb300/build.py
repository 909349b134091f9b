"""In-tree build of the CUDA library librsd_gb300.so (sm_103a only).

    python regularized-stokesian-dynamics_gb300/build.py [--force]

Each translation unit in csrc/ is compiled by its own nvcc process (in
parallel), then linked with -shared.  The generated headers ewald_gen.cuh and
overlap_gen.cuh are committed; each is regenerated from its generator
(gen_ewald.py, gen_overlap.py) only when sympy is importable and the
generator is newer than the header.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "librsd_gb300.so")
SOURCES = ["ewald.cu", "lub.cu", "dense.cu", "capi.cu", "step.cu", "mixed.cu", "noalloc.cu", "tc_gemm.cu", "learned.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.exists(cand) or cand == "nvcc"):
            return cand
    return "nvcc"


GENERATED = [("gen_ewald.py", "ewald_gen.cuh"), ("gen_overlap.py", "overlap_gen.cuh")]


def _maybe_regenerate():
    for gen_name, hdr_name in GENERATED:
        gen = os.path.join(CSRC, gen_name)
        hdr = os.path.join(CSRC, hdr_name)
        deps = [gen] + ([os.path.join(CSRC, "gen_ewald.py")] if gen_name != "gen_ewald.py" else [])
        if os.path.exists(hdr) and os.path.getmtime(hdr) >= max(os.path.getmtime(d) for d in deps):
            continue
        try:
            import sympy  # noqa: F401
        except ImportError:
            if not os.path.exists(hdr):
                raise RuntimeError("%s is missing and sympy is not available to generate it" % hdr_name)
            continue
        subprocess.check_call([sys.executable, gen])


def _deps_mtime():
    m = 0.0
    for f in os.listdir(CSRC):
        if f.endswith((".cu", ".cuh", ".h")):
            m = max(m, os.path.getmtime(os.path.join(CSRC, f)))
    hdr = os.path.join(os.path.dirname(HERE), "include", "rsd_capi.h")
    return max(m, os.path.getmtime(hdr))


def build(force=False, verbose=False):
    _maybe_regenerate()
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps_mtime():
        return LIB
    os.makedirs(BUILD, exist_ok=True)

    def compile_one(src):
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        cmd = [nvcc()] + ARCH + FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed on %s:\n%s\n%s" % (src, r.stdout, r.stderr))
        if verbose:
            sys.stderr.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
