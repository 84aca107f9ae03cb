"""Build libmatgb_f32.so and libmatgb_f64.so in-tree with nvcc for sm_103a.

Every translation unit under csrc/ is compiled twice (float, and
-DMAT_DOUBLE_PRECISION for double), in parallel, then linked with the static
CUDA runtime into libmat_gb300/lib/.  Objects live in libmat_gb300/_build/.
Usage: python -m libmat_gb300.build   (or build() from Python)
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "lib")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
          "-I", os.path.join(ROOT, "include"), "-I", CSRC]
PRECS = {"f32": [], "f64": ["-DMAT_DOUBLE_PRECISION"]}


def _nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _compile(args):
    src, prec, out, extra = args
    cmd = [_nvcc()] + ARCH + COMMON + PRECS[prec] + extra + \
        ["-c", os.path.join(CSRC, src), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src} ({prec}):\n{r.stderr}")
    return r.stderr


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(jobs=None, verbose=False, extra=()):
    """Compile and link both precisions; returns the two library paths."""
    os.makedirs(LIB, exist_ok=True)
    headers = [os.path.join(ROOT, "include", h)
               for h in os.listdir(os.path.join(ROOT, "include"))]
    headers += [os.path.join(CSRC, h) for h in os.listdir(CSRC)
                if h.endswith((".cuh", ".h"))]
    work, objs = [], {p: [] for p in PRECS}
    for prec in PRECS:
        os.makedirs(os.path.join(OBJ, prec), exist_ok=True)
        for s in sources():
            out = os.path.join(OBJ, prec, s + ".o")
            objs[prec].append(out)
            if _stale(out, [os.path.join(CSRC, s), __file__] + headers):
                work.append((s, prec, out, list(extra)))
    jobs = jobs or min(len(work) or 1, os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        for msg in ex.map(_compile, work):
            if verbose and msg:
                print(msg, file=sys.stderr)
    libs = []
    for prec in PRECS:
        lib = os.path.join(LIB, f"libmatgb_{prec}.so")
        if _stale(lib, objs[prec]):
            cmd = [_nvcc()] + ARCH + ["-shared", "-o", lib] + objs[prec] + ["-ldl"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"link failed ({prec}):\n{r.stderr}")
        libs.append(lib)
    return libs


if __name__ == "__main__":
    for p in build(verbose="-v" in sys.argv):
        print(p)
