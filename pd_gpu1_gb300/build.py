"""Build libpd_gb300.so in-tree with nvcc for sm_103a (GB300).

Each translation unit compiles in parallel; the setup and neighbour files are
built without FMA contraction so that their arithmetic rounds like the
reference's host code (bit-exact bond families and crack flags).
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpd_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
          "-I", CSRC, "--expt-relaxed-constexpr"]
UNITS = {
    "neighbor.cu": ["-fmad=false"],
    "setup.cu": ["-fmad=false"],
    "force.cu": [],
    "integrate.cu": [],
    "api.cu": [],
    "noalloc.cu": [],
    "batch.cu": [],
    "output.cu": [],
    "mlp.cu": [],
}


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.exists(cand) or cand == "nvcc"):
            return cand
    return "nvcc"


def _compile(unit, extra, verbose):
    src = os.path.join(CSRC, unit)
    obj = os.path.join(OUT_DIR, unit.replace(".cu", ".o"))
    cmd = [nvcc(), "-c", src, "-o", obj] + ARCH + COMMON + extra
    if verbose:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    srcs = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "pd.h"), __file__]
    return any(os.path.getmtime(s) > t for s in srcs)


def build(force=False, verbose=False):
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        futs = {ex.submit(_compile, u, e, verbose): u for u, e in UNITS.items()}
        objs = []
        for f in cf.as_completed(futs):
            obj, log = f.result()
            objs.append(obj)
            if verbose and log:
                sys.stderr.write(log)
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared", "-o", tmp] + ARCH + sorted(objs) + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
