"""Build the in-tree shared library ouranos_gb300/_lib/libouranos_gb300.so.

nvcc compiles every translation unit of ouranos_gb300/csrc for sm_103a only
(-gencode arch=compute_103a,code=sm_103a), in parallel, and links them into
one library exporting the C-ABI of include/ouranos_gb300.h.
"""
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libouranos_gb300.so")
ROOT = os.path.dirname(HERE)
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["quadrature.cpp", "fe.cpp", "operator.cu", "solvers.cu", "vec.cu",
           "sweep_f64.cu", "sweep_f32.cu", "sweep_df64.cu", "sweep_wide_f64.cu", "sweep_wide_f32.cu",
           "sweep_wide_df64.cu", "sweep_batch_f64.cu", "sweep_batch_f32.cu",
           "batch.cu", "noalloc.cu", "cnn.cu", "precond.cu", "dsa.cu", "contract_tc.cu", "contract_oz.cu", "cnn_tc.cu"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _digest():
    h = hashlib.sha256()
    for name in sorted(os.listdir(CSRC)) + ["../../include/ouranos_gb300.h", "../build.py"]:
        path = os.path.join(CSRC, name)
        if os.path.isfile(path):
            with open(path, "rb") as f:
                h.update(name.encode() + f.read())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def build(force=False, verbose=False, jobs=None):
    os.makedirs(OUT, exist_ok=True)
    stamp = os.path.join(OUT, "build.stamp")
    dig = _digest()
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as f:
            if f.read().strip() == dig:
                return LIB
    nvcc = _nvcc()
    objdir = os.path.join(OUT, "obj")
    os.makedirs(objdir, exist_ok=True)
    common = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include")]

    def compile_one(src):
        obj = os.path.join(objdir, src + ".o")
        cmd = [nvcc] + GENCODE + common + ["-x", "cu", "-c", os.path.join(CSRC, src), "-o", obj]
        if src.endswith(".cu"):
            cmd += ["-Xptxas", "-warn-spills"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
        if verbose and (r.stdout.strip() or r.stderr.strip()):
            print(r.stdout + r.stderr, flush=True)
        return obj

    jobs = jobs or min(len(SOURCES), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc] + GENCODE + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(dig)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
