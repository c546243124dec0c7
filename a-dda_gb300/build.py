"""Build recipe for libadda_gb300.so: hand-written CUDA kernels for sm_103a plus the C host code, one shared library.

Usage: python a-dda_gb300/build.py [--force]. Translation units compile in parallel; the result lands in
a-dda_gb300/_build/libadda_gb300.so (git-ignored). The CUDA runtime is linked statically, so the library needs only
the driver at run time.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libadda_gb300.so")
INCLUDE = os.path.join(ROOT, "include")

CU = ["api.cu", "matvec.cu", "matvec_f32.cu", "matvec_yz.cu", "dmatrix.cu", "solver.cu", "noalloc.cu"]
C = ["host_setup.c", "integrate.c"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return [os.path.join(CSRC, f) for f in CU + C] + [os.path.join(CSRC, f) for f in os.listdir(CSRC)
                                                       if f.endswith((".cuh", ".h"))] + \
        [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(force=False, verbose=False, out=None, defines=()):
    """compile the library into out (default a-dda_gb300/_build); defines: extra -D macros (a variant build, e.g. the
    scalar-sum reference build ADDA_NO_F32X2 of the tests)"""
    out_dir = out or OUT
    lib_path = os.path.join(out_dir, "libadda_gb300.so")
    os.makedirs(out_dir, exist_ok=True)
    if not force and not _stale(lib_path, _sources()):
        return lib_path
    nv = nvcc()
    jobs = []
    objs = []
    for f in CU:
        o = os.path.join(out_dir, f + ".o")
        objs.append(o)
        jobs.append([nv, "-c", os.path.join(CSRC, f), "-o", o, "-std=c++17", "-O3", "-lineinfo", *ARCH,
                     "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC, "--expt-relaxed-constexpr",
                     *["-D" + d for d in defines], "-Xptxas", "-v" if verbose else "-O3"])
    for f in C:
        o = os.path.join(out_dir, f + ".o")
        objs.append(o)
        jobs.append(["gcc", "-c", os.path.join(CSRC, f), "-o", o, "-O2", "-fPIC", "-std=gnu11", "-I", INCLUDE])
    logs = []
    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        for out in ex.map(_run, jobs):
            logs.append(out)
    _run([nv, "-shared", *ARCH, "-o", lib_path + ".tmp", *objs, "-lm"])
    os.replace(lib_path + ".tmp", lib_path)
    if verbose:
        print("\n".join(logs))
    return lib_path


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
