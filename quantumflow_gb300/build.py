"""Build the CUDA C-ABI library ``quantumflow_gb300/_lib/libqfgb300.so``.

Every translation unit in ``csrc/`` is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``) in parallel, then linked into
one shared library.  Nothing is installed: the library stays in the source
tree next to the Python package that loads it.

Usage:  python quantumflow_gb300/build.py [--force] [-v]
(run as a script: importing the package itself loads the library, so the
build must not depend on that import.)
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIBDIR = os.path.join(HERE, "_lib")
LIBNAME = "libqfgb300.so"
LIBPATH = os.path.join(LIBDIR, LIBNAME)
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc():
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    path = os.path.join(cuda, "bin", "nvcc")
    if os.path.exists(path):
        return path
    found = shutil.which("nvcc")
    if not found:
        raise RuntimeError("nvcc not found: set CUDA_HOME")
    return found


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _flags():
    return [ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
            "-I" + INCLUDE, "-I" + CSRC, "--expt-relaxed-constexpr"]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, obj, verbose):
    cmd = [_nvcc(), *_flags(), "-c", src, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stderr}")
    return r.stderr


def build(force=False, verbose=False, jobs=None):
    """Compile csrc/*.cu and link the shared library; returns its path."""
    os.makedirs(LIBDIR, exist_ok=True)
    objdir = os.path.join(LIBDIR, "obj")
    os.makedirs(objdir, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    srcs = sources()
    objs = [os.path.join(objdir, os.path.basename(s)[:-3] + ".o") for s in srcs]
    todo = [(s, o) for s, o in zip(srcs, objs) if force or _stale(o, [s, *headers])]
    logs = []
    if todo:
        n = jobs or min(len(todo), os.cpu_count() or 4)
        with concurrent.futures.ThreadPoolExecutor(max_workers=n) as ex:
            futs = [ex.submit(_compile, s, o, verbose) for s, o in todo]
            for f in futs:
                logs.append(f.result())
    if force or todo or _stale(LIBPATH, objs):
        tmp = LIBPATH + ".tmp"
        cmd = [_nvcc(), ARCH, "-shared", "-o", tmp, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
        os.replace(tmp, LIBPATH)
    if verbose:
        for log in logs:
            sys.stderr.write(log)
    return LIBPATH


if __name__ == "__main__":
    p = build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(p)
