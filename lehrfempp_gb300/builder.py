"""Build the GB300 library in-tree: lehrfempp_gb300/_build/liblfg.so.

Each CUDA / C++ translation unit under csrc/ is compiled by nvcc for sm_103a
only (-gencode arch=compute_103a,code=sm_103a), in parallel, and linked into
one shared library with the C-ABI of include/lfg.h.  Incremental: a unit is
recompiled when it or any header under csrc/ or include/ is newer than its
object file.
"""
import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liblfg.so")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include"),
          "--expt-relaxed-constexpr"]


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cc")))


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.inc")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h"))


def _obj(src):
    return os.path.join(OUT_DIR, os.path.basename(src) + ".o")


def _compile(src, verbose):
    cmd = [NVCC] + ARCH + COMMON + ["-c", src, "-o", _obj(src)]
    if src.endswith(".cc"):
        cmd = [NVCC] + COMMON + ["-x", "c++", "-c", src, "-o", _obj(src)]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return r.stderr


def build(force=False, verbose=False, jobs=None):
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = _sources()
    hdr_time = max(os.path.getmtime(h) for h in _headers())
    todo = []
    for s in srcs:
        o = _obj(s)
        if force or not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), hdr_time):
            todo.append(s)
    logs = {}
    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            futs = {ex.submit(_compile, s, verbose): s for s in todo}
            for f in cf.as_completed(futs):
                logs[futs[f]] = f.result()
    objs = [_obj(s) for s in srcs]
    if todo or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s" % r.stderr)
    if verbose:
        for s, l in sorted(logs.items()):
            sys.stderr.write("== %s\n%s" % (os.path.basename(s), l))
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
