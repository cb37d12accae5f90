"""Builds libfastbarnes_gb300.so (sm_103a) from csrc/ with nvcc, in-tree.

Usage: python build.py [--force] [--bounds-check]
The translation units compile in parallel; the library lands next to the
Python package (fastbarnes_gb300/libfastbarnes_gb300.so).  --bounds-check
builds the debug variant libfastbarnes_gb300_checked.so (-DFB_BOUNDS_CHECK:
kernels check their index ranges and report through the status word) into a
build folder of its own; select it at run time with FASTBARNES_GB300_LIB.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "fastbarnes_gb300", "libfastbarnes_gb300.so")
BUILD_CHECKED = os.path.join(HERE, "_build_checked")
LIB_CHECKED = os.path.join(HERE, "fastbarnes_gb300", "libfastbarnes_gb300_checked.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
          "-I", CSRC, "-I", INCLUDE]
# per-file extra flags: the sphere projection keeps separate multiply / add
EXTRA = {"fb_s2.cu": ["-fmad=false"]}
SOURCES = ["fb_sort.cu", "fb_axis.cu", "fb_axis_f32.cu", "fb_axis_f32l.cu", "fb_axis_f64.cu", "fb_axis_f64s.cu",
           "fb_cols.cu", "fb_cols_f32.cu", "fb_cols_f64.cu", "fb_s2.cu", "fb_grad.cu", "fb_naive.cu", "fb_capi.cu"]


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return p


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]


def up_to_date(lib=LIB):
    if not os.path.exists(lib):
        return False
    t = os.path.getmtime(lib)
    return all(os.path.getmtime(d) <= t for d in _deps())


def compile_one(src, verbose=False, checked=False):
    obj = os.path.join(BUILD_CHECKED if checked else BUILD, src.replace(".cu", ".o"))
    cmd = [nvcc()] + ARCH + COMMON + (["-DFB_BOUNDS_CHECK"] if checked else []) + EXTRA.get(src, []) + \
        ["-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(force=False, verbose=False, bounds_check=False):
    lib = LIB_CHECKED if bounds_check else LIB
    if not force and up_to_date(lib):
        return lib
    os.makedirs(BUILD_CHECKED if bounds_check else BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: compile_one(s, verbose, bounds_check), SOURCES))
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    objs = [o for o, _ in results]
    tmp = lib + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, bounds_check="--bounds-check" in sys.argv))
