"""Build the native libraries of the package in-tree.

* ``neopz_gb300/_build/libgpz.so``: the CUDA kernels and the C ABI of
  ``include/gpz.h`` (nvcc, sm_103a only).
* ``neopz_gb300/_build/libgpzhost.so``: the C++ host side that mirrors the
  reference's mesh / struct-matrix / solver API and calls the C ABI (g++).

Translation units are compiled in parallel; outputs are rebuilt only when a
source or header is newer.
"""
import concurrent.futures as cf
import glob
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
                  "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include")]

LIBGPZ = os.path.join(BUILD, "libgpz.so")
LIBHOST = os.path.join(BUILD, "libgpzhost.so")


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build(verbose=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    headers = (glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) +
               glob.glob(os.path.join(ROOT, "include", "*.h")))
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    objs, jobs_l = [], []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s) + ".o")
        objs.append(o)
        if _newer(o, [s] + headers):
            jobs_l.append([NVCC] + NVFLAGS + ["-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        for out in ex.map(_run, jobs_l):
            if verbose and out.strip():
                print(out)
    if _newer(LIBGPZ, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", LIBGPZ] + objs + ["-lcudart"])
    hsrcs = sorted(glob.glob(os.path.join(HOST, "*.cpp")))
    hheaders = glob.glob(os.path.join(HOST, "*.h")) + glob.glob(os.path.join(ROOT, "include", "*.h"))
    if hsrcs and _newer(LIBHOST, hsrcs + hheaders + [LIBGPZ]):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I" + os.path.join(ROOT, "include"), "-o", LIBHOST]
             + hsrcs + ["-L" + BUILD, "-lgpz", "-Wl,-rpath,$ORIGIN"])
    return LIBGPZ


if __name__ == "__main__":
    build(verbose=True)
    print("built", LIBGPZ)
