"""Build the native library ``gauxc_gb300/lib/libgauxc_gb300.so`` in-tree.

CUDA sources are compiled for sm_103a only; host sources with g++.  Objects go
to ``gauxc_gb300/_build`` and are reused while no source or header changed.
Usage: ``python -m gauxc_gb300.build`` (or ``build()`` from Python).
"""
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libgauxc_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall"] + ARCH
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-pthread"]


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _sources():
    cu, cxx, hdr = [], [], []
    for root, _, files in os.walk(CSRC):
        for f in sorted(files):
            p = os.path.join(root, f)
            if f.endswith(".cu"):
                cu.append(p)
            elif f.endswith(".cxx"):
                cxx.append(p)
            elif f.endswith((".cuh", ".hpp", ".inc", ".h")):
                hdr.append(p)
    hdr.append(os.path.join(INCLUDE, "gauxc_gb300.h"))
    return cu, cxx, hdr


def _digest(paths, extra=""):
    h = hashlib.sha256(extra.encode())
    for p in sorted(paths):
        with open(p, "rb") as f:
            h.update(p.encode())
            h.update(f.read())
    return h.hexdigest()


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build(verbose=False, jobs=None):
    cu, cxx, hdr = _sources()
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    hdr_digest = _digest(hdr, " ".join(NVCC_FLAGS + CXX_FLAGS))
    cmds, objs = [], []
    for src in cu + cxx:
        name = os.path.relpath(src, CSRC).replace(os.sep, "_")
        obj = os.path.join(BUILD, name + ".o")
        stamp = obj + ".stamp"
        key = _digest([src], hdr_digest)
        objs.append(obj)
        if os.path.exists(obj) and os.path.exists(stamp) and open(stamp).read() == key:
            continue
        if src.endswith(".cu"):
            cmd = [nvcc] + NVCC_FLAGS + ["-I", CSRC, "-I", INCLUDE, "-c", src, "-o", obj]
        else:
            cmd = ["g++"] + CXX_FLAGS + ["-I", CSRC, "-I", INCLUDE,
                                         "-I", "/usr/local/cuda/include", "-c", src, "-o", obj]
        cmds.append((cmd, stamp, key))
    jobs = jobs or min(16, os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(jobs) as ex:
        futs = {ex.submit(_run, c[0]): c for c in cmds}
        for fu in cf.as_completed(futs):
            out = fu.result()
            _, stamp, key = futs[fu]
            with open(stamp, "w") as f:
                f.write(key)
            if verbose and out.strip():
                print(out)
    link_key = _digest(objs)
    lstamp = LIB + ".stamp"
    if cmds or not os.path.exists(LIB) or not os.path.exists(lstamp) or open(lstamp).read() != link_key:
        tmp = LIB + ".tmp"
        _run([nvcc, "-shared"] + ARCH + objs + ["-o", tmp, "-lcudart_static", "-lrt", "-ldl",
                                                  "-lpthread"])
        os.replace(tmp, LIB)
        with open(lstamp, "w") as f:
            f.write(link_key)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
