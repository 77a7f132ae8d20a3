"""Build libcsadv.so (the CUDA kernels + C ABI) in-tree with nvcc for sm_103a.

    python py-cubed-sphere_gb300/csadv/build.py [--force] [--jobs N]

Each translation unit is compiled in parallel; the shared library is written next to this
file.  Translation units that must reproduce the reference's floating-point operation
order are compiled with ``-fmad=false`` (no fused multiply-add contraction); the fused
engine is compiled with contraction allowed.  Host code is compiled with
``-ffp-contract=off`` so x86-64 and aarch64 hosts round identically.
"""
import argparse
import concurrent.futures as cf
import hashlib
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
CSRC = os.path.join(PKG, "csrc")
ROOT = os.path.dirname(PKG)
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(HERE, "libcsadv.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "-I", os.path.join(ROOT, "include"), "--expt-relaxed-constexpr", "-rdc=false"]
# translation units and whether FMA contraction is allowed in their device code
UNITS = {
    "api.cu": False,
    "batch.cu": False,
    "grid.cu": False,
    "halo.cu": False,
    "wind.cu": False,
    "staged.cu": False,
    "io.cu": False,
    "fused_host.cu": False,
    "fused_f32.cu": True,
    "fused_f64.cu": True,
    "sweep_f32.cu": True,
    "sweep_f32_pairs.cu": True,
    "sweep_f32_one.cu": True,
    "sweep_f64.cu": True,
    "noalloc.cu": False,
    "latlon.cu": False,
    "peak.cu": True,
}


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


STAMP = LIB + ".sha256"


def source_digest():
    """SHA-256 over every source the library is built from (csrc/, the public header, this
    script), the compiler flags, the nvcc in use and the host architecture: the library is
    rebuilt whenever one of them differs from the build that wrote the stamp file."""
    h = hashlib.sha256()
    deps = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC))
    deps += [os.path.join(ROOT, "include", "csadv.h"), os.path.abspath(__file__)]
    for p in deps:
        if os.path.isfile(p):
            h.update(os.path.basename(p).encode() + b"\0")
            with open(p, "rb") as f:
                h.update(f.read())
    h.update(repr((ARCH, COMMON, sorted(UNITS.items()), platform.machine())).encode())
    try:
        h.update(os.path.realpath(nvcc()).encode())
    except RuntimeError:
        pass
    return h.hexdigest()


def up_to_date():
    if not (os.path.exists(LIB) and os.path.exists(STAMP)):
        return False
    with open(STAMP) as f:
        return f.read().strip() == source_digest()


def build(force=False, jobs=None, verbose=False):
    """Compile every unit and link libcsadv.so; returns the library path."""
    if not force and up_to_date():
        return LIB
    digest = source_digest()
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()

    def compile_unit(name):
        src = os.path.join(CSRC, name)
        obj = os.path.join(BUILD, name + ".o")
        flags = list(COMMON)
        if not UNITS[name]:
            flags.append("-fmad=false")
        cmd = [cc] + ARCH + flags + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (name, " ".join(cmd), r.stderr))
        if verbose and r.stderr.strip():
            print(r.stderr, file=sys.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_unit, sorted(UNITS)))
    tmp = LIB + ".tmp"
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, LIB)
    with open(STAMP, "w") as f:
        f.write(digest + "\n")
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--jobs", type=int, default=None)
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args()
    print(build(force=a.force, jobs=a.jobs, verbose=a.verbose))
