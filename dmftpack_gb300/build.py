"""Build libdmftgpu.so (sm_103a) in-tree: dmftpack_gb300/_build/libdmftgpu.so.

Every translation unit under csrc/ is compiled by nvcc in parallel and linked into one shared library
exporting the C ABI of include/dmftgpu.h.  A stamp (hash of sources + flags) skips up-to-date builds.
"""
import concurrent.futures as cf
import glob
import hashlib
import os
import platform
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libdmftgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INCLUDE, "-I" + CSRC]


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: libdmftgpu needs the CUDA toolkit to build")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _stamp():
    h = hashlib.sha256()
    h.update(" ".join(NVCC_FLAGS).encode())
    for p in sorted(_sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
                    + glob.glob(os.path.join(INCLUDE, "*.h"))):
        h.update(os.path.basename(p).encode())
        with open(p, "rb") as f:
            h.update(f.read())
    return h.hexdigest()


def _headers_hash():
    h = hashlib.sha256()
    h.update(" ".join(NVCC_FLAGS).encode())
    h.update(platform.machine().encode())
    for p in sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
                    + glob.glob(os.path.join(INCLUDE, "*.h"))):
        h.update(os.path.basename(p).encode())
        with open(p, "rb") as f:
            h.update(f.read())
    return h.hexdigest()


def build(verbose=False, force=False):
    """Compile every CUDA translation unit for sm_103a and link libdmftgpu.so; returns its path."""
    os.makedirs(os.path.join(BUILD, "obj"), exist_ok=True)
    stamp_path = os.path.join(BUILD, "stamp")
    stamp = _stamp()
    if not force and os.path.exists(LIB) and os.path.exists(stamp_path):
        with open(stamp_path) as f:
            if f.read().strip() == stamp:
                return LIB
    nvcc = _nvcc()
    srcs = _sources()
    objs = [os.path.join(BUILD, "obj", os.path.basename(s)[:-3] + ".o") for s in srcs]

    hh = _headers_hash()

    def compile_one(pair):
        src, obj = pair
        with open(src, "rb") as f:
            key = hashlib.sha256(hh.encode() + f.read()).hexdigest()
        key_path = obj + ".key"
        if not force and os.path.exists(obj) and os.path.exists(key_path):
            with open(key_path) as f:
                if f.read().strip() == key:
                    return obj  # this object is up to date for this machine, flags and headers
        cmd = [nvcc] + NVCC_FLAGS + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
        with open(key_path, "w") as f:
            f.write(key)
        if verbose:
            print("compiled", os.path.basename(src), flush=True)
        return obj

    workers = max(1, min(len(srcs), os.cpu_count() or 4))
    with cf.ThreadPoolExecutor(workers) as ex:
        list(ex.map(compile_one, zip(srcs, objs)))
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    with open(stamp_path, "w") as f:
        f.write(stamp)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
