"""Build the CUDA library liblqgpu.so for sm_103a (GB300) in-tree.

Each translation unit is compiled by its own nvcc process in parallel, then linked into
``_build/liblqgpu.so``; nothing is installed outside this directory.
"""
import concurrent.futures
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD_DIR, "liblqgpu.so")
INCLUDE = os.path.join(REPO, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC,
]
SOURCES = ["lq_api.cu", "lq_f64.cu", "lq_f32.cu", "lq_mixed.cu", "lq_noalloc.cu", "lq_peak.cu", "lq_batch.cu",
           "lq_batch_f64.cu", "lq_batch_f32.cu", "lq_batch_mixed.cu"]


def nvcc():
    for cand in (os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc"), "nvcc"):
        if os.path.sep not in cand or os.path.exists(cand):
            return cand
    return "nvcc"


def _deps():
    paths = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    paths.append(os.path.join(INCLUDE, "lqgpu.h"))
    paths.append(os.path.abspath(__file__))
    return max(os.path.getmtime(p) for p in paths)


def _compile(src, extra, obj_dir):
    obj = os.path.join(obj_dir, src.replace(".cu", ".o"))
    cmd = [nvcc()] + NVCC_FLAGS + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return obj, r.stderr


def build(force=False, verbose=False, extra=None, out=None):
    """Compile and link; returns the path of the shared library.  `extra` adds nvcc flags
    (e.g. -D tuning knobs) and `out` names another output library for such a variant."""
    extra = list(extra or [])
    lib = out or LIB
    obj_dir = os.path.join(BUILD_DIR, "obj_" + os.path.basename(lib).replace(".so", "")) if out else BUILD_DIR
    os.makedirs(obj_dir, exist_ok=True)
    os.makedirs(os.path.dirname(lib), exist_ok=True)
    if not force and not extra and os.path.exists(lib) and os.path.getmtime(lib) >= _deps():
        return lib
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, extra, obj_dir), SOURCES))
    if verbose:
        for _, err in results:
            if err:
                sys.stderr.write(err)
    tmp = lib + ".tmp.%d" % os.getpid()
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + [o for o, _ in results] + ["-lpthread", "-ldl", "-lrt"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    ex = ["-Xptxas", "-v"] if "--ptxas-v" in sys.argv else []
    print(build(force=True, verbose=True, extra=ex))
