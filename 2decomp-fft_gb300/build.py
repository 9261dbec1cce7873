"""Build recipe for the GB300 FFT backend library (libgbfft.so).

Every CUDA translation unit under csrc/ is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, then linked into
``lib/libgbfft.so`` next to this file.  The library exports the C ABI of
``include/gbfft.h`` and ``include/decomp_2d_fft.h``.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "lib", "obj")
LIB = os.path.join(HERE, "lib", "libgbfft.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
              "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC]


def nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith((".cu", ".cpp")))


def _newest_input():
    files = sources() + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    files += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    files.append(os.path.abspath(__file__))
    return max(os.path.getmtime(f) for f in files)


def paths(variant=""):
    """(object directory, library path) of a build variant: "" the product
    library lib/libgbfft.so, "debug" the bounds-checked build
    lib/debug/libgbfft.so (-DGB_DEBUG_BOUNDS)."""
    if not variant:
        return OBJ, LIB
    return os.path.join(HERE, "lib", "obj_" + variant), os.path.join(HERE, "lib", variant, "libgbfft.so")


VARIANT_FLAGS = {"": [], "debug": ["-DGB_DEBUG_BOUNDS"]}


def _compile(src, extra, obj_dir=OBJ):
    obj = os.path.join(obj_dir, os.path.basename(src) + ".o")
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + extra + ["-c", src, "-o", obj]
    if src.endswith(".cpp"):
        cmd[1:1] = ["-x", "cu"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj, r.stderr


def build(force=False, verbose=False, extra=(), variant=""):
    """Compile and link the library (or a variant of it) if any input is
    newer; return its path."""
    obj_dir, lib_path = paths(variant)
    os.makedirs(obj_dir, exist_ok=True)
    os.makedirs(os.path.dirname(lib_path), exist_ok=True)
    if not force and os.path.exists(lib_path) and os.path.getmtime(lib_path) >= _newest_input():
        return lib_path
    srcs = sources()
    flags = list(extra) + VARIANT_FLAGS[variant]
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda s: _compile(s, flags, obj_dir), srcs))
    if verbose:
        for _, log in results:
            if log.strip():
                print(log)
    tmp = lib_path + ".tmp.%d" % os.getpid()
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + [o for o, _ in results] + ["-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, lib_path)
    return lib_path


if __name__ == "__main__":
    extra = [a for a in sys.argv[1:] if a.startswith("-X") or a.startswith("-D")]
    variant = sys.argv[sys.argv.index("--variant") + 1] if "--variant" in sys.argv else ""
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, extra=extra, variant=variant))
