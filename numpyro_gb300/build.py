"""Builds libgbnuts.so (the C-ABI CUDA library) in-tree for sm_103a.

Each translation unit in csrc/ is compiled by nvcc in parallel and linked as a
shared library next to this file.  Used by ``__graft_entry__.build()``, and by
``python -m numpyro_gb300.build``.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgbnuts.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              "--expt-relaxed-constexpr", "-I", CSRC, "-I", INCLUDE]
SOURCES = ["nuts_engine.cu", "potentials_simt.cu", "logreg_tc.cu", "horseshoe_tc.cu", "capi.cu", "noalloc.cu"]


def nvcc():
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    path = os.path.join(cuda, "bin", "nvcc")
    return path if os.path.exists(path) else (shutil.which("nvcc") or "nvcc")


def _compile(src, verbose_ptxas=False):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
    if verbose_ptxas:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return obj, r.stderr


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    for f in os.listdir(CSRC):
        if os.path.getmtime(os.path.join(CSRC, f)) > t:
            return True
    return os.path.getmtime(os.path.join(INCLUDE, "gbnuts.h")) > t


XLA_LIB = os.path.join(HERE, "libgbnuts_xla.so")
# why libgbnuts_xla.so (the XLA FFI handlers of csrc/xla_ffi.cc) was not built, or None
XLA_FFI_STATUS = None


def xla_ffi_include():
    """(directory holding xla/ffi/api/ffi.h, None) or (None, reason): the headers come with jaxlib
    (jax.ffi.include_dir()); XLA_FFI_INCLUDE_DIR overrides."""
    cand = os.environ.get("XLA_FFI_INCLUDE_DIR")
    if not cand:
        try:
            import jax.ffi

            cand = jax.ffi.include_dir()
        except Exception as ex:  # jax absent: the jax side of the boundary cannot be built
            return None, "jax is not importable (%s): no XLA FFI headers" % str(ex).splitlines()[0]
    if not os.path.exists(os.path.join(cand, "xla", "ffi", "api", "ffi.h")):
        return None, "no xla/ffi/api/ffi.h under %s" % cand
    return cand, None


def build_xla_ffi():
    """Builds libgbnuts_xla.so from csrc/xla_ffi.cc when the XLA FFI headers are available;
    returns its path, or None (the reason is in XLA_FFI_STATUS)."""
    global XLA_FFI_STATUS
    inc, why = xla_ffi_include()
    if inc is None:
        XLA_FFI_STATUS = why
        return None
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I", inc, "-I", INCLUDE,
           "-I", os.path.join(cuda, "include"), os.path.join(CSRC, "xla_ffi.cc"), "-o", XLA_LIB + ".tmp",
           "-L", HERE, "-lgbnuts", "-Wl,-rpath,$ORIGIN", "-L", os.path.join(cuda, "lib64"), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        XLA_FFI_STATUS = "xla_ffi.cc failed to compile: " + (r.stderr or r.stdout)[-400:]
        return None
    os.replace(XLA_LIB + ".tmp", XLA_LIB)
    XLA_FFI_STATUS = None
    return XLA_LIB


def build(force=False, verbose_ptxas=False):
    """Compile csrc/*.cu for sm_103a and link libgbnuts.so (and, where the XLA FFI headers
    exist, libgbnuts_xla.so); returns the path of libgbnuts.so."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose_ptxas), SOURCES))
    objs = [o for o, _ in results]
    if verbose_ptxas:
        for _, log in results:
            sys.stderr.write(log)
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    build_xla_ffi()
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
