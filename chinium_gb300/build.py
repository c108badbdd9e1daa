"""In-tree build of the CUDA/C++ library (sm_103a only).

Compiles each translation unit of ``csrc/`` in parallel with nvcc and links
``_build/libchinium_xc.so``.  Used by ``__graft_entry__.build()`` and by the
package loader when the library is missing.
"""
import concurrent.futures
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libchinium_xc.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xcompiler", "-Wall,-Wno-unused-function,-Wno-unknown-pragmas", "-Xcompiler", "-fopenmp"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _compile(src, extra):
    obj = os.path.join(OUT, src + ".o")
    cmd = [_nvcc()] + ARCH + NVCC_FLAGS + extra + ["-x", "cu", "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed on %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return obj, r.stderr


def _stale(objs_inputs):
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    for p in objs_inputs:
        if os.path.getmtime(p) > t:
            return True
    return False


def build(force=False, verbose=False, extra=()):
    os.makedirs(OUT, exist_ok=True)
    inputs = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [
        os.path.join(os.path.dirname(HERE), "include", "chinium_xc.h"),
        os.path.join(os.path.dirname(HERE), "include", "chinium_int.h"),
        os.path.join(os.path.dirname(HERE), "include", "chinium_guess.h"), os.path.abspath(__file__)]
    if not force and not _stale(inputs):
        return LIB
    srcs = sources()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))] + inputs[-2:]
    newest_header = max(os.path.getmtime(h) for h in headers)

    def unit(src):
        obj = os.path.join(OUT, src + ".o")
        if (not force and os.path.exists(obj) and os.path.getmtime(obj) > newest_header
                and os.path.getmtime(obj) > os.path.getmtime(os.path.join(CSRC, src))):
            return obj, ""
        return _compile(src, list(extra))

    with concurrent.futures.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        results = list(ex.map(unit, srcs))
    if verbose:
        for _, err in results:
            if err:
                sys.stderr.write(err)
    cmd = [_nvcc()] + ARCH + ["-shared", "-o", LIB] + [o for o, _ in results] + ["-lcudart", "-lgomp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s" % r.stderr)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True,
          extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else [])
    print(LIB)
