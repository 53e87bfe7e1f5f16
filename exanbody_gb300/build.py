"""Build libxnb_gpu.so (the sm_103a CUDA library behind include/xnb_gpu.h).

Each .cu under csrc/ is compiled in parallel with
    nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo -O3
(host-only .cpp files, the dump file codec, through the same driver) and linked
into exanbody_gb300/_build/libxnb_gpu.so (in-tree, git-ignored).
Host code is compiled with -ffp-contract=off so host-side geometry (bucketing,
domain descriptors) rounds exactly like the reference on x86_64 and aarch64.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libxnb_gpu.so")
ROOT = os.path.dirname(HERE)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-I", os.path.join(ROOT, "include")]


def nvcc():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    for cand in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


HOST = os.path.join(HERE, "host")
EXEC = os.path.join(OUT, "xnb-exec")


def build_host(verbose=False):
    """xnb-exec: the C++ operator/deck runner over libxnb_gpu.so."""
    srcs = sorted(os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".cpp"))
    deps = srcs + [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".hpp")] + [LIB]
    if not _stale(EXEC, deps):
        return EXEC
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), *srcs,
           "-L", OUT, "-lxnb_gpu", "-Wl,-rpath,$ORIGIN", "-o", EXEC + ".tmp"]
    if verbose:
        print(" ".join(cmd), flush=True)
    if subprocess.call(cmd) != 0:
        raise RuntimeError("xnb-exec build failed")
    os.replace(EXEC + ".tmp", EXEC)
    return EXEC


def build(verbose=False, extra_flags=None):
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers += [os.path.join(ROOT, "include", f) for f in ("xnb_gpu.h", "xnb_dump.h")]
    flags = NVCC_FLAGS + (extra_flags or [])
    objs, procs = [], []
    for src in sources():
        obj = os.path.join(OUT, os.path.splitext(os.path.basename(src))[0] + ".o")
        objs.append(obj)
        if _stale(obj, [src, __file__] + headers):
            cmd = [nvcc(), *ARCH, *flags, "-c", src, "-o", obj]
            if verbose:
                print(" ".join(cmd), flush=True)
            procs.append((subprocess.Popen(cmd), src))
    for p, src in procs:
        if p.wait() != 0:
            raise RuntimeError("nvcc failed on %s" % src)
    if _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-ldl", "-lpthread"]
        if verbose:
            print(" ".join(cmd), flush=True)
        if subprocess.call(cmd) != 0:
            raise RuntimeError("link failed")
        os.replace(LIB + ".tmp", LIB)
    build_host(verbose)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
