"""The pair-functor API builds for a user: a functor written against
include/xnb_pair.cuh and include/xnb_gpu.h alone (tests/functors/morse_pair.cu)
compiles into its own sm_103a shared library, without the library's sources or
build tree (no GPU needed)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "functors", "morse_pair.cu")


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        pytest.skip("nvcc not found")
    return exe


def build_user_functor(out_dir):
    """nvcc with -I include only: the public headers are all a functor needs."""
    out = os.path.join(str(out_dir), "libmorse_pair.so")
    cmd = [nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-shared", "-Xcompiler",
           "-fPIC", "-I", os.path.join(ROOT, "include"), SRC, "-o", out]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def test_user_functor_compiles_against_include_alone(tmp_path):
    inc = tmp_path / "include"
    shutil.copytree(os.path.join(ROOT, "include"), inc)
    out = tmp_path / "libmorse_pair.so"
    cmd = [nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-shared", "-Xcompiler",
           "-fPIC", "-I", str(inc), SRC, "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True, cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    nm = subprocess.run(["nm", "-D", "--defined-only", str(out)], capture_output=True, text=True).stdout
    assert " morse_force" in nm
