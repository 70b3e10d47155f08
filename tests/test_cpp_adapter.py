"""The header-only C++ adapter (include/hyset_gb300.hpp) compiles against the
library and drives the reference-shaped handlers; on a GPU its counts are the
golden ones."""
import os
import shutil
import subprocess

import pytest

from conftest import GOLDEN, ROOT, load_golden

SRC = os.path.join(ROOT, "tests", "cpp", "adapter_join.cpp")
LIB_DIR = os.path.join(ROOT, "hyset_gb300")


def _build(tmp_path):
    if not shutil.which("g++"):
        pytest.skip("no C++ compiler")
    if not os.path.exists(os.path.join(LIB_DIR, "libhyset_gb300.so")):
        pytest.skip("library not built")
    exe = str(tmp_path / "adapter_join")
    cuda_lib = "/usr/local/cuda/lib64"
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe, "-L", LIB_DIR,
           "-lhyset_gb300", f"-Wl,-rpath,{LIB_DIR}"]
    if os.path.isdir(cuda_lib):
        cmd += [f"-Wl,-rpath,{cuda_lib}"]
    subprocess.run(cmd, check=True, capture_output=True)
    return exe


def test_adapter_compiles_and_runs(tmp_path):
    exe = _build(tmp_path)
    out = subprocess.run([exe, os.path.join(GOLDEN, "toy.sets.txt"), "0.5"], capture_output=True, text=True,
                         timeout=120)
    assert out.returncode == 0, out.stderr
    assert out.stdout.startswith(("no device", "fgss "))


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["toy", "c1_small"])
def test_adapter_counts_are_golden(tmp_path, name):
    exe = _build(tmp_path)
    _, _, _, results = load_golden(name)
    for tau, want in results.items():
        out = subprocess.run([exe, os.path.join(GOLDEN, f"{name}.sets.txt"), repr(tau)], capture_output=True,
                             text=True, timeout=300)
        assert out.returncode == 0, out.stderr
        f = out.stdout.split()
        counts = {f[i]: int(f[i + 1]) for i in range(0, len(f), 2)}
        assert counts == {"fgss": want["count"], "bitmap": want["count"], "fast": want["count"],
                          "verifier": want["count"]}, (name, tau, out.stdout)
