"""The C++ host mirror of the reference interfaces (rheotool_gb300/host):
tests/host/test_host.cpp compiled against librheogpu_host.so.  On the CPU:
dictionary parsing, run-time selection by the reference's names and its
FatalError messages, and the error raised when no GPU can be opened.  On the
GPU: LduSolver::New + solve (PCG-DIC, PBiCGStab-DILU) on a chain of cells
against a direct tridiagonal solve."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "rheotool_gb300")


def _binary(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    from rheotool_gb300 import build
    build.build_host()
    exe = str(tmp_path / "test_host")
    subprocess.check_call([cxx, "-std=c++17", "-O1", "-o", exe, os.path.join(ROOT, "tests", "host", "test_host.cpp"),
                           "-L" + PKG, "-lrheogpu_host", "-lrheogpu", "-Wl,-rpath," + PKG])
    return exe


def test_host_mirror_cpu(tmp_path):
    exe = _binary(tmp_path)
    r = subprocess.run([exe, "--cpu"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr


@pytest.mark.gpu
def test_host_mirror_gpu(tmp_path):
    exe = _binary(tmp_path)
    r = subprocess.run([exe, "--gpu"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
