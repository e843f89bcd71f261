"""The host sort (csrc/stdsort.h): a team of threads must produce std::sort's
exact permutation, ties included, since the order of equal-length reads
decides which read becomes a representative (cuda-version/func.cu:111-113).
A small C++ program compares the two on seeded random inputs of 65k-315k keys
(equal keys, two values, a few values, nearly distinct, presorted, reversed,
organ pipe) with 2-16 threads."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "gene-sequences-de-redundancy_gb300", "csrc")


def test_team_sort_is_std_sort(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    exe = tmp_path / "stdsort_check"
    subprocess.run([gxx, "-O2", "-std=c++17", "-pthread", "-I", CSRC,
                    os.path.join(HERE, "stdsort_check.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe), "160"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0 of 160" in r.stdout
