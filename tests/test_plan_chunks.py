"""The job layout computed in parts (csrc/plan_chunks.h): the FASTA path lays
out the reads' packed words and k-mer entries on the sort's threads, each over
the reads it gathered, then shifts each part by the parts before it.  A small
C++ program runs that protocol through the team sort (csrc/stdsort.h) and
compares offsets and sums with a serial restatement, for 0-200k reads, 1-16
threads, word lengths 1-12, drop mode, and lengths that clamp (0, below k,
above 4^k).  The serial pass is the one Job::init takes when no layout is
given."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "gene-sequences-de-redundancy_gb300", "csrc")


def test_layout_in_parts_is_the_serial_layout(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    exe = tmp_path / "plan_chunks_check"
    subprocess.run([gxx, "-O2", "-std=c++17", "-pthread", "-I", CSRC,
                    os.path.join(HERE, "plan_chunks_check.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe), "200"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0 of 200" in r.stdout
