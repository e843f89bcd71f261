"""The C-ABI libraries load without a GPU and export every function their
public headers declare (no compute calls)."""
import ctypes as C
import os
import re

import pytest

import gsdr

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DECL = re.compile(r"^[A-Za-z_][\w\s\*]*?\b(gsdr_\w+)\s*\(", re.M)


def declared(header):
    with open(os.path.join(ROOT, "include", header)) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(DECL.findall(text)) - {"gsdr_fasta", "gsdr_job", "gsdr_server"})


@pytest.mark.parametrize("header,path", [
    ("gsdr.h", gsdr.LIB_PATH),
    ("gsdr_testing.h", gsdr.LIB_PATH),
    ("gsdr_synth.h", gsdr.SYNTH_PATH),
])
def test_every_declared_symbol_is_exported(header, path):
    lib = C.CDLL(path)
    names = declared(header)
    assert len(names) >= 1
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, f"{header}: not exported by {os.path.basename(path)}: {missing}"


def test_cluster_without_device_fails_loudly():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    f = gsdr.Fasta.parse(b">a\nACGT\n>b\nACG\n")
    with pytest.raises(gsdr.GsdrError) as e:
        gsdr.clustering(f)
    assert e.value.status == gsdr.EDEVICE


def test_cli_usage_exit():
    import subprocess

    r = subprocess.run([gsdr.CLI_PATH, "t"], capture_output=True, text=True)
    assert r.returncode == 0 and "Please check parameters" in r.stdout
