"""Golden outputs of the reference program itself.

tests/golden/reference_outputs.json was made by tests/golden/make_golden.py:
the reference's cuda-version program, built unmodified for sm_103a by
oracle/build_ref.sh, run on a GB300 on every case of tests/golden/cases.py.
The inputs are rebuilt here byte for byte (their sha256 is checked), so the
oracle (CPU) and the GPU path must reproduce the reference's output bytes.
"""
import hashlib
import json
import os
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import cases  # noqa: E402
import gsdr  # noqa: E402
import oracle_binding as orc  # noqa: E402

with open(os.path.join(HERE, "golden", "reference_outputs.json")) as f:
    GOLDEN = json.load(f)

# cases small enough for the oracle in the CPU suite
CPU_CASES = ["c0_10k_t95", "c0_3k_t90", "c0_3k_t97", "c0_2k_t88", "c0_2k_w7",
             "c0_800_t85_drop", "c0_800_t95_d1", "c2_30k_t90", "ties_150bp_t95",
             "edge_mixed_t95", "edge_mixed_t90", "ref_result_t95", "c0_3k_t95_p1",
             "c0_2k_t90_p1", "c4_2k_t93_p1", "edge_mixed_t95_p1", "c0_2k_w8",
             "c0_2k_w10", "c0_1k_w12"]


def sha(b):
    return hashlib.sha256(b).hexdigest()


def case_input(name):
    spec, argv = cases.CASES[name]
    data = cases.build_input(spec)
    assert sha(data) == GOLDEN[name]["input_sha256"], f"{name}: generated input drifted"
    return data, dict(zip(argv[0::2], argv[1::2]))


def test_every_case_has_a_golden_record():
    assert set(GOLDEN) == set(cases.CASES)
    assert all(g["oracle_matches"] and g["reference_rc"] == 0 for g in GOLDEN.values())


def test_reference_result_fasta_is_a_fixed_point():
    # the reference's own output file (1,361 representatives at t = 0.95):
    # clustering it again keeps every record
    g = GOLDEN["ref_result_t95"]
    assert g["records"] == 1361 and g["output_bytes"] == g["input_bytes"]


@pytest.mark.parametrize("name", CPU_CASES)
def test_oracle_reproduces_reference(tmp_path, name):
    data, o = case_input(name)
    _, _, _, out = orc.run_bytes(data, tmp_path, t=float(o.get("t", 0.95)),
                                 w=int(o.get("w", 0)), d=int(o.get("d", 3)),
                                 p=int(o.get("p", 0)))
    assert sha(out) == GOLDEN[name]["output_sha256"]


@pytest.mark.gpu
@pytest.mark.parametrize("batch", [1, 0])
@pytest.mark.parametrize("name", sorted(cases.CASES))
def test_gpu_reproduces_reference(name, batch):
    data, o = case_input(name)
    f = gsdr.Fasta.parse(data)
    try:
        cl = gsdr.clustering(f, gsdr.default_opts(threshold=float(o.get("t", 0.95)),
                                                  word_length=int(o.get("w", 0)),
                                                  drop=int(o.get("d", 3)),
                                                  pigeon=int(o.get("p", 0)), batch=batch))
        out = f.format(cl)
    finally:
        f.close()
    assert sha(out) == GOLDEN[name]["output_sha256"]
    assert len(out) == GOLDEN[name]["output_bytes"]


@pytest.mark.gpu
def test_cli_reproduces_reference(tmp_path):
    import subprocess

    data, o = case_input("c0_3k_t90")
    inp, outp = tmp_path / "in.fa", tmp_path / "out.fa"
    inp.write_bytes(data)
    r = subprocess.run([gsdr.CLI_PATH, "i", str(inp), "o", str(outp), "t", o["t"]],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert sha(outp.read_bytes()) == GOLDEN["c0_3k_t90"]["output_sha256"]
    # the membership extension (c <path>) leaves the FASTA bytes unchanged
    clstr = tmp_path / "out.clstr"
    r = subprocess.run([gsdr.CLI_PATH, "i", str(inp), "o", str(outp), "t", o["t"],
                        "c", str(clstr)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert sha(outp.read_bytes()) == GOLDEN["c0_3k_t90"]["output_sha256"]
    text = clstr.read_bytes().decode()
    assert text.count(">Cluster ") == GOLDEN["c0_3k_t90"]["records"]
    assert text.count("\n") == text.count(">Cluster ") + len(data.split(b">")) - 1


# ---- the two reference programs' own result files --------------------------
#
# cuda-version/result.fasta (1,361 records) and the SYCL program's top-level
# result.fasta (1,378 records) come from the same input (not distributed) at
# t = 0.95 under the two programs' semantics.  Clustering the union of both
# (longest first, ties led by the records of the file being reproduced) with
# one program's semantics must give back exactly that program's file: 32
# records absorbed with the cuda-version rules, 15 with the SYCL rules.

@pytest.mark.parametrize("which,variant,absorbed", [("cuda", 0, 32), ("sycl", 1, 15)])
def test_oracle_union_of_result_files(tmp_path, which, variant, absorbed):
    recs, have = cases.union_of_results(which)
    data = b"".join(n + b"\n" + s + b"\n" for n, s in recs)
    _, cl, st, out = orc.run_bytes_in_order(data, tmp_path, t=0.95, variant=variant)
    assert out == cases.reference_result(which)
    assert st.accepted == absorbed == len(recs) - len(have)


def test_sycl_result_file_is_a_fixed_point(tmp_path):
    data = cases.reference_result("sycl")
    _, cl, st, out = orc.run_bytes(data, tmp_path, t=0.95, variant=1)
    # every record stays (std::sort may order equal lengths differently)
    assert st.accepted == 0
    assert sorted(cases.records(out)) == sorted(cases.records(data))


@pytest.mark.gpu
@pytest.mark.parametrize("batch", [1, 0])
@pytest.mark.parametrize("which,variant", [("cuda", 0), ("sycl", 1)])
def test_gpu_union_of_result_files(which, variant, batch):
    recs, have = cases.union_of_results(which)
    cl = gsdr.cluster_reads([s for _, s in recs], gsdr.default_opts(threshold=0.95,
                                                                  variant=variant, batch=batch))
    keep = [recs[i] for i in range(len(recs)) if cl[i] == i]
    assert keep == cases.records(cases.reference_result(which))
