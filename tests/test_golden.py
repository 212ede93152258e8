"""Golden vectors from the reference's own CPU path (tests/golden/owm_golden.json,
made by tests/golden/make_golden.py from CPP-TBB-CPU/src/optim3_func.cpp).

CPU: the generator reproduces every cloud bit for bit (SHA-256), and the
oracle restatement equals the reference on every tie-free case; on clouds
with z ties the reference and the (z, id) restatement differ only in which of
two equal-z points a window keeps.
GPU: every stage of the CUDA path equals the golden vectors (the reference's
on tie-free clouds, the restatement's on clouds with ties).
"""
import base64
import hashlib
import json
import zlib
from pathlib import Path

import numpy as np
import pytest

GOLDEN = json.loads((Path(__file__).resolve().parent / "golden" / "owm_golden.json").read_text())
CASES = {c["name"]: c for c in GOLDEN["cases"]}


def unpack(s):
    return np.frombuffer(zlib.decompress(base64.b64decode(s)), dtype=np.int64).copy()


def cloud(owm, case):
    r = case["recipe"]
    if "points" in r:
        xyz = np.array(r["points"], dtype=np.float64)
        bb = owm.bbox_of(xyz)
    else:
        spec = owm.SynthSpec()
        for k, v in r["spec"].items():
            setattr(spec, k, v)
        xyz, bb = owm.synth_cloud(spec, r["seed"])
    assert hashlib.sha256(np.ascontiguousarray(xyz).tobytes()).hexdigest() == case["sha256"], "generator drift"
    assert list(bb.astuple()) == case["bbox"]
    return xyz, bb


def expected(case):
    """Parity target: the reference where it is tie-free, else the restatement."""
    src = case["reference"] if ("reference" in case and not case["ties"]) else case["restated"]
    return unpack(src["win_min"]), unpack(src["llp"]), unpack(src["stage3"])


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_golden(owm, oracle, name):
    case = CASES[name]
    xyz, bb = cloud(owm, case)
    p = oracle.params(bb, case["n"], case["wsize"], case["overlap"], case["bsize"])
    win = oracle.stage1(xyz, p)
    llp = oracle.stage2(win, case["overlap"])
    s3 = oracle.stage3(xyz, p, llp)
    rw, rl, rs = (unpack(case["restated"][k]) for k in ("win_min", "llp", "stage3"))
    np.testing.assert_array_equal(win, rw)
    np.testing.assert_array_equal(llp, rl)
    np.testing.assert_array_equal(s3, rs)
    if "reference" in case:
        ref_win = unpack(case["reference"]["win_min"])
        assert case["reference"]["min_num_points"] == p.min_num_points
        if not case["ties"]:
            assert case["reference_equals_restatement"]
            np.testing.assert_array_equal(win, ref_win)
        else:
            # differences are tie-breaks only: same validity, same z
            d = np.nonzero(win != ref_win)[0]
            assert np.array_equal(win[d] >= 0, ref_win[d] >= 0)
            z = np.concatenate([[np.finfo(np.float64).max], xyz[:, 2]])
            np.testing.assert_array_equal(z[win[d]], z[ref_win[d]])


def test_golden_covers_edge_cases():
    names = set(CASES)
    assert {"c1_full", "c2_sample", "c3_o05", "c3_o08", "c4_tile0", "sparse", "tiny5", "c1_overlap0",
            "c1_odd_w_b"} <= names
    assert any(c["ties"] for c in CASES.values())
    assert any(unpack(c["restated"]["llp"]).size and unpack(c["restated"]["llp"])[0] == 0 for c in CASES.values()), \
        "a case where the sentinel id 0 is an LLP (minNumPoints == 0)"
    assert any(unpack(c["restated"]["stage3"]).size > 0 for c in CASES.values())


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_matches_golden(owm, ctx, name):
    case = CASES[name]
    xyz, bb = cloud(owm, case)
    W, Ov, B = case["wsize"], case["overlap"], case["bsize"]
    ew, el, es = expected(case)
    p = owm.params(bb, case["n"], W, Ov, B)
    c = ctx.cloud(xyz, bb)
    t = ctx.tree(c, case["policy"], case["max_number"])
    win = ctx.stage1(t, p)
    np.testing.assert_array_equal(win, ew)
    llp = ctx.stage2(win, Ov)
    np.testing.assert_array_equal(llp, el)
    s3 = ctx.stage3(t, p, llp)
    np.testing.assert_array_equal(s3, es)
    seeds = ctx.run(c, owm.run_cfg(W, Ov, B, case["max_number"], case["policy"]))
    np.testing.assert_array_equal(seeds, np.concatenate([es, el]))
    t.close()
    c.close()


@pytest.mark.parametrize("name", sorted(n for n, c in CASES.items() if "reference" in c))
def test_reference_port_matches_golden(owm, oracle, name):
    """The C port of the reference's quadtree algorithm (the timed CPU
    baseline on machines without the reference sources) returns the
    reference's seeds exactly, ties included: same tree, same visiting order."""
    case = CASES[name]
    xyz, bb = cloud(owm, case)
    ref = case["reference"]
    seeds, n_llp, _, _ = oracle.port_run(xyz, bb, case["wsize"], case["overlap"], case["bsize"],
                                         policy=case["policy"], max_number=case["max_number"], nthreads=2)
    assert n_llp == ref["n_llp"]
    n3 = len(seeds) - n_llp  # seeds = stage-3 ids ++ LLPs
    np.testing.assert_array_equal(seeds[n3:], unpack(ref["llp"]))
    np.testing.assert_array_equal(seeds[:n3], unpack(ref["stage3"]))
