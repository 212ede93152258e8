"""CPU checks of the cloud-text oracle (oracle_xyz_parse), the checker of the
device ingest.

* Pinned against the reference's own readXYZfile (optim3_func.cpp:665-722,
  compiled from the reference sources into oracle/_ref) on header files in
  several number formats: same points, bit for bit, and the header bbox.
* The product's host loader (owm_xyz_read) follows the same rules: same
  points and bbox as the oracle, and the same verdict on malformed files.
"""
import numpy as np
import pytest

from oracle import oracle as O


def _fmt_lines(xyz, fmt, extra=""):
    return "".join(f"{fmt % x} {fmt % y} {fmt % z}{extra}\n" for x, y, z in xyz)


def _header(xyz, bbox):
    return f"{len(xyz)}\n{bbox[0]!r}\n{bbox[2]!r}\n{bbox[1]!r}\n{bbox[3]!r}\n"


FORMATS = ["%.2f", "%.3f", "%.6f", "%.17g", "%.10e", "%.20g"]


def _cloud(seed, n=3000):
    rng = np.random.default_rng(seed)
    xyz = np.column_stack([600000 + rng.random(n) * 2000, 4500000 + rng.random(n) * 2000, 80 + rng.random(n) * 60])
    return xyz, (600000.0, 4500000.0, 602000.0, 4502000.0)


@pytest.mark.parametrize("fmt", FORMATS)
def test_oracle_equals_reference_loader(tmp_path, fmt):
    if not O.ref_available():
        pytest.skip("reference sources not present")
    xyz, bb = _cloud(FORMATS.index(fmt))
    text = _header(xyz, bb) + _fmt_lines(xyz, fmt, " 12 7 1")
    f = tmp_path / "sampleArzuaH.xyz"  # a header name readXYZfile knows
    f.write_text(text)
    ref = O.ref_read_xyz(f, len(xyz) + 4)
    got = O.xyz_parse(text.encode())
    assert ref is not None and got is not None
    np.testing.assert_array_equal(got[0], ref[0])
    assert got[1] == ref[1] and got[2]


def test_oracle_equals_reference_loader_with_blank_lines_and_crlf(tmp_path):
    if not O.ref_available():
        pytest.skip("reference sources not present")
    xyz, bb = _cloud(7, 500)
    body = _fmt_lines(xyz, "%.4f").replace("\n", "\r\n")
    lines = body.split("\r\n")
    body = "\r\n\r\n".join(lines[:200]) + "\r\n" + "\r\n".join(lines[200:])
    text = _header(xyz, bb) + body
    f = tmp_path / "blankArzuaH.xyz"
    f.write_text(text, newline="")
    ref = O.ref_read_xyz(f, len(xyz) + 4)
    got = O.xyz_parse(text.encode())
    np.testing.assert_array_equal(got[0], ref[0])


@pytest.mark.parametrize("header", [True, False])
def test_host_loader_equals_oracle(owm, tmp_path, header):
    xyz, bb = _cloud(11 + header, 2000)
    text = (_header(xyz, bb) if header else "") + _fmt_lines(xyz, "%.17g", "\t5")
    f = tmp_path / "c.xyz"
    f.write_text(text)
    pts, hb = owm.read_xyz(f)
    want = O.xyz_parse(text.encode())
    np.testing.assert_array_equal(pts, want[0])
    assert (hb.min_x, hb.min_y, hb.max_x, hb.max_y) == want[1]


MALFORMED = [
    b"",                                 # empty
    b"\n\n",                             # blank only
    b"1 2\n",                            # two numbers
    b"5\n0\n1\n0\n1\n1 2 3\n",           # short file
    b"2\n0\n1\n0\n1\n1 2 3\nbad\n9 9 9\n",  # error before the declared count
    b"1 2 3\n4 5 inf\n",                 # non-finite
    b"1 2 3\n4 5 nan\n",
    b"1 2 3\n4 5 1e400\n",               # overflow
    b"3\n0\n1\n0\n",                     # truncated header
]
ACCEPTED = [
    b"1\n0\n1\n0\n1\n1 2 3\nthis line is never read\n",
    b"1 2 3",                             # no trailing newline
    b"1e+ 2 3\n",                         # sscanf takes the dangling exponent
    b"0x1p3 0X.8P1 -0x1.8p-1\n",
    b"1.-2.5e1+4\n",                      # numbers need no separators
    b"  \t1 2 3  \r\n\n \t \n4 5 6",
    b"1 2 3\x00garbage\n4 5 6\n",         # a NUL ends what sscanf sees
    b"00012 -0 +0.\n",
    b"2.4703282292062328e-324 1e-400 4.9406564584124654e-324\n",
]


@pytest.mark.parametrize("text", MALFORMED + ACCEPTED)
def test_host_loader_verdicts_match_oracle(owm, tmp_path, text):
    f = tmp_path / "m.xyz"
    f.write_bytes(text)
    want = O.xyz_parse(text)
    if want is None:
        with pytest.raises(owm.OwmError):
            owm.read_xyz(f)
        assert text in MALFORMED
    else:
        pts, hb = owm.read_xyz(f)
        np.testing.assert_array_equal(pts, want[0])
        assert text in ACCEPTED


def test_check_results_equals_reference(tmp_path, owm):
    """owm_check_results against the reference's own check_results
    (optim3_func.cpp:725-794, compiled into oracle/_ref) on seeded gold/output
    pairs: gold files in the reference's dump format ("%.2f"), outputs that
    drop seeds, add non-seed points, repeat ids and hold the sentinel id 0."""
    if not O.ref_available():
        pytest.skip("reference sources not present")
    spec, W, Ov, B, _, seed = O.synth_config(1)
    spec.n = 60_000
    spec.x1, spec.y1 = spec.x0 + 60.0, spec.y0 + 50.0
    xyz, bb = O.synth_cloud(spec, seed)
    seeds, _ = O.run(xyz, bb, W, Ov, B)
    p = O.params(bb, spec.n, W, Ov, B)
    rng = np.random.default_rng(3)
    cases = [
        (seeds, seeds),  # identical
        (seeds, rng.choice(seeds, size=len(seeds) // 2, replace=False)),  # half the seeds
        (seeds, np.concatenate([seeds, rng.integers(1, spec.n + 1, 40)])),  # plus random points
        (seeds[: len(seeds) // 3], np.concatenate([[0], seeds, [0]])),  # sentinel ids, gold a third
        (rng.integers(1, spec.n + 1, 200), np.concatenate([seeds[:50], seeds[:50]])),  # repeats
    ]
    for k, (gold_ids, out_ids) in enumerate(cases):
        gold_file = tmp_path / f"gold{k}.xyz"
        owm.write_xyz_ids(gold_file, xyz, gold_ids)
        gold = np.loadtxt(gold_file, ndmin=2)
        for displace in (float(p.displace), 1.0, 0.25):
            want = O.ref_check_results(gold_file, xyz, out_ids, displace)
            got = owm.check_results(gold, xyz, out_ids, displace)
            assert got == want, (k, displace, got, want)


def test_check_results_sentinel_matches_like_reference(tmp_path, owm):
    """Id 0 is the reference's sentinel {0, 0, DBL_MAX}: it matches a gold
    point only when the gold list holds that sentinel too."""
    if not O.ref_available():
        pytest.skip("reference sources not present")
    xyz = np.array([[10.0, 20.0, 1.0], [30.0, 40.0, 2.0]])
    gold_file = tmp_path / "goldS.xyz"
    gold_file.write_text("0 0 1.7976931348623157e308\n10 20 1\n")
    gold = np.loadtxt(gold_file, ndmin=2)
    for ids in ([0], [0, 1], [1, 2], [2]):
        want = O.ref_check_results(gold_file, xyz, ids, 1.0)
        assert owm.check_results(gold, xyz, ids, 1.0) == want, ids
    assert owm.check_results(gold, xyz, [0, 1], 1.0) == 100.0
