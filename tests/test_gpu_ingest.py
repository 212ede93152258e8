"""GPU parity of the device cloud ingest (owm_cloud_parse_xyz /
owm_cloud_load_xyz) against the cloud-text oracle (oracle_xyz_parse: the C
library's sscanf conversions under readXYZfile's rules, pinned on the
reference's own loader by tests/test_ingest_oracle.py).

The bar is bit-exact doubles, the same point count and bbox, and the same
verdict (OWM_EIO exactly where the oracle fails).
"""
import math
import random
import struct
from decimal import Decimal, getcontext
from fractions import Fraction

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _same(owm, ctx, text: bytes):
    want = O.xyz_parse(text)
    if want is None:
        with pytest.raises(owm.OwmError) as e:
            ctx.cloud_parse_xyz(text)
        assert e.value.status == -5
        return None
    c = ctx.cloud_parse_xyz(text)
    got = c.points()
    bb = (c.bbox.min_x, c.bbox.min_y, c.bbox.max_x, c.bbox.max_y)
    c.close()
    assert got.shape == want[0].shape
    # bit-exact, signed zeros included
    np.testing.assert_array_equal(got.view(np.uint64), want[0].view(np.uint64))
    assert bb == want[1]
    return got


def _cloud_text(owm, config, n, fmt, header, extra=""):
    spec, *_ , seed = owm.synth_config(config)
    spec.n = n
    xyz, bb = owm.synth_cloud(spec, seed)
    head = f"{n}\n{bb.min_x!r}\n{bb.max_x!r}\n{bb.min_y!r}\n{bb.max_y!r}\n" if header else ""
    return xyz, (head + "".join(f"{fmt % x} {fmt % y} {fmt % z}{extra}\n" for x, y, z in xyz)).encode()


@pytest.mark.parametrize("fmt,header", [("%.3f", True), ("%.6f", False), ("%.17g", True), ("%.9e", False),
                                        ("%.20g", False)])
def test_lidar_text_equals_oracle(owm, ctx, fmt, header):
    _, text = _cloud_text(owm, 1, 60_000, fmt, header, " 1 0 2")
    _same(owm, ctx, text)


def test_full_precision_text_round_trips(owm, ctx):
    xyz, text = _cloud_text(owm, 1, 200_000, "%.17g", True)
    got = _same(owm, ctx, text)
    np.testing.assert_array_equal(got, xyz)  # 17 digits give the doubles back


def _bits(d):
    return struct.unpack("<Q", struct.pack("<d", d))[0]


def _from_bits(b):
    return struct.unpack("<d", struct.pack("<Q", b))[0]


def _exact_decimal(fr: Fraction) -> str:
    """Exact decimal string of a dyadic fraction."""
    getcontext().prec = 2000
    s = format(Decimal(fr.numerator) / Decimal(fr.denominator), "f")
    return s.rstrip("0").rstrip(".") if "." in s else s


def _hard_numbers(seed, count):
    rng = random.Random(seed)
    out = []
    for _ in range(count):
        kind = rng.randrange(6)
        if kind <= 2:  # halfway points between neighbouring doubles, and just off them
            e = rng.choice([rng.randrange(1, 2046), rng.randrange(0, 3), rng.randrange(2000, 2046)])
            b = (e << 52) | rng.getrandbits(52)
            d = _from_bits(b)
            nxt = _from_bits(b + 1)
            if math.isinf(nxt):
                continue
            mid = (Fraction(d) + Fraction(nxt)) / 2
            s = _exact_decimal(mid)
            if kind == 1:
                s = s + "1" if "." in s else s + ".1"  # just above
            elif kind == 2:
                digits = s.replace(".", "")
                cut = rng.randrange(15, min(40, len(digits)) + 1) if len(digits) > 15 else len(digits)
                dot = s.find(".")
                s = s[: cut + (1 if 0 <= dot < cut else 0)]  # truncated: just below
                if s.endswith("."):
                    s = s[:-1]
            out.append(s)
        elif kind == 3:  # long random significands, any exponent
            nd = rng.randrange(17, 60)
            digits = "".join(rng.choice("0123456789") for _ in range(nd)).lstrip("0") or "7"
            p = rng.randrange(0, len(digits) + 1)
            out.append(f"{digits[:p]}.{digits[p:]}e{rng.randrange(-340, 300)}")
        elif kind == 4:  # hex floats, more digits than a double holds
            m = "".join(rng.choice("0123456789abcdef") for _ in range(rng.randrange(1, 22)))
            p = rng.randrange(0, len(m) + 1)
            out.append(f"0x{m[:p]}.{m[p:]}p{rng.randrange(-1090, 1000)}")
        else:  # subnormals and the extremes
            out.append(rng.choice(["4.9406564584124654e-324", "2.4703282292062328e-324", "2.4703282292062327e-324",
                                   "1.7976931348623157e308", "1.7976931348623158e308", "2.2250738585072011e-308",
                                   "2.2250738585072014e-308", "0.000000000000000000000000000000001", "9007199254740993",
                                   "123456789012345678901234567890", "1e-400", "-0.0", "1e22", "1e23"]))
    # keep every value finite (an infinity fails the whole load)
    return [s for s in out if math.isfinite(_py_float(s))]


def _py_float(s: str) -> float:
    if "x" not in s:
        return float(s)
    try:
        return float.fromhex(s)
    except OverflowError:
        return math.inf


def test_hard_numbers_equal_oracle(owm, ctx):
    nums = _hard_numbers(1, 30_000)
    lines = [" ".join(nums[i : i + 3]) for i in range(0, len(nums) - 2, 3)]
    text = ("\n".join(lines) + "\n").encode()
    got = _same(owm, ctx, text)
    assert got is not None and got.shape[0] == len(lines)


def test_numbers_match_python_conversion(owm, ctx):
    # an independent check of the oracle itself: Python's float() and
    # float.fromhex() are correctly rounded too
    nums = _hard_numbers(2, 6000)
    lines = [" ".join(nums[i : i + 3]) for i in range(0, len(nums) - 2, 3)]
    got = _same(owm, ctx, ("\n".join(lines) + "\n").encode())
    want = np.array([[_py_float(t) for t in ln.split()] for ln in lines])
    np.testing.assert_array_equal(got.view(np.uint64), want.view(np.uint64))


EDGE = [
    b"", b"\n\n", b"1 2\n", b"5\n0\n1\n0\n1\n1 2 3\n", b"2\n0\n1\n0\n1\n1 2 3\nbad\n9 9 9\n", b"1 2 3\n4 5 inf\n",
    b"1 2 3\n4 5 nan\n", b"1 2 3\n4 5 1e400\n", b"3\n0\n1\n0\n", b"1\n0\n1\n0\n1\n1 2 3\nthis line is never read\n",
    b"1 2 3", b"1e+ 2 3\n", b"0x1p3 0X.8P1 -0x1.8p-1\n", b"1.-2.5e1+4\n", b"  \t1 2 3  \r\n\n \t \n4 5 6",
    b"1 2 3\x00garbage\n4 5 6\n", b"00012 -0 +0.\n", b"2.4703282292062328e-324 1e-400 4.9406564584124654e-324\n",
    b"0xg 1 2\n", b"0x. 1 2\n", b"1ex 2 3\n", b".5 .5 .5\n", b". 1 2\n", b"+-1 2 3\n", b"1..2 3 4\n",
    b"\v1 2 3\n", b"1 2 3\n\v\n", b"1 2 3\ninfinit 1 2\n", b"1,2 3 4\n", b"1 2 3\n" + b" " * 70000 + b"\n4 5 6\n",
    b"1 2 " + b"0" * 5000 + b"3\n",
]


@pytest.mark.parametrize("k", range(len(EDGE)))
def test_edge_texts_match_oracle(owm, ctx, k):
    _same(owm, ctx, EDGE[k])


def test_load_file_equals_parse_and_host_loader(owm, ctx, tmp_path):
    xyz, text = _cloud_text(owm, 1, 300_000, "%.6f", True, " 3")
    f = tmp_path / "c.xyz"
    f.write_bytes(text)
    c = ctx.cloud_load_xyz(f)
    got = c.points()
    hp, hb = owm.read_xyz(f)
    np.testing.assert_array_equal(got, hp)
    assert (c.bbox.min_x, c.bbox.min_y, c.bbox.max_x, c.bbox.max_y) == (hb.min_x, hb.min_y, hb.max_x, hb.max_y)
    c.close()


def test_parsed_cloud_runs_the_path(owm, ctx):
    """A cloud made by the device parser gives the same seeds as one made from
    the same points on the host."""
    xyz, text = _cloud_text(owm, 1, 250_000, "%.17g", False)
    spec, W, Ov, B, mn, seed = owm.synth_config(1)
    a = ctx.cloud_parse_xyz(text)
    b = ctx.cloud(xyz)
    cfg = owm.run_cfg(W, Ov, B, mn)
    np.testing.assert_array_equal(ctx.run(a, cfg), ctx.run(b, cfg))
    a.close()
    b.close()


def test_load_file_larger_than_a_staging_chunk(owm, ctx, tmp_path):
    """A file of several 64 MB staging chunks: the chunked read / copy
    pipeline gives the exact values (the generator's X / 1000.0 etc.)."""
    import importlib.util
    from pathlib import Path

    spec = importlib.util.spec_from_file_location("bench", Path(__file__).resolve().parents[1] / "bench.py")
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    text, pts = bench.lidar_text(2_700_000, 3)  # 84 MB: two chunks
    f = tmp_path / "big.xyz"
    f.write_bytes(text.tobytes())
    assert f.stat().st_size > (64 << 20)
    c = ctx.cloud_load_xyz(f)
    got = c.points()
    c.close()
    np.testing.assert_array_equal(got.view(np.uint64), pts.view(np.uint64))
