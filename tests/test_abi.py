"""CPU tests of the C ABI: the library loads, exports every symbol the header
declares, the host-side entry points (parameters, generator, file I/O)
behave like the reference's, and compute entry points fail loudly without a
GPU (no CPU fallback)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def _declared():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        txt = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(owm_[a-z0-9_]+)\s*\(", txt))
    return names


def test_library_exports_every_declared_symbol(owm):
    lib = owm.lib()
    declared = _declared()
    assert len(declared) >= 30
    missing = [n for n in sorted(declared) if not hasattr(lib, n)]
    assert not missing, missing


def test_bindings_cover_the_header(owm):
    from fastowm_gb300._lib import SIGNATURES

    assert _declared() == set(SIGNATURES)


def test_status_strings(owm):
    lib = owm.lib()
    for s in range(0, -8, -1):
        assert lib.owm_status_string(s)
    assert lib.owm_version() >= 10000


@pytest.mark.parametrize("bbox,n,W,O,B", [
    ((500000.0008, 4700000.0002, 500199.9994, 4700249.9994), 1_000_000, 10, 0.8, 20),
    ((600000.0, 4500000.0, 602000.0, 4502000.0), 100_000_000, 12, 0.8, 20),
    ((700000.01, 4600000.02, 700799.99, 4600799.98), 20_000_000, 10, 0.5, 15),
    ((1.5, 2.5, 90.25, 80.75), 12345, 9, 0.3, 0),
    ((0.0, 0.0, 3000.0, 10.0), 70_000_000, 16, 0.8, 20),   # minNumPoints above 65535 -> ushort wrap
    ((10.0, 10.0, 500.0, 400.0), 5000, 8, 0.0, 20),
])
def test_params_match_oracle(owm, oracle, bbox, n, W, O, B):
    p = owm.params(bbox, n, W, O, B)
    q = oracle.params(bbox, n, W, O, B)
    for f in ("ncols", "nrows", "ncols_grid", "nrows_grid", "min_num_points", "ncells", "ngrid"):
        assert getattr(p, f) == getattr(q, f), f
    for f in ("width", "height", "density", "displace"):
        assert getattr(p, f) == getattr(q, f), f


def test_params_reference_formulas(owm):
    """owm_optim3.cpp:92-132 spelled out for config 1's nominal box."""
    p = owm.params((500000.0, 4700000.0, 500200.0, 4700250.0), 1_000_000, 10, 0.8, 20)
    assert (p.width, p.height) == (200.0, 250.0)
    assert p.density == 20.0
    assert p.min_num_points == 1000          # (uint32)(0.5*20*10*10)
    assert p.displace == 2.0                 # round2d(10*(1-0.8))
    assert (p.ncols, p.nrows) == (107, 132)  # round((200+16)/2)-1, round((250+16)/2)-1
    assert (p.ncols_grid, p.nrows_grid) == (11, 13)


def test_params_reject_bad_input(owm):
    with pytest.raises(owm.OwmError):
        owm.params((0, 0, 10, 10), 100, 10, 1.0, 20)
    with pytest.raises(owm.OwmError):
        owm.params((0, 0, 10, 10), 0, 10, 0.8, 20)
    with pytest.raises(owm.OwmError):
        owm.params((0, 0, 0, 10), 10, 10, 0.8, 20)  # zero width: density undefined


def test_synth_deterministic_and_thread_independent(owm):
    spec, W, Ov, B, mn, seed = owm.synth_config(1)
    spec.n = 50_000
    a, ba = owm.synth_cloud(spec, seed, nthreads=1)
    b, bb = owm.synth_cloud(spec, seed, nthreads=7)
    assert a.tobytes() == b.tobytes()
    assert ba.astuple() == bb.astuple()
    assert np.unique(a[:, 2]).size == spec.n  # tie-free by construction
    assert a[:, 0].min() == ba.min_x and a[:, 1].max() == ba.max_y


def test_oracle_generator_equals_library_generator(owm, oracle):
    """The CPU baseline makes its clouds with the oracle library's copy of the
    generator (oracle_synth_*, the same source compiled separately), so that
    it never loads the GPU library: both give the same bits."""
    for c, t, n in ((1, 0, 120_000), (2, 0, 150_000), (3, 0, 90_000), (4, 11, None), (5, 40, None)):
        s1, *k1 = owm.synth_config(c, t)
        s2, *k2 = oracle.synth_config(c, t)
        assert k1 == k2
        if n:
            s1.n = s2.n = n
        assert s1.n == s2.n and (s1.x0, s1.x1, s1.y0, s1.y1) == (s2.x0, s2.x1, s2.y0, s2.y1)
        a, ba = owm.synth_cloud(s1, k1[-1], nthreads=3)
        b, bb = oracle.synth_cloud(s2, k2[-1], nthreads=5)
        assert a.tobytes() == b.tobytes()
        assert list(bb) == [ba.min_x, ba.min_y, ba.max_x, ba.max_y]


def test_synth_configs(owm):
    for c in (1, 2, 3):
        spec, W, Ov, B, mn, seed = owm.synth_config(c)
        assert seed == c * 1000
    s3 = owm.synth_config(3)[0]
    assert s3.z_quantum == 0.01 and s3.holes == 8 and s3.strips == 1 and s3.tie_free == 0
    sizes = [owm.synth_config(4, t)[0].n for t in range(512)]
    assert 50_000 <= min(sizes) and max(sizes) <= 2_000_000
    assert 1.5e8 < sum(sizes) < 4e8
    ws = {owm.synth_config(4, t)[1] for t in range(512)}
    assert ws == set(range(8, 17))


def test_xyz_read_header_and_plain(owm, tmp_path):
    xyz = np.array([[1.25, 2.5, 3.0], [4.0, 5.0, 6.5], [7.0, 8.0, 9.0]])
    f = tmp_path / "cloudH.xyz"
    f.write_text("3\n1.0\n8.0\n2.0\n9.0\n" + "".join(f"{x} {y} {z} 1 2 3\n" for x, y, z in xyz))
    got, bb = owm.read_xyz(f)
    np.testing.assert_array_equal(got, xyz)
    assert bb.astuple() == (1.0, 2.0, 8.0, 9.0)  # header box, not the data's
    g = tmp_path / "plain.xyz"
    g.write_text("".join(f"{x} {y} {z}\n" for x, y, z in xyz))
    got, bb = owm.read_xyz(g)
    np.testing.assert_array_equal(got, xyz)
    assert bb.astuple() == (1.25, 2.5, 7.0, 8.0)


def test_xyz_read_errors(owm, tmp_path):
    short = tmp_path / "short.xyz"
    short.write_text("5\n0\n1\n0\n1\n0.5 0.5 1\n")
    with pytest.raises(owm.OwmError) as e:
        owm.read_xyz(short)
    assert e.value.status == -5
    bad = tmp_path / "bad.xyz"
    bad.write_text("1 2 3\nnot a number\n")
    with pytest.raises(owm.OwmError):
        owm.read_xyz(bad)
    with pytest.raises(owm.OwmError):
        owm.read_xyz(tmp_path / "missing.xyz")


def test_xyz_write_and_check_results(owm, tmp_path):
    xyz = np.array([[10.0, 20.0, 1.0], [30.0, 40.0, 2.0], [50.0, 60.0, 3.0]])
    out = tmp_path / "seeds.xyz"
    owm.write_xyz_ids(out, xyz, [3, 1])
    assert out.read_text() == "50.00 60.00 3.00\n10.00 20.00 1.00\n"
    gold = np.array([[10.1, 20.1, 1.005], [50.0, 60.0, 3.0]])
    assert owm.check_results(gold, xyz, [1, 3], 1.0) == 100.0
    assert owm.check_results(gold, xyz, [1], 1.0) == 50.0


def test_compute_without_gpu_fails_loudly(owm):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    rc = owm.lib().owm_ctx_create(0, C.byref(h))
    assert rc == -3  # OWM_ECUDA: no CPU fallback
    with pytest.raises(owm.OwmError):
        owm.Context(0)
