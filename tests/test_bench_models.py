"""The bench's byte models and its reading of the committed ncu summaries, on CPU.

`roofline.achieved` divides a kernel's algorithmic bytes by its measured time,
`path_roofline` divides the whole step's lower-bound bytes by the step time,
and `roofline.traffic` scales the DRAM bytes per point of a committed ncu
summary; these tests pin the figures those numbers rest on.
"""
import re
import sys
from pathlib import Path
from types import SimpleNamespace

import pytest

pytest.importorskip("torch")
ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
import bench  # noqa: E402


def test_path_model_is_154_bytes_a_point_40_a_window_8_a_cell():
    p = SimpleNamespace(ncells=705_600, ngrid=10_201)
    assert bench.path_bytes(100_000_000, p) == 154.0 * 100_000_000 + 40.0 * 705_600 + 8.0 * 10_201
    assert bench.path_bytes(0, SimpleNamespace(ncells=0, ngrid=0)) == 0.0


def test_kernel_models():
    p = SimpleNamespace(ncells=705_600, ngrid=10_201)
    n, leaves = 100_000_000, 390_625
    # the whole-step model's permute step (56 B/pt) and 48 B per leaf node
    assert bench.kernel_bytes("k_gather_leaves", n, p, leaves) == 56.0 * n + 48.0 * leaves
    assert bench.kernel_bytes("k_gather_leaves<256, 1, 4>", n, p, leaves) == 56.0 * n + 48.0 * leaves
    assert bench.kernel_bytes("k_rs_downsweep", n, p, leaves) == 16.0 * n
    assert bench.kernel_bytes("k_morton", n, p, leaves) == 28.0 * n
    assert bench.kernel_bytes("k_query_s1", n, p, leaves) == 24.0 * n + 48.0 * leaves + 8.0 * p.ncells
    assert bench.kernel_bytes("k_refit", n, p, leaves) is None


def test_measured_traffic_reads_the_committed_summary():
    """The gather's DRAM bytes per point come from its committed ncu summary,
    scaled by the points of the workload."""
    summaries = sorted((ROOT / "profiles").glob("k_gather_leaves_*_dram.md"))
    assert summaries, "the gather's DRAM summary is committed"
    lines = [ln for ln in summaries[0].read_text().splitlines() if ln.startswith("traffic_bytes_per_point:")]
    assert len(lines) == 1
    per_point = float(lines[0].split(":", 1)[1])
    assert 28.0 < per_point < 200.0  # at least the kernel's own algorithmic bytes, far below a re-read per window
    assert bench.measured_traffic("k_gather_leaves", 1_000_000) == pytest.approx(per_point * 1_000_000)
    assert bench.measured_traffic("k_no_such_kernel", 1_000_000) is None


def test_committed_profiles_run_committed_files_only():
    """Every command line in a committed summary runs committed files (bench.py
    and the ncu CLI), never a working script."""
    for f in (ROOT / "profiles").glob("*.md"):
        text = f.read_text()
        assert "_work/" not in text, f.name
        for cmd in re.findall(r"^\s+(python\s+\S+)", text, flags=re.M):
            script = cmd.split()[1]
            if script.endswith(".py"):
                assert (ROOT / script).exists(), (f.name, script)


def test_summary_keeps_the_headline_figures():
    line = {"value": 23000.0, "ms_per_step": 4.3, "serial": {"value": 22500.0},
            "e2e": {"value": 8300.0}, "path_roofline": {"frac": 0.52},
            "roofline": {"kernel": "k_gather_leaves", "frac": 0.36}, "cpu_baseline": {"value": 35.0},
            "batched": {"batched_mpts": 18900.0, "speedup": 9.1, "seeds_equal": True},
            "served": {"saturation_mpts": 7300.0, "saturation_vs_plain": 3.7,
                       "sweep": [{"lambda_tiles_s": 50, "p50_ms": 0.37, "p99_ms": 1.2}]}}
    s = bench.summary(line)
    assert s["value"] == 23000.0 and s["e2e"] == 8300.0 and s["path_roofline_frac"] == 0.52
    assert s["dominant_kernel"] == "k_gather_leaves" and s["kernel_frac"] == 0.36
    assert s["batched"]["speedup"] == 9.1 and s["batched"]["seeds_equal"] is True
    assert s["served"]["p50_p99_ms_by_lambda"] == {"50": [0.37, 1.2]}
