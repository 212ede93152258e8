"""Generates tests/golden/owm_golden.json from the reference's own CPU path.

The reference (CPP-TBB-CPU/src/optim3_func.cpp, exact stage1 = the o3memoB
build) is compiled in place from its sources by oracle/Makefile and run on
seeded synthetic clouds made by this project's generator
(owm_synth_cloud, bit-identical on x86-64 and aarch64).  Each case stores:

  * the cloud recipe (generator spec + seed, or the points themselves for
    tiny clouds) and the SHA-256 of the generated coordinates,
  * the OWM knobs, and the reference's outputs: window minima (stage 1, in
    step order), LLPs (stage 2), stage-3 ids,
  * for clouds with z ties, also the (z, id)-tie restatement's outputs,
    which are the parity target there (the reference keeps the first
    minimum its tree visits).

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import base64
import hashlib
import json
import sys
import zlib
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import fastowm_gb300 as F  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent / "owm_golden.json"


def pack(a) -> str:
    a = np.asarray(a, dtype=np.int64)
    return base64.b64encode(zlib.compress(a.tobytes(), 9)).decode()


def spec_case(name, config, n=None, w=None, h=None, W=None, Ov=None, B=None, mn=None, policy=1, tile=0, **extra):
    spec, W0, O0, B0, mn0, seed = F.synth_config(config, tile)
    if n is not None:
        spec.n = n
    if w is not None:
        spec.x1 = spec.x0 + w
    if h is not None:
        spec.y1 = spec.y0 + h
    for k, v in extra.items():
        setattr(spec, k, v)
    xyz, bb = F.synth_cloud(spec, seed)
    fields = {f: getattr(spec, f) for f, _ in spec._fields_ if f != "_pad"}
    recipe = {"config": config, "tile": tile, "seed": seed, "spec": fields}
    return name, recipe, xyz, bb, W or W0, Ov if Ov is not None else O0, B if B is not None else B0, mn or mn0, policy


def explicit_case(name, xyz, W, Ov, B, mn=4):
    bb = F.bbox_of(xyz)
    return name, {"points": xyz.tolist()}, np.ascontiguousarray(xyz), bb, W, Ov, B, mn, 1


def run_case(name, recipe, xyz, bb, W, Ov, B, mn, policy):
    digest = hashlib.sha256(np.ascontiguousarray(xyz).tobytes()).hexdigest()
    ties = np.unique(xyz[:, 2]).size < xyz.shape[0]
    case = {"name": name, "recipe": recipe, "sha256": digest, "n": int(xyz.shape[0]), "bbox": list(bb.astuple()),
            "wsize": W, "overlap": Ov, "bsize": B, "max_number": mn, "policy": policy, "ties": bool(ties)}
    p = O.params(bb, xyz.shape[0], W, Ov, B)
    # restatement
    win_r = O.stage1(xyz, p)
    llp_r = O.stage2(win_r, Ov)
    s3_r = O.stage3(xyz, p, llp_r)
    case["restated"] = {"win_min": pack(win_r), "llp": pack(llp_r), "stage3": pack(s3_r)}
    if Ov > 0.0:  # the reference's overlap-0 branch leaves -1 inside the LLP prefix (owm_optim3.cpp:185-188)
        seeds, nllp, win, res = O.ref_run(xyz, bb, W, Ov, B, policy=policy, max_number=mn, nthreads=1)
        llp = np.sort(seeds[len(seeds) - nllp:])
        s3 = seeds[: len(seeds) - nllp]
        case["reference"] = {"win_min": pack(win), "llp": pack(llp), "stage3": pack(s3),  # cell order (1 thread)
                             "n_llp": int(nllp), "n_stage3": int(len(s3)),
                             "min_num_points": int(res.min_num_points)}
        same = np.array_equal(win, win_r) and np.array_equal(llp, llp_r) and np.array_equal(s3, s3_r)
        case["reference_equals_restatement"] = bool(same)
        print(f"{name:>14}: n={xyz.shape[0]} windows={p.ncells} llp={nllp} s3={len(s3)} ties={ties} "
              f"reference==restatement: {same}")
    else:
        print(f"{name:>14}: n={xyz.shape[0]} overlap 0: restatement only")
    return case


def main():
    if not O.ref_available():
        raise SystemExit("reference sources not found: set OWM_REFERENCE")
    rng = np.random.default_rng(20240601)
    cases = [
        spec_case("c1_full", 1),
        spec_case("c1_minradius", 1, n=300_000, w=100, h=150, policy=0),
        spec_case("c1_odd_w_b", 1, n=200_000, w=90, h=110, W=9, B=15),
        spec_case("c1_w7_o03", 1, n=150_000, w=80, h=60, W=7, Ov=0.3, B=11),
        spec_case("c1_overlap0", 1, n=100_000, w=60, h=70, Ov=0.0),
        spec_case("c2_sample", 2, n=2_000_000, w=283, h=283),
        spec_case("c3_o05", 3, n=1_000_000, w=320, h=320, Ov=0.5),
        spec_case("c3_o08", 3, n=1_000_000, w=320, h=320, Ov=0.8),
        spec_case("c4_tile0", 4, tile=0),
        spec_case("c4_tile7", 4, tile=7),
        spec_case("sparse", 1, n=400, w=300, h=300),
        explicit_case("tiny5", np.column_stack([1000 + rng.random(5) * 7, 2000 + rng.random(5) * 5,
                                                50 + rng.random(5)]), 10, 0.8, 20),
        explicit_case("tiny40", np.column_stack([-20 + rng.random(40) * 40, -15 + rng.random(40) * 30,
                                                 np.round(rng.random(40), 1)]), 4, 0.5, 3),
    ]
    out = {"generator": "owm_synth_cloud (fastowm_gb300/csrc/owm_host.cpp)",
           "reference": "CPP-TBB-CPU/src/optim3_func.cpp via oracle/ref_runner.cpp, exact stage1, 1 thread",
           "cases": [run_case(*c) for c in cases]}
    OUT.write_text(json.dumps(out, indent=1))
    print("wrote", OUT, OUT.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
