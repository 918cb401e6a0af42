"""The CPU oracle: pinned to the reference's own solver, and self-consistent."""
import json
import os

import numpy as np
import pytest

import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _pins():
    meta = json.load(open(os.path.join(GOLDEN, "reference_pins.json")))
    data = np.load(os.path.join(GOLDEN, "reference_pins.npz"))
    return meta["cases"], data


def _case_arrays(data, c):
    name = c["name"]
    dp = data[f"{name}__dp"].astype(np.int32)
    dn = data[f"{name}__dn"].astype(np.int32)
    kw = {"penalty": c["penalty"]}
    if c["arrays"]:
        for k in ("up", "down", "left", "right"):
            kw[k] = data[f"{name}__{k}"].astype(np.int32)
    n = c["W"] * c["H"]
    labels = np.unpackbits(data[f"{name}__ref_labels"])[:n].reshape(c["H"], c["W"])
    return dp, dn, kw, labels


CASES, DATA = _pins()


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
@pytest.mark.parametrize("solver", ["pr", "bk"])
def test_oracle_matches_reference_pins(case, solver):
    """Oracle labels == the reference's GC_Optimize labels (S_max, border 0),
    and the reference's printed energy is reproduced exactly."""
    dp, dn, kw, ref_labels = _case_arrays(DATA, case)
    r = O.solve(dp, dn, solver=solver, **kw)
    assert np.array_equal(r["smax"], ref_labels)
    assert O.reference_energy(dp, r["excess"]) == case["ref_energy"]
    assert r["flow"] == case["oracle_flow"]
    # max-flow == min-cut energy for both canonical cuts, S_min within S_max
    assert O.cut_energy(r["smax"], dp, dn, **kw) == r["flow"]
    assert O.cut_energy(r["smin"], dp, dn, **kw) == r["flow"]
    assert not np.any(r["smin"] & ~r["smax"])


def test_all_pins_agree_with_reference():
    assert all(c["oracle_agrees"] for c in CASES)
    assert len(CASES) >= 25


@pytest.mark.parametrize("seed", range(6))
def test_solvers_agree_random(seed):
    rng = np.random.default_rng(100 + seed)
    for _ in range(40):
        H, W = (int(v) for v in rng.integers(3, 24, 2))
        dp = rng.integers(0, 300, (H, W)).astype(np.int32)
        dn = rng.integers(0, 300, (H, W)).astype(np.int32)
        if rng.random() < 0.5:
            kw = {k: rng.integers(0, 120, (H, W)).astype(np.int32) for k in ("up", "down", "left", "right")}
        else:
            kw = {"penalty": int(rng.integers(0, 150))}
        a = O.solve(dp, dn, solver="pr", **kw)
        b = O.solve(dp, dn, solver="bk", **kw)
        assert a["flow"] == b["flow"]
        assert np.array_equal(a["smin"], b["smin"]) and np.array_equal(a["smax"], b["smax"])


def test_generator_is_pinned():
    """The cfg-0 image (256x256, seed 0) is byte-identical everywhere."""
    rgb, scrib = O.generate(0, 256, 256, 0)
    assert O.fnv1a(rgb) == 0xEB03D0172E0C83E2
    assert int((scrib == 1).sum()) == 400 and int((scrib == 2).sum()) == 9840


def test_det_math():
    xs = np.linspace(1e-6, 1.0, 1001)
    import synth
    assert max(abs(synth.lib().gs_det_log(float(x)) - np.log(x)) for x in xs) < 1e-13
    ts = np.linspace(-7, 7, 1001)
    assert max(abs(synth.lib().gs_det_cos(float(t)) - np.cos(t)) for t in ts) < 1e-13


def test_cfg0_pipeline_solvers_agree():
    rgb, scrib = O.generate(0, 256, 256, 0)
    a = O.segment(rgb, scrib, 50.0, solver="pr")
    b = O.segment(rgb, scrib, 50.0, solver="bk")
    assert a["flow"] == b["flow"]
    assert np.array_equal(a["smax"], b["smax"]) and np.array_equal(a["smin"], b["smin"])
