"""The oracle's GJK/EPA against the reference's own known answers (tests/gjk, tests/epa)."""
import json
import math
import os

import numpy as np
import pytest

import pyoracle

HERE = os.path.dirname(os.path.abspath(__file__))
KA = json.load(open(os.path.join(HERE, "golden", "known_answers.json")))
TOL = KA["tolerances"]


def moved(spec, off):
    spec = json.loads(json.dumps(spec))
    if spec[0] == "aabb":
        spec[1] = [a + b for a, b in zip(spec[1], off)]
        spec[2] = [a + b for a, b in zip(spec[2], off)]
    elif spec[0] == "obb":
        spec[1] = [a + b for a, b in zip(spec[1], off)]
    else:
        spec[2] = [a + b for a, b in zip(spec[2], off)]
    return spec


@pytest.fixture(scope="module")
def world():
    w = pyoracle.OracleWorld()
    yield w
    w.close()


@pytest.mark.parametrize("case", KA["gjk"], ids=[c["src"].split("/")[-1] for c in KA["gjk"]])
def test_gjk_boolean(world, case):
    r = world.gjk_epa(case["a"], case["b"])
    assert (r is not None) == case["hit"]
    if case["both_orders"]:
        r2 = world.gjk_epa(case["b"], case["a"])
        assert (r2 is not None) == case["hit"]


def check_unit(n):
    assert abs(np.linalg.norm(n) - 1.0) < TOL["unit_normal"]


@pytest.mark.parametrize("case", KA["epa"], ids=[c["src"].split("/")[-1] for c in KA["epa"]])
def test_epa_known_answer(world, case):
    r = world.gjk_epa(case["a"], case["b"])
    assert r is not None
    check_unit(r["normal"])
    if case["depth"] is not None:
        assert abs(r["depth"] - case["depth"]) <= case["tol"], r["depth"]
    if case["positive"]:
        assert r["depth"] > 0.0
    if case["axis"] is not None:
        ax = case["axis"]
        assert abs(r["normal"][ax]) > (0.8 if case["a"][0] == "mesh" and case["a"][1][0] == "sphere" else 0.9)
        for k in range(3):
            if k != ax and case["a"][0] != "mesh":
                assert abs(r["normal"][k]) < 0.1
    if case["mtv"]:
        off = r["normal"] * (r["depth"] + TOL["mtv_nudge"])
        assert world.gjk_epa(moved(case["a"], off), case["b"]) is None
    if case["sym_depth_tol"] is not None or case["normal_sum_max"] is not None or case["both_depth"]:
        r2 = world.gjk_epa(case["b"], case["a"])
        assert r2 is not None
        if case["sym_depth_tol"] is not None:
            assert abs(r["depth"] - r2["depth"]) <= case["sym_depth_tol"]
        if case["normal_sum_max"] is not None:
            assert np.linalg.norm(r["normal"] + r2["normal"]) < case["normal_sum_max"]
        if case["both_depth"]:
            assert abs(r2["depth"] - case["depth"]) <= case["tol"]


def test_epa_depth_always_positive(world):
    for case in KA["epa_positive"]:
        r = world.gjk_epa(case["a"], case["b"])
        if r is not None:
            assert r["depth"] > 0.0
            check_unit(r["normal"])
