"""Pin the CPU oracle against independently computed golden vectors.

tests/golden/dimers.json holds dimer energies (closed form) and forces/torques
(finite differences) written without the oracle; tests/golden/pairset_small.json
holds an O(N^2) minimum-image pair set.
"""
import json
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _dimers():
    with open(os.path.join(GOLD, "dimers.json")) as f:
        return json.load(f)


@pytest.mark.parametrize("case", _dimers(), ids=lambda c: "%s-%s-%s" % (c["model"], c["path"], c["name"]))
def test_dimer_energy_force_torque(orc, case):
    com = np.array(case["com"]); quat = np.array(case["quat"]); L = np.array(case["L"])
    F, tau, E, vir, npair = orc.compute(case["model"], case["path"], com, quat, L, [case["rc"]] * 3, case["rin"],
                                        case["rc"])
    # energy: closed form, FP64 rounding only
    assert E == pytest.approx(case["E"], rel=1e-12, abs=1e-9)
    Fg = np.array(case["F"]); tg = np.array(case["tau"])
    scale = max(1.0, np.abs(Fg).max())
    # forces/torques: 4th-order finite differences (h = 1e-4) are good to ~1e-8 relative
    assert np.abs(F - Fg).max() <= 2e-7 * scale
    assert np.abs(tau - tg).max() <= 2e-7 * max(1.0, np.abs(tg).max())
    if case["name"] == "outside":
        assert npair == 0 and E == 0.0
    else:
        assert npair == 1
        # Newton's third law on the COM forces
        assert np.abs(F[0] + F[1]).max() <= 1e-9 * scale


def test_pairset_matches_bruteforce(orc):
    with open(os.path.join(GOLD, "pairset_small.json")) as f:
        g = json.load(f)
    com = np.array(g["com"])
    for req in (g["rc"], 0.5 * g["rc"], 3.0 * g["rc"]):   # ndiv = many, large, 1
        cell, p = orc.pairsearch(com, g["L"], [req] * 3, g["rin"], g["rc"])
        got = sorted((min(a, b), max(a, b)) for a, b in zip(p["i"], p["j"]))
        want = sorted(tuple(x) for x in g["pairs"])
        if req >= g["rc"]:
            assert got == want
        assert len(set(got)) == len(got)
