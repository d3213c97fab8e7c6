"""The reference's in-code consistency checks, restated on the oracle.

- hand-unrolled TIP4P kernel vs StdForce (TIP4PConst.F90:4-18 makes them agree)
- finite-difference forces/torques on a small periodic box
- energy of a molecule against all others equals its pair sum (mc2.F90:489-505)
- cell ids follow Address_Assign, and the grid never changes the pair set
"""
import numpy as np
import pytest

from genesis6_gb300 import config


def _box(model, n, seed, jitter=0.3):
    return config.water_box(model, n, seed, jitter=jitter)


def test_tip4p_hand_kernel_equals_std(orc):
    b = _box("TIP4P", 216, 1)
    a = orc.compute("TIP4P", "custom", b["com"], b["quat"], b["L"], [8.5] * 3, 6.5, 8.5)
    s = orc.compute("TIP4P", "std", b["com"], b["quat"], b["L"], [8.5] * 3, 6.5, 8.5)
    assert a[2] == pytest.approx(s[2], rel=1e-13)
    assert np.abs(a[0] - s[0]).max() <= 1e-11 * np.abs(a[0]).max()
    assert np.abs(a[3] - s[3]).max() <= 1e-11 * np.abs(a[3]).max()


@pytest.mark.parametrize("model,path", [("TIP4P", "custom"), ("TIP5P", "std"), ("ST2", "custom"), ("ST2", "std")])
def test_finite_difference_forces(orc, model, path):
    b = _box(model, 64, 3)
    L = b["L"]; rc = 0.49 * L[0]; rin = rc - 2.0
    com, quat = b["com"], b["quat"]
    F, tau, E, vir, _ = orc.compute(model, path, com, quat, L, [rc] * 3, rin, rc)
    rng = np.random.default_rng(0)
    h = 1e-5
    for i in rng.choice(len(com), 4, replace=False):
        for k in range(3):
            cp = com.copy(); cp[i, k] += h
            cm = com.copy(); cm[i, k] -= h
            fd = -(orc.compute(model, path, cp, quat, L, [rc] * 3, rin, rc)[2] -
                   orc.compute(model, path, cm, quat, L, [rc] * 3, rin, rc)[2]) / (2 * h)
            assert fd == pytest.approx(F[i, k], rel=1e-5, abs=1e-4 * np.abs(F).max())


def test_molecule_energy_sums_to_total(orc):
    b = _box("ST2", 128, 5)
    L = b["L"]; rc = 0.5 * L[0]; rin = rc - 2.0
    _, _, E, _, _ = orc.compute("ST2", "custom", b["com"], b["quat"], L, [rc] * 3, rin, rc)
    e = [orc.molecule_energy("ST2", "custom", b["com"], b["quat"], t, b["com"][t], b["quat"][t], L, rin, rc)
         for t in range(len(b["com"]))]
    assert 0.5 * sum(e) == pytest.approx(E, rel=1e-12)


def test_cells_follow_address_assign(orc):
    b = _box("TIP4P", 512, 9, jitter=2.0)
    L = b["L"]
    ndiv, cell, _, _ = orc.grid(L, [8.5] * 3)
    cid, _ = orc.pairsearch(b["com"], L, [8.5] * 3, 6.5, 8.5)
    d = b["com"] - np.round(b["com"] / L) * L
    j = np.floor(np.abs(d / cell) + 0.5) * np.sign(d)
    j = np.where(j < 0, j + ndiv, j).astype(int)
    j = np.where(j >= ndiv, j - ndiv, j)
    want = (j[:, 2] * ndiv[1] + j[:, 1]) * ndiv[0] + j[:, 0]
    assert np.array_equal(cid, want)


def test_grid_does_not_change_pairset(orc):
    b = _box("TIP4P", 343, 11, jitter=1.0)
    L = b["L"]
    sets = []
    for req in (8.5, 4.0, 20.0):
        _, p = orc.pairsearch(b["com"], L, [req] * 3, 6.5, 8.5)
        sets.append(sorted(zip(np.minimum(p["i"], p["j"]), np.maximum(p["i"], p["j"]))))
    # req = 8.5 and req >= L/2 (one cell) are complete; both must agree
    assert sets[0] == sets[2]


def test_homo_stencil_counts(orc):
    for nd, want in [(5, (13, 1)), (3, (13, 1)), (2, (0, 8)), (1, (0, 1))]:
        ndiv, _, n, n0 = orc.grid([nd * 10.0] * 3, [10.0] * 3)
        assert tuple(ndiv) == (nd, nd, nd)
        assert (len(n), len(n0)) == want


def test_md_conserves_energy(orc):
    b = config.water_box("TIP4P", 125, 2, temp=300.0, dt=0.001)
    L = b["L"]
    rec, th, log = orc.md_run("TIP4P", "custom", b["rec"], L, [L[0] / 2] * 3, 0.5 * L[0] - 2.0, 0.5 * L[0] - 0.01,
                              0.001, 60, np.zeros(10))
    H = log[10:, 5]
    assert np.isfinite(H).all()
    assert np.ptp(H) < 2e-3 * np.abs(log[10:, 1] + log[10:, 2]).mean() * 10.0
