"""The oracle's two-component (mixture) path, pinned without the GPU.

- hetero pair search (NeighborCell_ListHetero + Grid_NeighborList +
  Interaction_Compress2, GridModule.F90:557-899): equal to a direct
  minimum-image scan over all (A, B) pairs, image offsets and switch values
  included;
- the site-pair-table force on two components: for one model it is StdForce
  itself (bit-equal to the one-component call); the TIP4P-OPLS methanol hand
  kernel's constants (OPLSMeOHModule.F90:1-7, 1189-1198) give StdForce's
  LB-mixed result to rounding; forces and torques are the derivatives of the
  pair energy (central differences, inside and in the switching zone)."""
import numpy as np
import pytest

from genesis6_gb300 import config


def mixture(na, nb, seed, L=None):
    rng = np.random.default_rng(seed)
    L = L or config.box_edge(na + nb)
    ca = rng.uniform(-0.5 * L, 0.5 * L, (na, 3))
    cb = rng.uniform(-0.5 * L, 0.5 * L, (nb, 3))
    qa = config.random_quaternions(na, rng)
    qb = config.random_quaternions(nb, rng)
    return np.array([L, L, L]), ca, qa, cb, qb


def cutoff(dd, rin, rc):
    if dd <= rin * rin:
        return 1.0, 0.0
    r = np.sqrt(dd)
    c1 = 1.0 / (rin - rc) ** 5
    u, l = r - rc, r - rin
    return c1 * u ** 3 * (10 * l * l - 5 * u * l + u * u), -30.0 * c1 * u * u * l * l / r


@pytest.mark.parametrize("na,nb,L", [(300, 150, None), (40, 30, 17.5), (20, 12, 12.0)])
def test_hetero_pairset_is_the_direct_scan(orc, na, nb, L):
    rc, rin = (8.5, 6.5) if L is None or L > 17.5 else (5.5, 3.5)
    box, ca, _, cb, _ = mixture(na, nb, 3 + na, L)
    _, _, p = orc.pairsearch_hetero(ca, cb, box, [rc] * 3, rin, rc)
    d = ca[:, None, :] - cb[None, :, :]
    o = np.round(d / box) * box                      # dnint: half away from zero, as np.round except ties
    dd = ((d - o) ** 2).sum(-1)
    ii, jj = np.nonzero(dd < rc * rc)
    want = set(zip(ii.tolist(), jj.tolist()))
    got = list(zip(p["i"].tolist(), p["j"].tolist()))
    assert len(got) == len(set(got)) and set(got) == want
    for k, (i, j) in enumerate(got):
        assert np.allclose([p["ox"][k], p["oy"][k], p["oz"][k]], o[i, j], atol=0)
        h, dh = cutoff(dd[i, j], rin, rc)
        assert p["hh"][k] == pytest.approx(h, rel=1e-12, abs=1e-15)
        assert p["dh"][k] == pytest.approx(dh, rel=1e-9, abs=1e-15)


def sites(orc, model, com, quat):
    x, y, z = orc.place_sites(model, com, quat)[:3]
    return x, y, z


def test_one_model_table_is_stdforce(orc):
    box, ca, qa, _, _ = mixture(120, 0, 5)
    _, p = orc.pairsearch(ca, box, [8.5] * 3, 6.5, 8.5)
    x, y, z = sites(orc, "TIP4P", ca, qa)
    f1 = orc.force_sites("TIP4P", "std", x, y, z, p)
    f2 = orc.force_sites_hetero("TIP4P", "TIP4P", "std", x, y, z, 0, 0, p)
    for a, b in zip(f1, f2):
        assert np.array_equal(a, b)


def test_custom_cross_kernel_equals_std_to_rounding(orc):
    box, ca, qa, cb, qb = mixture(200, 100, 7)
    _, _, p = orc.pairsearch_hetero(ca, cb, box, [8.5] * 3, 6.5, 8.5)
    xa, ya, za = sites(orc, "TIP4P", ca, qa)
    xb, yb, zb = sites(orc, "OPLSMEOH", cb, qb)
    x, y, z = np.concatenate([xa, xb]), np.concatenate([ya, yb]), np.concatenate([za, zb])
    s = orc.force_sites_hetero("TIP4P", "OPLSMEOH", "std", x, y, z, 0, len(xa), p)
    c = orc.force_sites_hetero("TIP4P", "OPLSMEOH", "custom", x, y, z, 0, len(xa), p)
    fs = np.abs(np.concatenate(s[:3])).max()
    for a, b in zip(s[:3], c[:3]):
        assert np.abs(a - b).max() <= 1e-12 * fs
    assert np.abs(s[3] - c[3]).max() <= 1e-12 * np.abs(s[3]).max()


@pytest.mark.parametrize("dist", [5.0, 7.6])      # full interaction, switching zone (rin 6.5, rc 8.5)
def test_cross_forces_are_energy_derivatives(orc, dist):
    rng = np.random.default_rng(int(dist * 10))
    box = np.array([40.0, 40.0, 40.0])
    qa = config.random_quaternions(1, rng); qb = config.random_quaternions(1, rng)
    ca = np.zeros((1, 3)); cb = np.array([[dist, 0.7, -0.4]])

    def energy(cb_):
        _, _, p = orc.pairsearch_hetero(ca, cb_, box, [8.5] * 3, 6.5, 8.5)
        xa, ya, za = sites(orc, "TIP4P", ca, qa)
        xb, yb, zb = sites(orc, "OPLSMEOH", cb_, qb)
        x, y, z = np.concatenate([xa, xb]), np.concatenate([ya, yb]), np.concatenate([za, zb])
        return orc.force_sites_hetero("TIP4P", "OPLSMEOH", "std", x, y, z, 0, len(xa), p)
    fx, fy, fz, ep, _ = energy(cb)
    Fb = np.array([fx[5:].sum(), fy[5:].sum(), fz[5:].sum()])
    h = 1e-5
    for k in range(3):
        e = []
        for sgn in (-2, -1, 1, 2):
            c = cb.copy(); c[0, k] += sgn * h
            e.append(energy(c)[3].sum())
        de = (e[0] - 8 * e[1] + 8 * e[2] - e[3]) / (12 * h)
        assert Fb[k] == pytest.approx(-de, rel=2e-7, abs=1e-6 * np.abs(Fb).max())
