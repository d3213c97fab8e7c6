"""Site-site distance histograms (radialdistrib, RDFModule.F90:101-137).

CPU: the oracle (oracle/analysis.py) against a direct O(N^2) statement of the
definition, and the normalisation (genesis6_gb300/analysis.py) on an ideal gas.
GPU: the device counts equal the oracle's bin for bin.
"""
import math

import numpy as np
import pytest

from genesis6_gb300 import analysis, config
from oracle import analysis as A


def brute_counts(orc, model, com, quat, L, rc, nbin, w, vmin=0.0):
    ns = orc.model_info(model)["nsite"]
    x, y, z = orc.place_sites(model, com, quat)[:3]
    h = np.zeros((ns, ns, nbin), np.int64)
    n = len(com)
    for i in range(n):
        for j in range(i + 1, n):
            d = com[i] - com[j]
            shift = L * np.array([math.copysign(math.floor(abs(v) / Lk + 0.5), v) for v, Lk in zip(d, L)])
            dd = d - shift
            if (dd[0] * dd[0] + dd[1] * dd[1]) + dd[2] * dd[2] >= rc * rc:   # Interaction_Compress2: strict
                continue
            for a in range(ns):
                for b in range(ns):
                    v = np.array([x[i * ns + a] - x[j * ns + b], y[i * ns + a] - y[j * ns + b],
                                  z[i * ns + a] - z[j * ns + b]]) - shift
                    r = math.sqrt(v @ v)
                    t = (r - vmin) / w
                    k = int(math.floor(t + 0.5)) if t >= 0 else -int(math.floor(-t + 0.5))
                    if 0 <= k < nbin:
                        h[min(a, b), max(a, b), k] += 1
    return h


@pytest.mark.parametrize("model", ["TIP4P", "SPCE"])
def test_oracle_counts_follow_the_definition(orc, model):
    b = config.water_box(model, 64, 3, jitter=0.3)
    L = np.asarray(b["L"], float)
    h = A.rdf_counts(model, b["com"], b["quat"], L, 6.0, 130, 0.05)
    hb = brute_counts(orc, model, b["com"], b["quat"], L, 6.0, 130, 0.05)
    assert np.array_equal(h, hb)
    assert h[1, 0].sum() == 0 and h[0, 0].sum() > 0     # a <= b only


def test_nint_is_half_away_from_zero():
    assert list(A.nint([0.5, 1.5, 2.5, -0.5, -1.5, 0.49999999999999994])) == [1, 2, 3, -1, -2, 0]


def test_ideal_gas_normalises_to_one(orc):
    """Uniform random centres (no exclusion): g_COM-COM ~ 1 (SPC/E: the blank name is the COM only)."""
    rng = np.random.default_rng(5)
    n, L = 1500, 30.0
    ns = orc.model_info("SPCE")["nsite"]
    tot = np.zeros((ns, ns, 140), np.int64)
    for c in range(3):
        com = rng.uniform(0, L, (n, 3))
        q = rng.normal(size=(n, 4)); q /= np.linalg.norm(q, axis=1, keepdims=True)
        tot += A.rdf_counts("SPCE", com, q, np.full(3, L), 9.0, 140, 0.05)
    r, g = analysis.rdf(tot, "SPCE", n, L ** 3, 3, 0.05)
    band = (r > 2.0) & (r < 8.5)
    assert abs(g[(" ", " ")][band].mean() - 1.0) < 0.03


@pytest.mark.gpu
@pytest.mark.parametrize("model,n,rc,prec", [("TIP4P", 4096, 9.0, "mixed"), ("SPCE", 343, 8.5, "fp64"),
                                             ("ST2", 512, 9.0, "mixed")])
def test_device_counts_equal_oracle(orc, model, n, rc, prec):
    import genesis6_gb300 as g6
    b = config.water_box(model, n, 17, jitter=0.3)
    s = g6.RigidWater(model, n, b["L"], path="std", precision=prec, rc=rc)
    s.upload_state(b["rec"])
    h = s.rdf_counts(200, 0.05)
    ho = A.rdf_counts(model, b["com"], b["quat"], np.asarray(b["L"], float), rc, 200, 0.05)
    assert h.shape == (1,) + ho.shape
    assert np.array_equal(h[0], ho)
    h2 = s.rdf_counts(200, 0.05)                       # counts are added to the caller's array each call
    assert np.array_equal(h2, h)


@pytest.mark.gpu
def test_device_counts_per_replica(orc):
    import genesis6_gb300 as g6
    sizes = [216, 343]
    boxes = [config.water_box("TIP4P", m, 30 + k, jitter=0.3) for k, m in enumerate(sizes)]
    s = g6.RigidWater("TIP4P", sizes, np.array([bx["L"] for bx in boxes]), path="custom", rc=8.0)
    s.upload_state(np.concatenate([bx["rec"] for bx in boxes]))
    h = s.rdf_counts(120, 0.07, minvalue=0.5)
    for k, bx in enumerate(boxes):
        ho = A.rdf_counts("TIP4P", bx["com"], bx["quat"], np.asarray(bx["L"], float), 8.0, 120, 0.07, 0.5)
        assert np.array_equal(h[k], ho)


def brute_hbonds(orc, model, com, quat, L, rc):
    """A direct loop over molecule pairs of the reference's O-H test."""
    ns = orc.model_info(model)["nsite"]
    h1 = 2 if model == "TIP4P" else 1
    x, y, z = orc.place_sites(model, com, quat)[:3]
    out = set()
    n = len(com)
    for i in range(n):
        for j in range(i + 1, n):
            d = com[i] - com[j]
            shift = L * np.array([math.copysign(math.floor(abs(v) / Lk + 0.5), v) for v, Lk in zip(d, L)])
            dd = d - shift
            if (dd[0] * dd[0] + dd[1] * dd[1]) + dd[2] * dd[2] >= rc * rc:
                continue
            best, pb, wb, pnum = 1e10, 0, 0, 0
            for blk in range(2):
                for h in range(2):
                    a = i * ns + (0 if blk == 0 else h1 + h)
                    b = j * ns + (h1 + h if blk == 0 else 0)
                    v = np.array([x[a] - x[b], y[a] - y[b], z[a] - z[b]]) - shift
                    dist = v[0] ** 2 + v[1] ** 2 + v[2] ** 2
                    pnum += 1
                    if dist < best:
                        best, pb, wb = dist, pnum, h + 1
            if best < 6.25:
                out.add((j, wb, i) if pb <= 2 else (i, wb, j))
    return out


@pytest.mark.parametrize("model", ["TIP4P", "ST2"])
def test_oracle_hbonds_follow_the_definition(orc, model):
    b = config.water_box(model, 64, 4, jitter=0.3)
    L = np.asarray(b["L"], float)
    hb = A.hbonds(model, b["com"], b["quat"], L, 6.0)
    assert len(hb) > 10
    assert set(map(tuple, hb.tolist())) == brute_hbonds(orc, model, b["com"], b["quat"], L, 6.0)


def test_graph_text_layout():
    txt = analysis.graph_text([[3, 1, 7], [10, 2, 4]], 16, "WGPH")
    assert txt.splitlines() == ["@WGPH", " 16", "    3    7    1", "   10    4    2", "   -1   -1   -1"]
    assert analysis.graph_text([[3, 1, 7]], 16).splitlines()[-2:] == ["    3    7", "   -1   -1"]


@pytest.mark.gpu
@pytest.mark.parametrize("model,n,prec", [("TIP4P", 4096, "mixed"), ("ST2", 512, "fp64"), ("SPCE", 343, "mixed")])
def test_device_hbonds_equal_oracle(orc, model, n, prec):
    import genesis6_gb300 as g6
    b = config.water_box(model, n, 23, temp=300.0, dt=0.002, jitter=0.3)
    s = g6.RigidWater(model, n, b["L"], path="std", precision=prec, rc=8.5)
    s.upload_state(b["rec"])
    # a few short steps away from the lattice (random orientations start hot)
    s.md_run(0.0005, 40, s.thermostats(1, "nose", temp=300.0, q=300.0 * 0.25 ** 2 / 0.0005), log=False)
    rec = s.download_state()
    hb = s.hbonds()
    ho = A.hbonds(model, rec[:, 0:3], rec[:, 33:37], np.asarray(b["L"], float), 8.5)
    assert len(hb) > n // 10
    assert set(map(tuple, hb.tolist())) == set(map(tuple, ho.tolist()))
