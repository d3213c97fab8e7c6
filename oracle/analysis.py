"""CPU reference of the site-site distance histogram (test infrastructure).

radialdistrib (RDFModule.F90:101-137) over the oracle's pair set and site
positions: for every pair k and every site a of molecule i and b of molecule j,
dx = x(i,a) - x(j,b) - ox(k) (the same for y, z), r = sqrt(dx^2 + dy^2 + dz^2),
bin = nint((r - minvalue) / binwidth) (Histogram_Accumulate,
DistribModule.F90:149-158, 0-based here), counted when 0 <= bin < nbin.  The
count is kept per unordered site pair (a <= b), the sum of both orders of a
pair, which does not depend on which molecule the pair list names first.
All arithmetic is FP64 in the reference's order (numpy evaluates the sums left
to right without contraction; the oracle library is built without contraction).
"""
from __future__ import annotations

import numpy as np

from . import pairsearch, place_sites, model_info


def nint(t):
    """Fortran nint: round half away from zero, exactly (no t + 0.5 rounding)."""
    t = np.asarray(t, dtype=np.float64)
    a = np.abs(t)
    w = np.trunc(a)
    r = w + (a - w >= 0.5)
    return np.copysign(r, t)


def rdf_counts(model, com, quat, L, rc, nbin, binwidth, minvalue=0.0):
    """(nsite, nsite, nbin) int64 counts for one configuration (a <= b filled)."""
    ns = model_info(model)["nsite"]
    x, y, z = place_sites(model, com, quat)[:3]
    _, p = pairsearch(com, L, [rc] * 3, rc - 2.0, rc)
    hist = np.zeros((ns, ns, nbin), dtype=np.int64)
    i, j = p["i"].astype(np.int64), p["j"].astype(np.int64)
    for a in range(ns):
        for b in range(ns):
            dx = (x[i * ns + a] - x[j * ns + b]) - p["ox"]
            dy = (y[i * ns + a] - y[j * ns + b]) - p["oy"]
            dz = (z[i * ns + a] - z[j * ns + b]) - p["oz"]
            r = np.sqrt(dx * dx + dy * dy + dz * dz)
            k = nint((r - minvalue) / binwidth)
            ok = (k >= 0) & (k < nbin)
            lo, hi = min(a, b), max(a, b)
            hist[lo, hi] += np.bincount(k[ok].astype(np.int64), minlength=nbin)
    return hist


def hbonds(model, com, quat, L, rc):
    """interaction_hb_by_oh_distance (InteractionModule.F90:682-777) over the
    oracle's pair set: the four squared distances O(i)-H1(j), O(i)-H2(j),
    O(j)-H1(i), O(j)-H2(i) (dx = x(ii) - x(jj) - ox, ii on molecule i), the first
    strict minimum, a bond below 2.5^2 A^2 from the hydrogen's molecule.
    Returns (m, 3) rows (donor, hydrogen 1/2, acceptor), 0-based."""
    ns = model_info(model)["nsite"]
    osite, h1 = 0, (2 if model == "TIP4P" else 1)
    x, y, z = place_sites(model, com, quat)[:3]
    _, p = pairsearch(com, L, [rc] * 3, rc - 2.0, rc)
    i, j = p["i"].astype(np.int64), p["j"].astype(np.int64)
    d = []
    for blk in range(2):
        for h in range(2):
            ii = i * ns + (osite if blk == 0 else h1 + h)
            jj = j * ns + (h1 + h if blk == 0 else osite)
            dx = (x[ii] - x[jj]) - p["ox"]
            dy = (y[ii] - y[jj]) - p["oy"]
            dz = (z[ii] - z[jj]) - p["oz"]
            d.append(dx * dx + dy * dy + dz * dz)
    d = np.stack(d, axis=1)
    k = np.argmin(d, axis=1)                      # first minimum, as the strict sequential test
    dmin = d[np.arange(len(k)), k]
    ok = dmin < 6.25
    donor = np.where(k <= 1, j, i)
    acceptor = np.where(k <= 1, i, j)
    return np.stack([donor[ok], (k % 2 + 1)[ok], acceptor[ok]], axis=1)
