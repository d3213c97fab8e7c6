"""Normalisation of the device's site-site distance counts (RigidWater.rdf_counts)
into radial distribution functions, as rdf_normalize and comrdf_normalize do
(RDFModule.F90:60-84, DistribModule.F90:200-226) for one homogeneous component.

Sites are grouped by the reference's site names (TIP4PConst.F90:22,
TIP5PModule.F90:51, ST2Module.F90:26, SPCEModule.F90:18; a blank name is the
massless charge sites and the centre of mass).  For names A and B the counts
S_AB (A on one molecule, B on the other, both orders) give
    g_AB(r) = S_AB / (K shell(r)) / (2 if A != B else 1),
    K = nconf N m_A m_B (N - 1) / (2 V),  shell(r) = 4/3 pi 2 (3 r^2 x + x^3), x = binwidth / 2,
with m_A the number of sites named A in a molecule and r = minvalue + k binwidth
the centre of bin k; for A = B this is the reference's normalisation of its
single histogram, for A != B the mean of its two ordered histograms.
"""
from __future__ import annotations

import math
from typing import Dict, Tuple

import numpy as np

SITE_NAMES = {
    "TIP4P": ["O", " ", "H", "H", " "],
    "TIP5P": ["O", "H", "H", " ", " ", " "],
    "ST2": ["O", "H", "H", "M", "M", " "],
    "SPCE": ["O", "H", "H", " "],
}


def rdf(counts, model: str, nmol: int, volume: float, nconf: int, binwidth: float,
        minvalue: float = 0.0) -> Tuple[np.ndarray, Dict[Tuple[str, str], np.ndarray]]:
    """counts: (nsite, nsite, nbin) summed over nconf configurations of one
    replica.  Returns the bin centres and g(r) per pair of site names."""
    counts = np.asarray(counts)
    names = SITE_NAMES[model]
    nbin = counts.shape[-1]
    r = minvalue + binwidth * np.arange(nbin)
    x = 0.5 * binwidth
    shell = 4.0 / 3.0 * math.pi * 2.0 * (3.0 * r ** 2 * x + x ** 3)
    groups: Dict[str, list] = {}
    for s, nm in enumerate(names):
        groups.setdefault(nm, []).append(s)
    out = {}
    keys = sorted(groups)
    for ia, A in enumerate(keys):
        for B in keys[ia:]:
            s_ab = np.zeros(nbin)
            for a in groups[A]:
                for b in groups[B]:
                    lo, hi = min(a, b), max(a, b)
                    s_ab += counts[lo, hi]
            K = nconf * nmol * len(groups[A]) * len(groups[B]) * (nmol - 1) / (2.0 * volume)
            out[(A, B)] = s_ab / (K * shell) / (2.0 if A != B else 1.0)
    return r, out


def graph_text(bonds, nmol: int, kind: str = "NGPH") -> str:
    """@NGPH (donor, acceptor) or @WGPH (donor, acceptor, hydrogen) lines of
    interaction_SaveGraph (InteractionModule.F90:783-823): 0-based molecules in
    '(99i5)' fields, terminated by -1 entries."""
    bonds = np.asarray(bonds).reshape(-1, 3)
    out = ["@" + kind, " %d" % nmol]
    for f, w, t in bonds:
        out.append("%5d%5d" % (f, t) + ("%5d" % w if kind == "WGPH" else ""))
    out.append("%5d%5d" % (-1, -1) + ("%5d" % -1 if kind == "WGPH" else ""))
    return "\n".join(out) + "\n"
