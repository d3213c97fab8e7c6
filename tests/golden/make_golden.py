"""Generate the golden vectors that pin the oracle.

Genesis6 ships no test vectors, so these are computed here independently of
the oracle: a direct Python statement of the model definitions (site geometry
and parameters of TIP4PModule.F90:43-97, TIP5PModule.F90:38-83,
RigidModule.F90:429-477, ST2Module.F90:10-100, SPCEModule.F90:8-71) and of the pair energy (site
sums of Coulomb and 12-6 LJ scaled by the centre-of-mass switch of
CutoffModule.F90:38-59, and for ST2 the Coulomb taper of ST2Module.F90:206-225).
Forces and torques come from 4th-order central finite differences of that
energy (translations of the COM; rotations of the lab-frame site offsets about
the lab axes), not from an analytic formula, so they check the oracle's
analytic derivatives.  Pair sets come from an O(N^2) minimum-image scan.

Run:  python tests/golden/make_golden.py   (writes dimers.json, pairset_small.json)
"""
from __future__ import annotations

import json
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

PI = 3.1415926535897932
NA = 6.0225e23
CA = 4.184
COEFF = CA * 332.17752
F32 = lambda v: float(np.float32(v))   # Fortran default-real literal promoted to double


def geometry(model):
    if model == "TIP4P":
        body = [[0, 0, -6.50980307353661025e-02], [0, 0, 8.49019692646338919e-02],
                [0, 7.56950327263661182e-01, 5.20784245882928820e-01],
                [0, -7.56950327263661182e-01, 5.20784245882928820e-01], [0, 0, 0]]
        q = [0, -1.04, 0.52, 0.52, 0]
        eps, sig = 0.15504166666666666666666 * CA, 3.15357794197649532464
        return np.array(body, float), np.array(q, float), eps, sig
    if model == "SPCE":   # the oxygen carries both the LJ site and a charge
        th = 109.5 * PI / 180
        s, c = math.sin(0.5 * th), math.cos(0.5 * th)
        body = np.array([[0, 0, 0], [0, s, c], [0, -s, c], [0, 0, 0]], float)
        body[:3, 2] -= body[1, 2] * 2.0 / 18.0
        return body, np.array([-0.8476, 0.4238, 0.4238, 0.0]), 78.208 / 0.120273 * 1e-3, 3.166
    if model == "TIP5P":
        theta, phi, l1, l2 = 104.52 * PI / 180, 109.47 * PI / 180, 0.9572, 0.70
        q = [0, 0.2410, 0.2410, -0.2410, -0.2410, 0]
        eps, sig = 0.6694, 3.12
    else:
        theta = phi = 109.47 * PI / 180
        l1, l2 = 1.0, 0.8
        qh, qm = F32(0.2357), F32(-0.2357)
        q = [0, qh, qh, qm, qm, 0]
        eps, sig = F32(0.52605e-21) * NA * 1e-3, 3.1
    s, c = math.sin(0.5 * theta), math.cos(0.5 * theta)
    sp, cp = math.sin(0.5 * phi), math.cos(0.5 * phi)
    body = np.array([[0, 0, 0], [0, l1 * s, l1 * c], [0, -l1 * s, l1 * c], [l2 * sp, 0, -l2 * cp],
                     [-l2 * sp, 0, -l2 * cp], [0, 0, 0]], float)
    zshift = body[1, 2] * 2.0 / 18.0
    body[:5, 2] -= zshift
    return body, np.array(q, float), eps, sig


def rotation(q):
    a, b, c, d = q
    return np.array([[a * a + b * b - c * c - d * d, -2 * (a * d + b * c), 2 * (b * d - a * c)],
                     [2 * (a * d - b * c), a * a + c * c - b * b - d * d, -2 * (a * b + c * d)],
                     [2 * (a * c + b * d), 2 * (a * b - c * d), a * a + d * d - b * b - c * c]])


def switch(r, rin, rout):
    if r >= rout:
        return 0.0
    if r <= rin:
        return 1.0
    x = (r - rin) / (rout - rin)            # smoothstep of degree 5, written independently
    return 1.0 - x ** 3 * (10 - 15 * x + 6 * x * x)


def taper(r, rl=2.016, ru=3.1287):
    if r <= rl:
        return 0.0
    if r >= ru:
        return 1.0
    x = (r - rl) / (ru - rl)
    return x * x * (3 - 2 * x)


def dimer_energy(model, custom, off_i, off_j, ci, cj, L, rin, rout):
    """Energy of one molecule pair: lab-frame site offsets and COMs, minimum image."""
    body, q, eps, sig = geometry(model)
    d = ci - cj
    d = d - L * np.array([math.floor(v / Lk + 0.5) if v >= 0 else -math.floor(-v / Lk + 0.5)
                          for v, Lk in zip(d, L)])
    r = float(np.sqrt(d @ d))
    if r >= rout:
        return 0.0
    if model == "TIP4P" and custom:
        A, B = 600000.0 * CA * 100.0, -610.0 * CA * 100.0
        qq = lambda a, b: q[a] * q[b] * COEFF * 100.0
    else:
        s6 = ((sig + sig) / 2) ** 6
        A, B = 4 * eps * s6 * s6 * 100.0, -4 * eps * s6 * 100.0
        qq = lambda a, b: q[a] * q[b] * COEFF * 100.0
    ns = len(q)
    ecoul = 0.0
    for a in range(0, ns - 1):          # every charged site (site 0 only for SPC/E)
        for b in range(0, ns - 1):
            if q[a] == 0.0 or q[b] == 0.0:
                continue
            v = d + off_i[a] - off_j[b]
            ecoul += qq(a, b) / math.sqrt(v @ v)
    v = d + off_i[0] - off_j[0]
    r2 = v @ v
    elj = A / r2 ** 6 + B / r2 ** 3
    S = switch(r, rin, rout)
    if model == "ST2" and custom:
        return S * elj + S * taper(r) * ecoul
    return S * (elj + ecoul)


def fd(f, h):
    return (-f(2 * h) + 8 * f(h) - 8 * f(-h) + f(-2 * h)) / (12 * h)


def rot_axis(k, th):
    c, s = math.cos(th), math.sin(th)
    R = np.eye(3)
    i, j = [(1, 2), (2, 0), (0, 1)][k]
    R[i, i] = c; R[i, j] = -s; R[j, i] = s; R[j, j] = c
    return R


def dimer_case(model, custom, com, quat, L, rin, rout):
    body, *_ = geometry(model)
    offs = [np.array([rotation(qq) @ b for b in body]) for qq in quat]
    E = dimer_energy(model, custom, offs[0], offs[1], com[0], com[1], L, rin, rout)
    F = np.zeros((2, 3)); tl = np.zeros((2, 3))
    for m in range(2):
        for k in range(3):
            def e_tr(h, m=m, k=k):
                c = [com[0].copy(), com[1].copy()]
                c[m][k] += h
                return dimer_energy(model, custom, offs[0], offs[1], c[0], c[1], L, rin, rout)
            F[m, k] = -fd(e_tr, 1e-4)

            def e_rot(th, m=m, k=k):
                o = [offs[0], offs[1]]
                o[m] = o[m] @ rot_axis(k, th).T
                return dimer_energy(model, custom, o[0], o[1], com[0], com[1], L, rin, rout)
            tl[m, k] = -fd(e_rot, 1e-4)
    tau = np.array([rotation(quat[m]).T @ tl[m] for m in range(2)])
    return E, F, tau


def unit(v):
    v = np.asarray(v, float)
    return v / np.linalg.norm(v)


def dimers():
    rng = np.random.default_rng(20261203)
    cases = []
    L = np.array([20.0, 20.0, 20.0])
    seps = [("full", [2.9, 0.3, -0.2]), ("switch", [7.3, 0.4, 0.5]), ("image", [-17.0, 0.3, 0.2]),
            ("outside", [8.6, 0.3, 0.0])]
    for model in ["TIP4P", "TIP5P", "ST2", "SPCE"]:
        for custom in ([True, False] if model in ("TIP4P", "ST2") else [False]):
            for name, sep in seps:
                quat = [unit(rng.standard_normal(4)), unit(rng.standard_normal(4))]
                c0 = np.array([0.5, -0.3, 0.2])
                com = [c0, c0 - np.array(sep)]
                E, F, tau = dimer_case(model, custom, com, quat, L, 6.5, 8.5)
                cases.append({"model": model, "path": "custom" if custom else "std", "name": name,
                              "L": L.tolist(), "rin": 6.5, "rc": 8.5, "com": [c.tolist() for c in com],
                              "quat": [q.tolist() for q in quat], "E": E, "F": F.tolist(), "tau": tau.tolist()})
    return cases


def pairset_small():
    rng = np.random.default_rng(7)
    n = 200
    L = (n / 0.033456) ** (1 / 3)
    com = rng.uniform(-0.5 * L, 0.5 * L, (n, 3))
    com[:10] += L * rng.integers(-2, 3, (10, 3))     # a few molecules outside the primary box
    rc = 7.0
    pairs = []
    for i in range(n):
        for j in range(i + 1, n):
            d = com[i] - com[j]
            d = d - L * np.array([math.floor(abs(v) / L + 0.5) * (1 if v >= 0 else -1) for v in d])
            if (d[0] * d[0] + d[1] * d[1]) + d[2] * d[2] < rc * rc:
                pairs.append([i, j])
    return {"L": [L, L, L], "rc": rc, "rin": rc - 2.0, "com": com.tolist(), "pairs": pairs}


if __name__ == "__main__":
    with open(os.path.join(HERE, "dimers.json"), "w") as f:
        json.dump(dimers(), f, indent=1)
    with open(os.path.join(HERE, "pairset_small.json"), "w") as f:
        json.dump(pairset_small(), f)
    print("wrote", os.listdir(HERE))
