"""Reference-facing pair-list calls (the Interaction2 dispatcher surface).

``force`` and ``pair_potential`` take the same data the Fortran routines take
-- the global site arrays (sSite, SiteModule.F90:29-37) and a compressed pair
list with image offsets and switch factors (sInteraction,
InteractionModule.F90:35-74) -- and run on the GPU through g6_force_sites /
g6_pair_potential.  Site forces accumulate into the caller's arrays exactly as
``force`` does (the caller zeroes them first, site_resetforce).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import _capi
from ._capi import dptr, iptr


@dataclass
class Sites:
    """sSite: x, y, z and fx, fy, fz over all sites (molecule m, site s at m*nsite+s)."""
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    fx: np.ndarray
    fy: np.ndarray
    fz: np.ndarray

    @classmethod
    def of(cls, x, y, z):
        f = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        x, y, z = f(x), f(y), f(z)
        return cls(x, y, z, np.zeros_like(x), np.zeros_like(x), np.zeros_like(x))

    def resetforce(self):
        """site_resetforce, SiteModule.F90:70-76."""
        self.fx[:] = 0.0; self.fy[:] = 0.0; self.fz[:] = 0.0


@dataclass
class Interaction:
    """sInteraction after Interaction_Compress2 + CutOff_Dimmer2 (0-based pair indices)."""
    pair_i: np.ndarray
    pair_j: np.ndarray
    ox: np.ndarray
    oy: np.ndarray
    oz: np.ndarray
    eratio: np.ndarray
    fratio: np.ndarray

    @classmethod
    def from_pairs(cls, p):
        i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
        f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        return cls(i32(p["i"]), i32(p["j"]), f64(p["ox"]), f64(p["oy"]), f64(p["oz"]), f64(p["hh"]), f64(p["dh"]))

    @property
    def npair(self):
        return len(self.pair_i)


def force(system, site: Sites, iv: Interaction):
    """force(iv, mi, mj, site, ep, vrmat, custom, si, sj), Interaction2.F90:19-68.

    Returns (ep per pair, vrmat 3x3); site forces are accumulated in ``site``.
    Model and `custom` path are those of ``system`` (a RigidWater).
    """
    ep = np.zeros(max(iv.npair, 1))
    vr = np.zeros(9)
    system._check(system.L.g6_force_sites(
        system.ctx, len(site.x), dptr(site.x), dptr(site.y), dptr(site.z), dptr(site.fx), dptr(site.fy),
        dptr(site.fz), iv.npair, iptr(iv.pair_i), iptr(iv.pair_j), dptr(iv.ox), dptr(iv.oy), dptr(iv.oz),
        dptr(iv.eratio), dptr(iv.fratio), dptr(ep), dptr(vr)))
    return ep[:iv.npair], vr.reshape(3, 3)


def pair_potential(system, site: Sites, iv: Interaction):
    """PairPotential(iv, mi, mj, site, ep, custom, si, sj), Interaction2.F90:71-121."""
    ep = np.zeros(max(iv.npair, 1))
    system._check(system.L.g6_pair_potential(
        system.ctx, len(site.x), dptr(site.x), dptr(site.y), dptr(site.z), iv.npair, iptr(iv.pair_i),
        iptr(iv.pair_j), dptr(iv.ox), dptr(iv.oy), dptr(iv.oz), dptr(iv.eratio), dptr(ep)))
    return ep[:iv.npair]


def site_positions(model: str, com, quat):
    """rigid_setsiteposition (RigidModule.F90:146) on the host: sites = COM + R(q) body."""
    info = _capi.model_info(model)
    com = np.asarray(com, dtype=np.float64)
    q = np.asarray(quat, dtype=np.float64)
    qa, qb, qc, qd = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    t = np.empty((len(q), 3, 3))
    t[:, 0, 0] = qa * qa + qb * qb - (qc * qc + qd * qd)
    t[:, 0, 1] = -2.0 * (qa * qd + qb * qc)
    t[:, 0, 2] = 2.0 * (qb * qd - qa * qc)
    t[:, 1, 0] = 2.0 * (qa * qd - qb * qc)
    t[:, 1, 1] = qa * qa + qc * qc - (qb * qb + qd * qd)
    t[:, 1, 2] = -2.0 * (qa * qb + qc * qd)
    t[:, 2, 0] = 2.0 * (qa * qc + qb * qd)
    t[:, 2, 1] = 2.0 * (qa * qb - qc * qd)
    t[:, 2, 2] = qa * qa + qd * qd - (qb * qb + qc * qc)
    s = com[:, None, :] + np.einsum("nab,sb->nsa", t, info["body"])
    return s[..., 0].ravel(), s[..., 1].ravel(), s[..., 2].ravel()
