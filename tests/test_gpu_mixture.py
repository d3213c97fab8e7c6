"""Mixtures through the C ABI against the oracle: the hetero pair search
(bit-exact pair set, image offsets and switch values) and the two-component
force (Interaction2.F90:19-68 cross branch: TIP4P-OPLS methanol on the custom
hand-kernel constants and on StdForce, methanol-methanol and water-water on
StdForce) at 1e-12."""
import ctypes

import numpy as np
import pytest

import genesis6_gb300 as g6
from genesis6_gb300 import _capi
from genesis6_gb300._capi import dptr, iptr
from test_mixture_oracle import mixture, sites

pytestmark = pytest.mark.gpu


def ctx_with_cutoff(rin, rc):
    L = g6.lib()
    ctx = ctypes.c_void_p()
    assert L.g6_ctx_create(0, ctypes.byref(ctx)) == _capi.G6_OK
    assert L.g6_set_cutoff(ctx, rin, rc) == _capi.G6_OK
    return L, ctx


def gpu_pairs(L, ctx, box, ca, cb):
    n = ctypes.c_int64()
    assert L.g6_pairsearch_hetero(ctx, dptr(box), len(ca), dptr(np.ascontiguousarray(ca)), len(cb),
                                  dptr(np.ascontiguousarray(cb)), ctypes.byref(n)) == _capi.G6_OK
    m = n.value
    p = dict(i=np.zeros(m, np.int32), j=np.zeros(m, np.int32), ox=np.zeros(m), oy=np.zeros(m), oz=np.zeros(m),
             hh=np.zeros(m), dh=np.zeros(m))
    assert L.g6_get_pairs(ctx, m, iptr(p["i"]), iptr(p["j"]), dptr(p["ox"]), dptr(p["oy"]), dptr(p["oz"]),
                          dptr(p["hh"]), dptr(p["dh"])) == _capi.G6_OK
    return p


@pytest.mark.parametrize("na,nb,L,rc", [(2000, 1000, None, 9.0), (300, 150, None, 8.5), (40, 30, 17.5, 5.5)])
def test_hetero_pairset_bitexact(orc, na, nb, L, rc):
    box, ca, _, cb, _ = mixture(na, nb, 11 + na, L)
    Lib, ctx = ctx_with_cutoff(rc - 2.0, rc)
    pg = gpu_pairs(Lib, ctx, box, ca, cb)
    _, _, po = orc.pairsearch_hetero(ca, cb, box, [rc] * 3, rc - 2.0, rc)
    kg = pg["i"].astype(np.int64) * 10 ** 7 + pg["j"]
    ko = po["i"].astype(np.int64) * 10 ** 7 + po["j"]
    assert len(kg) == len(ko) == len(np.unique(kg))
    og, oo = np.argsort(kg), np.argsort(ko)
    assert np.array_equal(kg[og], ko[oo])
    for k in ("ox", "oy", "oz", "hh", "dh"):
        assert np.array_equal(pg[k][og], po[k][oo]), k
    Lib.g6_ctx_destroy(ctx)


@pytest.mark.parametrize("mi,mj,path", [("TIP4P", "OPLSMEOH", "custom"), ("TIP4P", "OPLSMEOH", "std"),
                                        ("OPLSMEOH", "OPLSMEOH", "std"), ("TIP5P", "TIP5P", "std"),
                                        ("OPLSMEOH", "TIP4P", "std")])
def test_hetero_force_matches_oracle(orc, mi, mj, path):
    rc = 8.5
    box, ca, qa, cb, qb = mixture(400, 250, 21)
    Lib, ctx = ctx_with_cutoff(rc - 2.0, rc)
    p = gpu_pairs(Lib, ctx, box, ca, cb)
    xa, ya, za = sites(orc, mi, ca, qa)
    xb, yb, zb = sites(orc, mj, cb, qb)
    x, y, z = np.concatenate([xa, xb]), np.concatenate([ya, yb]), np.concatenate([za, zb])
    offb = len(xa)
    fx, fy, fz = np.zeros_like(x), np.zeros_like(x), np.zeros_like(x)
    ep, vr = np.zeros(len(p["i"])), np.zeros(9)
    st = Lib.g6_force_sites_hetero(ctx, _capi.MODELS[mi], _capi.MODELS[mj], _capi.PATHS[path], len(x), dptr(x),
                                   dptr(y), dptr(z), dptr(fx), dptr(fy), dptr(fz), 0, offb, len(p["i"]), iptr(p["i"]),
                                   iptr(p["j"]), dptr(p["ox"]), dptr(p["oy"]), dptr(p["oz"]), dptr(p["hh"]),
                                   dptr(p["dh"]), dptr(ep), dptr(vr))
    assert st == _capi.G6_OK
    ofx, ofy, ofz, oep, ovr = orc.force_sites_hetero(mi, mj, path, x, y, z, 0, offb, p)
    fs = np.abs(np.concatenate([ofx, ofy, ofz])).max()
    for a, b in ((fx, ofx), (fy, ofy), (fz, ofz)):
        assert np.abs(a - b).max() <= 1e-12 * fs
    assert np.abs(ep - oep).max() <= 1e-12 * np.abs(oep).max()
    assert np.abs(vr.reshape(3, 3) - ovr).max() <= 1e-12 * np.abs(ovr).max()
    # energies only (PairPotential)
    e2 = np.zeros(len(p["i"]))
    st = Lib.g6_force_sites_hetero(ctx, _capi.MODELS[mi], _capi.MODELS[mj], _capi.PATHS[path], len(x), dptr(x),
                                   dptr(y), dptr(z), None, None, None, 0, offb, len(p["i"]), iptr(p["i"]),
                                   iptr(p["j"]), dptr(p["ox"]), dptr(p["oy"]), dptr(p["oz"]), dptr(p["hh"]), None,
                                   dptr(e2), None)
    assert st == _capi.G6_OK
    assert np.abs(e2 - oep).max() <= 1e-12 * np.abs(oep).max()
    Lib.g6_ctx_destroy(ctx)


def test_methanol_is_not_an_md_model():
    Lib = g6.lib()
    ctx = ctypes.c_void_p()
    assert Lib.g6_ctx_create(0, ctypes.byref(ctx)) == _capi.G6_OK
    nm = np.array([10], np.int32)
    box = np.full(3, 30.0)
    assert Lib.g6_system(ctx, _capi.OPLSMEOH, 0, 0, 1, iptr(nm), dptr(box)) == _capi.G6_ERR_ARG
    Lib.g6_ctx_destroy(ctx)
