"""CPU oracle for the rigid-water force/energy path (test infrastructure).

The oracle is an FP64 C++ restatement of Genesis6's Fortran (g6_oracle.cpp,
every function cites the reference file:line it follows).  It exists to check
the CUDA library: only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` may load it.

Parity unpinned: the reference ships no test vectors and its Fortran cannot be
compiled here, so no output of the reference itself pins this restatement.  It
is checked against independently computed closed-form dimer vectors
(tests/golden) and the reference's own self-consistency checks restated as
tests.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "g6_oracle.cpp")
LIB = os.path.join(HERE, "libg6oracle.so")

MODEL = {"TIP4P": 1, "TIP5P": 2, "ST2": 3, "SPCE": 4, "OPLSMEOH": 5}
PATH = {"std": 0, "custom": 1}
REC = 53  # per-molecule rigid record: com[3], d[5][3], w[5][3], q[5][4]


def build(force: bool = False) -> str:
    """Compile the oracle with IEEE-exact FP64 settings (no FMA contraction)."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        cmd = ["g++", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-shared", "-fPIC",
               "-o", LIB + ".tmp", SRC]
        subprocess.run(cmd, check=True)
        os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
        ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
        c_int, c_long, c_double = ctypes.c_int, ctypes.c_long, ctypes.c_double
        L.orc_model_info.argtypes = [c_int, ctypes.POINTER(c_int), dp, dp, dp]
        L.orc_constants.argtypes = [dp]
        L.orc_place_sites.argtypes = [c_int, c_int, dp, dp, dp, dp, dp, dp, dp]
        L.orc_grid.argtypes = [dp, dp, ip, dp, ctypes.POINTER(c_int), ctypes.POINTER(c_int), ip]
        L.orc_pairsearch.restype = c_long
        L.orc_pairsearch.argtypes = [c_int, dp, dp, dp, c_double, c_double, ip, c_long, ip, ip, dp, dp, dp, dp, dp]
        L.orc_force_sites.argtypes = [c_int, c_int, c_int, dp, dp, dp, dp, dp, dp, c_long, ip, ip, dp, dp, dp, dp,
                                      dp, dp, dp]
        L.orc_pair_potential.argtypes = [c_int, c_int, dp, dp, dp, c_long, ip, ip, dp, dp, dp, dp, dp]
        L.orc_compute.restype = c_long
        L.orc_compute.argtypes = [c_int, c_int, c_int, dp, dp, dp, dp, c_double, c_double, dp, dp, dp, dp]
        L.orc_compute_threaded.restype = c_long
        L.orc_compute_threaded.argtypes = [c_int, c_int, dp, dp, dp, dp, c_double, c_double, c_int, dp, dp, dp, dp]
        L.orc_md_run.argtypes = [c_int, c_int, c_int, dp, dp, dp, c_double, c_double, c_double, c_int, dp, dp]
        L.orc_kinetic.argtypes = [c_int, c_int, dp, c_double, dp]
        L.orc_philox_uniform2.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                          ctypes.c_uint32, dp]
        L.orc_molecule_energy.restype = c_double
        L.orc_molecule_energy.argtypes = [c_int, c_int, c_int, dp, dp, c_int, dp, dp, dp, c_double, c_double]
        L.orc_md_run_threaded.argtypes = [c_int, c_int, dp, dp, dp, c_double, c_double, c_double, c_int, dp, dp,
                                          c_int]
        L.orc_mc_run.argtypes = [c_int, c_int, c_int, dp, dp, dp, c_double, c_double, c_double, c_double, c_double,
                                 c_int, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint64, dp, dp]
        L.orc_max_threads.restype = c_int
        L.orc_vreset2.argtypes = [c_int, c_int, c_double, c_double, dp, dp, dp]
        L.orc_replica_exchange_trial.argtypes = [c_int, c_int, ip, c_double, dp, dp, c_int, dp, dp]
        L.orc_pairsearch_hetero.restype = c_long
        L.orc_pairsearch_hetero.argtypes = [c_int, dp, c_int, dp, dp, dp, c_double, c_double, ip, ip, c_long, ip, ip,
                                            dp, dp, dp, dp, dp]
        L.orc_force_sites_hetero.argtypes = [c_int, c_int, c_int, dp, dp, dp, dp, dp, dp, c_int, c_int, c_long, ip,
                                             ip, dp, dp, dp, dp, dp, dp, dp]
        L.orc_order_parameter.restype = c_double
        L.orc_order_parameter.argtypes = [c_int, c_int, dp, dp, dp, c_int, c_double, dp, dp]
        L.orc_mc_umbrella_run.argtypes = [c_int, c_int, c_int, dp, dp, dp, c_double, c_double, c_double, c_double,
                                          c_double, c_int, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint64, c_int,
                                          c_double, c_double, dp, c_int, dp, dp, dp]
        _lib = L
    return _lib


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a if shape is None else a.reshape(shape)


def model_info(model: str):
    L = lib()
    ns = ctypes.c_int()
    body = np.zeros(24)
    param = np.zeros(24)
    mi = np.zeros(4)
    if L.orc_model_info(MODEL[model], ctypes.byref(ns), body, param, mi):
        raise ValueError(model)
    n = ns.value
    return {"nsite": n, "body": body[:3 * n].reshape(n, 3).copy(), "param": param[:3 * n].reshape(n, 3).copy(),
            "mass": mi[0], "inertia": mi[1:].copy()}


def constants():
    out = np.zeros(12)
    lib().orc_constants(out)
    keys = ["PI", "NA", "KB", "RGAS", "COEFF", "I2J", "J2I", "J2K", "KX2X", "P2A", "ANG2M", "X2KX"]
    return dict(zip(keys, out.tolist()))


def place_sites(model: str, com, quat):
    com = _f64(com); quat = _f64(quat)
    n = com.shape[0]
    ns = model_info(model)["nsite"]
    sx = np.zeros(n * ns); sy = np.zeros(n * ns); sz = np.zeros(n * ns)
    intra = np.zeros(n * ns * 3); tmat = np.zeros(n * 9)
    lib().orc_place_sites(MODEL[model], n, com, quat, sx, sy, sz, intra, tmat)
    return sx, sy, sz, intra.reshape(n, ns, 3), tmat.reshape(n, 3, 3)


def grid(L, req):
    ndiv = np.zeros(3, dtype=np.int32); cell = np.zeros(3)
    nn = ctypes.c_int(); nn0 = ctypes.c_int(); st = np.zeros(81, dtype=np.int32)
    lib().orc_grid(_f64(L), _f64(req), ndiv, cell, ctypes.byref(nn), ctypes.byref(nn0), st)
    k = nn.value + nn0.value
    s = st[:3 * k].reshape(k, 3)
    return ndiv, cell, s[:nn.value].copy(), s[nn.value:].copy()


def pairsearch(com, L, req, rin, rc):
    """Cell ids (0-based) and the exact pair set with image offsets and switch values."""
    com = _f64(com)
    n = com.shape[0]
    L = _f64(L); req = _f64(req)
    cell = np.zeros(n, dtype=np.int32)
    cap = 1
    while True:
        pi = np.zeros(cap, dtype=np.int32); pj = np.zeros(cap, dtype=np.int32)
        ox, oy, oz, hh, dh = (np.zeros(cap) for _ in range(5))
        npair = lib().orc_pairsearch(n, com, L, req, rin, rc, cell, cap, pi, pj, ox, oy, oz, hh, dh)
        if npair <= cap:
            break
        cap = npair
    s = slice(0, npair)
    return cell, dict(i=pi[s].copy(), j=pj[s].copy(), ox=ox[s].copy(), oy=oy[s].copy(), oz=oz[s].copy(),
                      hh=hh[s].copy(), dh=dh[s].copy())


def pairsearch_hetero(com_a, com_b, L, req, rin, rc):
    """Cell ids of both components and the exact pair set (i in A, j in B) of the hetero stencil."""
    ca = _f64(com_a); cb = _f64(com_b)
    na, nb = ca.shape[0], cb.shape[0]
    cell_a = np.zeros(na, dtype=np.int32); cell_b = np.zeros(nb, dtype=np.int32)
    cap = 1
    while True:
        pi = np.zeros(cap, dtype=np.int32); pj = np.zeros(cap, dtype=np.int32)
        ox, oy, oz, hh, dh = (np.zeros(cap) for _ in range(5))
        npair = lib().orc_pairsearch_hetero(na, ca, nb, cb, _f64(L), _f64(req), rin, rc, cell_a, cell_b, cap, pi, pj,
                                            ox, oy, oz, hh, dh)
        if npair <= cap:
            break
        cap = npair
    s = slice(0, npair)
    return cell_a, cell_b, dict(i=pi[s].copy(), j=pj[s].copy(), ox=ox[s].copy(), oy=oy[s].copy(), oz=oz[s].copy(),
                                hh=hh[s].copy(), dh=dh[s].copy())


def force_sites_hetero(model_i, model_j, path, x, y, z, offi, offj, pairs):
    """force(iv, mi, mj, site, ...) for two components on one global site store."""
    x = _f64(x); y = _f64(y); z = _f64(z)
    nt = x.shape[0]
    fx = np.zeros(nt); fy = np.zeros(nt); fz = np.zeros(nt)
    np_ = len(pairs["i"])
    ep = np.zeros(max(np_, 1)); vr = np.zeros(9)
    pi = np.ascontiguousarray(pairs["i"], dtype=np.int32); pj = np.ascontiguousarray(pairs["j"], dtype=np.int32)
    lib().orc_force_sites_hetero(MODEL[model_i], MODEL[model_j], PATH[path], x, y, z, fx, fy, fz, int(offi),
                                 int(offj), np_, pi, pj, _f64(pairs["ox"]), _f64(pairs["oy"]), _f64(pairs["oz"]),
                                 _f64(pairs["hh"]), _f64(pairs["dh"]), ep, vr)
    return fx, fy, fz, ep[:np_], vr.reshape(3, 3)


def force_sites(model, path, x, y, z, pairs, fx=None, fy=None, fz=None):
    x = _f64(x); y = _f64(y); z = _f64(z)
    nt = x.shape[0]
    fx = np.zeros(nt) if fx is None else fx
    fy = np.zeros(nt) if fy is None else fy
    fz = np.zeros(nt) if fz is None else fz
    np_ = len(pairs["i"])
    ep = np.zeros(max(np_, 1)); vr = np.zeros(9)
    pi = np.ascontiguousarray(pairs["i"], dtype=np.int32); pj = np.ascontiguousarray(pairs["j"], dtype=np.int32)
    lib().orc_force_sites(MODEL[model], PATH[path], nt, x, y, z, fx, fy, fz, np_, pi, pj, _f64(pairs["ox"]),
                          _f64(pairs["oy"]), _f64(pairs["oz"]), _f64(pairs["hh"]), _f64(pairs["dh"]), ep, vr)
    return fx, fy, fz, ep[:np_], vr.reshape(3, 3)


def pair_potential(model, path, x, y, z, pairs):
    np_ = len(pairs["i"])
    ep = np.zeros(max(np_, 1))
    pi = np.ascontiguousarray(pairs["i"], dtype=np.int32); pj = np.ascontiguousarray(pairs["j"], dtype=np.int32)
    lib().orc_pair_potential(MODEL[model], PATH[path], _f64(x), _f64(y), _f64(z), np_, pi, pj, _f64(pairs["ox"]),
                             _f64(pairs["oy"]), _f64(pairs["oz"]), _f64(pairs["hh"]), ep)
    return ep[:np_]


def compute(model, path, com, quat, L, req, rin, rc):
    """Full force path: returns F (n,3), body torque (n,3), Epot, virial (3,3), npair."""
    com = _f64(com); quat = _f64(quat)
    n = com.shape[0]
    F = np.zeros((n, 3)); tau = np.zeros((n, 3)); ep = np.zeros(1); vir = np.zeros(9)
    npair = lib().orc_compute(MODEL[model], PATH[path], n, com, quat, _f64(L), _f64(req), rin, rc, F, tau, ep, vir)
    return F, tau, ep[0], vir.reshape(3, 3), npair


def compute_threaded(model, com, quat, L, req, rin, rc, nthreads):
    com = _f64(com); quat = _f64(quat)
    n = com.shape[0]
    F = np.zeros((n, 3)); tau = np.zeros((n, 3)); ep = np.zeros(1); vir = np.zeros(9)
    npair = lib().orc_compute_threaded(MODEL[model], n, com, quat, _f64(L), _f64(req), rin, rc, nthreads, F, tau,
                                       ep, vir)
    return F, tau, ep[0], vir.reshape(3, 3), npair


def md_run(model, path, rec, L, req, rin, rc, dt, nsteps, thermo):
    """Gear MD (Mixture.F90 step order).  rec (n,53) and thermo[10] updated in place."""
    rec = np.ascontiguousarray(rec, dtype=np.float64)
    n = rec.shape[0]
    thermo = np.ascontiguousarray(thermo, dtype=np.float64)
    log = np.zeros((nsteps, 8))
    lib().orc_md_run(MODEL[model], PATH[path], n, rec, _f64(L), _f64(req), rin, rc, dt, nsteps, thermo, log)
    return rec, thermo, log


def md_run_threaded(model, rec, L, req, rin, rc, dt, nsteps, thermo, nthreads):
    """Gear MD with the StdForce arithmetic threaded over nthreads host threads (timing only)."""
    rec = np.ascontiguousarray(rec, dtype=np.float64)
    thermo = np.ascontiguousarray(thermo, dtype=np.float64)
    log = np.zeros((nsteps, 8))
    lib().orc_md_run_threaded(MODEL[model], rec.shape[0], rec, _f64(L), _f64(req), rin, rc, dt, nsteps, thermo,
                              log, int(nthreads))
    return rec, thermo, log


def kinetic(model, rec, dt):
    rec = np.ascontiguousarray(rec, dtype=np.float64)
    out = np.zeros(2)
    lib().orc_kinetic(MODEL[model], rec.shape[0], rec, dt, out)
    return out


def philox_uniform2(seed, c0, c1, c2, c3):
    out = np.zeros(2)
    lib().orc_philox_uniform2(seed, c0, c1, c2, c3, out)
    return out


def molecule_energy(model, path, com, quat, t, com_t, quat_t, L, rin, rc):
    com = _f64(com); quat = _f64(quat)
    return lib().orc_molecule_energy(MODEL[model], PATH[path], com.shape[0], com, quat, int(t), _f64(com_t),
                                     _f64(quat_t), _f64(L), rin, rc)


def mc_run(model, path, com, quat, L, rin, rc, beta, sig_t, sig_r, ntrial, seed, chain, counter, energy):
    """One Monte Carlo chain on the CPU (same draws as the device).  Returns com, quat, energy, trace (ntrial,4)."""
    com = np.ascontiguousarray(com, dtype=np.float64).copy()
    quat = np.ascontiguousarray(quat, dtype=np.float64).copy()
    e = np.array([energy], dtype=np.float64)
    trace = np.zeros((ntrial, 4))
    lib().orc_mc_run(MODEL[model], PATH[path], com.shape[0], com, quat, _f64(L), rin, rc, beta, sig_t, sig_r, ntrial,
                     seed, chain, counter, e, trace)
    return com, quat, e[0], trace


OP_EP, OP_Q6, OP_TRIANGLE = 0, 1, 2


def order_parameter(kind, com, L, ref=None, logarithmic=False, energy=0.0):
    """Order parameter of one configuration (kind OP_Q6: local Q6, Q6Local.F90;
    OP_TRIANGLE: divergence of the 4-neighbour angle histogram from ref,
    Triangle.F90; OP_EP: the given energy).  Returns (op, per-molecule q6 (n),
    triangle counts (21))."""
    com = _f64(com)
    n = com.shape[0]
    q6 = np.zeros(n)
    hist = np.zeros(21)
    refv = _f64(np.ones(21) if ref is None else ref)
    op = lib().orc_order_parameter(int(kind), n, com, _f64(L), refv, int(bool(logarithmic)), float(energy), q6, hist)
    return op, q6, hist


def mc_umbrella_run(model, path, com, quat, L, rin, rc, beta, sig_t, sig_r, ntrial, seed, chain, counter, kind, center,
                    coeff, energy, op, ref=None, logarithmic=False):
    """Umbrella Monte Carlo chain on the CPU (same draws as the device).
    Returns com, quat, energy, op, trace (ntrial, 5): dE, energy, accepted, target, op."""
    com = np.ascontiguousarray(com, dtype=np.float64).copy()
    quat = np.ascontiguousarray(quat, dtype=np.float64).copy()
    e = np.array([energy], dtype=np.float64)
    o = np.array([op], dtype=np.float64)
    trace = np.zeros((ntrial, 5))
    refv = _f64(np.ones(21) if ref is None else ref)
    lib().orc_mc_umbrella_run(MODEL[model], PATH[path], com.shape[0], com, quat, _f64(L), rin, rc, beta, sig_t, sig_r,
                              ntrial, seed, chain, counter, int(kind), center, coeff, refv, int(bool(logarithmic)), e, o,
                              trace)
    return com, quat, e[0], o[0], trace


def vreset2(model, n, temp, dt, u):
    """rigid_vreset2 on a given stream of uniforms u (n, 12): returns d1 (n,3) = v*dt and w1 (n,3)."""
    d1 = np.zeros((n, 3)); w1 = np.zeros((n, 3))
    lib().orc_vreset2(MODEL[model], n, temp, dt, _f64(u), d1, w1)
    return d1, w1


def replica_exchange_trial(j, jj, node_in_charge, u, energy, beta, umbrella=None, op=None):
    """Replica.F90:7-73 on temperature slots j, jj (0-based); node_in_charge (int32),
    beta and umbrella (nrep, numbrella, 2) are updated in place.  Returns accept."""
    nb = 0 if umbrella is None else umbrella.shape[1]
    umb = np.zeros(1) if umbrella is None else umbrella
    opv = np.zeros(1) if op is None else _f64(op)
    return bool(lib().orc_replica_exchange_trial(int(j), int(jj), node_in_charge, float(u), _f64(energy), beta, nb,
                                                 umb, opv))


def max_threads() -> int:
    return lib().orc_max_threads()
