"""Host-side owner of one device system (one g6_ctx).

``RigidWater`` mirrors the set-up the reference drivers perform (Mixture.F90
and mc2.F90: model constructor + @BOX3 + @RCOA + @VOXA, then the per-step force
path) on top of the C ABI.  All compute goes through libg6gpu.so; there is no
CPU fallback: without a GPU, ``RigidWater(...)`` raises G6Error.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi
from ._capi import G6Error, Thermostat, dptr, iptr


class RigidWater:
    """nrep replicas of one rigid water model on one GPU."""

    def __init__(self, model: str, nmol, box, *, path: str = "custom", precision: str = "fp64", rc: float = 9.0,
                 switch: float = 2.0, cell_edge: float = 0.0, skin: float = 1.0, device: int = 0):
        self.L = _capi.lib()
        self.model = model
        self.path = path
        self.precision = precision
        nmol = np.atleast_1d(np.asarray(nmol, dtype=np.int32))
        box = np.ascontiguousarray(np.asarray(box, dtype=np.float64).reshape(len(nmol), 3))
        self.nmol = nmol
        self.box = box
        self.nrep = len(nmol)
        self.n = int(nmol.sum())
        self.rc = float(rc)
        self.rin = float(rc - switch)
        ptr = ctypes.c_void_p()
        st = self.L.g6_ctx_create(device, ctypes.byref(ptr))
        if st != _capi.G6_OK:
            raise G6Error(st, "g6_ctx_create(%d) failed (no usable CUDA device?)" % device)
        self.ctx = ptr
        self._check(self.L.g6_system(self.ctx, _capi.MODELS[model], _capi.PATHS[path],
                                     _capi.PRECISIONS[precision], self.nrep, iptr(np.ascontiguousarray(nmol)),
                                     dptr(box)))
        self._check(self.L.g6_set_cutoff(self.ctx, self.rin, self.rc))   # cutoff_initialize(in, out)
        self._check(self.L.g6_set_grid(self.ctx, float(cell_edge)))
        self._check(self.L.g6_set_skin(self.ctx, float(skin)))
        self.info = _capi.model_info(model)

    # -- plumbing -------------------------------------------------------
    def _check(self, status):
        if status != _capi.G6_OK:
            msg = self.L.g6_last_error(self.ctx).decode() if getattr(self, "ctx", None) else ""
            raise G6Error(status, msg)

    def close(self):
        if getattr(self, "ctx", None):
            self.L.g6_ctx_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- state ----------------------------------------------------------
    def upload_state(self, rec):
        rec = np.ascontiguousarray(rec, dtype=np.float64)
        assert rec.shape == (self.n, _capi.REC)
        self._check(self.L.g6_upload_state(self.ctx, dptr(rec)))

    def download_state(self):
        rec = np.zeros((self.n, _capi.REC))
        self._check(self.L.g6_download_state(self.ctx, dptr(rec)))
        return rec

    def upload_poses(self, com, quat):
        com = np.ascontiguousarray(com, dtype=np.float64)
        quat = np.ascontiguousarray(quat, dtype=np.float64)
        self._check(self.L.g6_upload_poses(self.ctx, dptr(com), dptr(quat)))

    # -- parity surface ---------------------------------------------------
    def cells(self):
        c = np.zeros(self.n, dtype=np.int32)
        self._check(self.L.g6_cells(self.ctx, iptr(c)))
        return c

    def pairsearch(self):
        npair = ctypes.c_int64()
        self._check(self.L.g6_pairsearch(self.ctx, ctypes.byref(npair)))
        m = npair.value
        pi = np.zeros(max(m, 1), np.int32); pj = np.zeros(max(m, 1), np.int32)
        ox, oy, oz, hh, dh = (np.zeros(max(m, 1)) for _ in range(5))
        self._check(self.L.g6_get_pairs(self.ctx, m, iptr(pi), iptr(pj), dptr(ox), dptr(oy), dptr(oz), dptr(hh),
                                        dptr(dh)))
        s = slice(0, m)
        return dict(i=pi[s], j=pj[s], ox=ox[s], oy=oy[s], oz=oz[s], hh=hh[s], dh=dh[s])

    def force(self):
        """F (n,3), body torque (n,3), epot (nrep,), virial (nrep,3,3)."""
        F = np.zeros((self.n, 3)); tau = np.zeros((self.n, 3))
        ep = np.zeros(self.nrep); vir = np.zeros((self.nrep, 9))
        self._check(self.L.g6_force(self.ctx, dptr(F), dptr(tau), dptr(ep), dptr(vir)))
        return F, tau, ep, vir.reshape(self.nrep, 3, 3)

    def step_forces(self):
        """The mixed MD step's pair-kernel forces on the uploaded poses (its
        list form and lanes): F (n,3), body torque (n,3), epot (nrep,)."""
        F = np.zeros((self.n, 3)); tau = np.zeros((self.n, 3))
        ep = np.zeros(self.nrep)
        self._check(self.L.g6_step_forces(self.ctx, dptr(F), dptr(tau), dptr(ep)))
        return F, tau, ep

    def molecule_energies(self):
        e = np.zeros(self.n)
        self._check(self.L.g6_molecule_energies(self.ctx, dptr(e)))
        return e

    def hbonds(self):
        """Hydrogen bonds by O-H distance (interaction_hb_by_oh_distance,
        InteractionModule.F90:682-777): donor, hydrogen (1, 2), acceptor for
        each pair that forms one (0-based molecules), as an (m, 3) array."""
        cap = 4 * self.n
        while True:
            f = np.zeros(cap, np.int32); w = np.zeros(cap, np.int32); t = np.zeros(cap, np.int32)
            nb = ctypes.c_int64()
            self._check(self.L.g6_hbonds(self.ctx, cap, iptr(f), iptr(w), iptr(t), ctypes.byref(nb)))
            if nb.value <= cap:
                break
            cap = nb.value
        out = np.stack([f[:nb.value], w[:nb.value], t[:nb.value]], axis=1)
        return out[np.lexsort((out[:, 2], out[:, 0]))]   # by donor, then acceptor

    def rdf_counts(self, nbin, binwidth, minvalue=0.0):
        """Site-site distance counts of the uploaded poses (radialdistrib,
        RDFModule.F90:101-137): (nrep, nsite, nsite, nbin) int64, site pair
        a <= b counted over both orders of each molecule pair within the cutoff."""
        ns = self.info["nsite"]
        h = np.zeros((self.nrep, ns, ns, int(nbin)), dtype=np.int64)
        self._check(self.L.g6_rdf(self.ctx, int(nbin), float(binwidth), float(minvalue),
                                  h.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))))
        return h

    # -- dynamics ---------------------------------------------------------
    @staticmethod
    def thermostats(nrep, kind="nve", temp=300.0, q=0.0, dump=0.0, rate=0.0, seed=0):
        arr = (Thermostat * nrep)()
        kinds = {"nve": _capi.NVE, "nose": _capi.NOSE, "andersen": _capi.ANDERSEN}
        temps = np.broadcast_to(np.asarray(temp, dtype=np.float64), (nrep,))
        for r in range(nrep):
            arr[r].kind = kinds[kind]
            arr[r].temp = float(temps[r]); arr[r].q = q; arr[r].dump = dump
            arr[r].collision_rate = rate; arr[r].seed = seed
        return arr

    def md_run(self, dt, nsteps, thermo=None, log=True):
        if thermo is None:
            thermo = self.thermostats(self.nrep)
        buf = np.zeros((nsteps, self.nrep, _capi.LOG_WIDTH)) if log else None
        self._check(self.L.g6_md_run(self.ctx, float(dt), int(nsteps), thermo, dptr(buf)))
        return buf

    def md_step_host(self, dt, rec, thermo=None, log=None):
        if thermo is None:
            thermo = self.thermostats(self.nrep)
        for a in (rec, log):
            if a is not None and (a.dtype != np.float64 or not a.flags.c_contiguous):
                raise ValueError("rec and log must be C-contiguous float64 arrays")
        adr = lambda a: None if a is None else a.__array_interface__["data"][0]
        self._check(self.L.md_step_host_addr(self.ctx, float(dt), ctypes.addressof(thermo), adr(rec), adr(log)))
        return rec

    # -- Monte Carlo (mc2.F90 trial/accept loop, one chain per replica) --------
    def mc_run(self, ntrial, seed, counter, beta, sigma_t=0.15, sigma_r=0.15, mode="plain", sample_every=0,
               trace=False):
        """`ntrial` single-molecule trials on every chain.  beta, sigma_t, sigma_r
        are scalars or per-chain arrays; mode is "plain" (fixed widths),
        "learned" (widths from the network) or "collect" (fixed widths, training
        records kept on the device).  Returns a dict with accepted/trial counts,
        the running energies, the energy every `sample_every` trials and, with
        trace=True, (dE, energy, accepted, target) per trial."""
        R = self.nrep
        per = lambda v: np.ascontiguousarray(np.broadcast_to(np.asarray(v, dtype=np.float64), (R,)))
        beta, st, sr = per(beta), per(sigma_t), per(sigma_r)
        modes = {"plain": _capi.MC_PLAIN, "learned": _capi.MC_LEARNED, "collect": _capi.MC_COLLECT}
        counts = np.zeros(2 * R, np.int64)
        energy = np.zeros(R)
        nsm = ntrial // sample_every if sample_every else 0
        samples = np.zeros((R, max(nsm, 1)))
        tr = np.zeros((R, ntrial, 4)) if trace else None
        self._check(self.L.g6_mc_run(self.ctx, int(ntrial), int(seed), int(counter), dptr(beta), dptr(st), dptr(sr),
                                     modes[mode], int(sample_every), dptr(samples) if nsm else None,
                                     counts.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), dptr(energy), dptr(tr)))
        return {"accepted": counts[0::2].copy(), "trials": counts[1::2].copy(), "energy": energy,
                "samples": samples[:, :nsm], "trace": tr}

    _OP_KINDS = {"ep": _capi.OP_EP, "q6": _capi.OP_Q6, "triangle": _capi.OP_TRIANGLE}

    def order_parameter(self, kind, refhist=None, logarithmic=False):
        """Order parameter of every chain at the current state (g6_order_parameter):
        kind "q6" (local Q6, Q6Local.F90), "triangle" (divergence of the
        4-neighbour angle histogram from refhist, Triangle.F90) or "ep"."""
        op = np.zeros(self.nrep)
        ref = None if refhist is None else np.ascontiguousarray(refhist, dtype=np.float64)
        self._check(self.L.g6_order_parameter(self.ctx, self._OP_KINDS[kind], dptr(ref), int(bool(logarithmic)),
                                              dptr(op)))
        return op

    def mc_run_umbrella(self, ntrial, seed, counter, beta, kind, center, coeff, sigma_t=0.15, sigma_r=0.15,
                        refhist=None, logarithmic=False, sample_every=0, trace=False):
        """Umbrella Monte Carlo (g6_mc_run_umbrella): fixed-width trials with
        coeff (op - center)^2 on the order parameter `kind` added to dE in the
        Metropolis test (mc2.F90:684-722).  center, coeff and the other
        parameters are scalars or per-chain arrays.  Returns accepted/trial
        counts, energies, final order parameters, sampled energies and order
        parameters and, with trace=True, (dE, energy, accepted, target, op) per
        trial."""
        R = self.nrep
        per = lambda v: np.ascontiguousarray(np.broadcast_to(np.asarray(v, dtype=np.float64), (R,)))
        beta, st, sr = per(beta), per(sigma_t), per(sigma_r)
        umb = np.ascontiguousarray(np.stack([per(center), per(coeff)], axis=1))
        ref = None if refhist is None else np.ascontiguousarray(refhist, dtype=np.float64)
        counts = np.zeros(2 * R, np.int64)
        energy = np.zeros(R)
        op = np.zeros(R)
        nsm = ntrial // sample_every if sample_every else 0
        samples = np.zeros((R, max(nsm, 1)))
        opsamp = np.zeros((R, max(nsm, 1)))
        tr = np.zeros((R, ntrial, 5)) if trace else None
        self._check(self.L.g6_mc_run_umbrella(
            self.ctx, int(ntrial), int(seed), int(counter), dptr(beta), dptr(st), dptr(sr), self._OP_KINDS[kind],
            dptr(umb), dptr(ref), int(bool(logarithmic)), dptr(op), int(sample_every), dptr(samples) if nsm else None,
            dptr(opsamp) if nsm else None, counts.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), dptr(energy),
            dptr(tr)))
        return {"accepted": counts[0::2].copy(), "trials": counts[1::2].copy(), "energy": energy, "op": op,
                "samples": samples[:, :nsm], "op_samples": opsamp[:, :nsm], "trace": tr}

    def last_epot(self):
        """Potential energy of each replica at the last MD step (g6_last_epot)."""
        e = np.zeros(self.nrep)
        self._check(self.L.g6_last_epot(self.ctx, dptr(e)))
        return e

    def replica_scale(self, scale):
        """Scale every replica's COM and angular velocities (g6_replica_scale)."""
        scale = np.ascontiguousarray(scale, dtype=np.float64)
        self._check(self.L.g6_replica_scale(self.ctx, dptr(scale)))

    def replica_exchange(self, parity, seed, counter, beta, thermo, umbrella=None, op=None):
        """Neighbour exchange (Replica.F90:7-73).  With umbrella (nrep, k, 2) =
        (center, coeffi) and op (nrep, k), the umbrella-aware test; the umbrellas
        are swapped with beta on acceptance and returned as well."""
        beta = np.ascontiguousarray(beta, dtype=np.float64)
        acc = np.zeros(self.nrep, np.int32)
        if umbrella is None:
            self._check(self.L.g6_replica_exchange(self.ctx, int(parity), int(seed), int(counter), dptr(beta),
                                                   thermo, iptr(acc)))
            return beta, acc
        umb = np.ascontiguousarray(umbrella, dtype=np.float64).reshape(self.nrep, -1, 2).copy()
        opv = np.ascontiguousarray(op, dtype=np.float64).reshape(self.nrep, umb.shape[1])
        self._check(self.L.g6_replica_exchange_umbrella(self.ctx, int(parity), int(seed), int(counter), dptr(beta),
                                                        thermo, umb.shape[1], dptr(umb), dptr(opv), iptr(acc)))
        return beta, acc, umb
