"""Replica exchange for ensembles spread over several processes (one GPU each).

Genesis6 runs one replica per process and exchanges temperatures through
FakeMPI: every process sends (E, beta) to rank 0 (fakempif_gather), rank 0
tests neighbouring temperature slots with replica_exchange_trial and sends the
new beta back (fakempif_scatter); Mixture.F90:1583-1653 (MD) and
mc2.F90:901-1001 (Monte Carlo, with umbrellas).  Here each process owns a
contiguous block of the global replica list (rank-major order), usually all
the replicas of one g6 context on its GPU.  At an exchange every rank gathers
the (E, beta, T, umbrella, order parameter) of all replicas, and all ranks run
the same decision routine (g6_exchange_plan, host code of libg6gpu.so, the
draws of g6_replica_exchange) on the same gathered arrays, so they agree
without a broadcast; each rank then applies its own slice: beta and the
thermostat temperature, velocities scaled by sqrt(T_new/T_old)
(Rigid_ScaleVelocity) and the Nose zeta reset for a replica whose temperature
changed.  The only communication is the gather of a few doubles per replica.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi
from ._capi import G6Error, dptr


def exchange_plan(parity, seed, counter, epot, beta, temp, umbrella=None, op=None):
    """g6_exchange_plan on global arrays.  Returns a dict with the new beta,
    temp and umbrella, the velocity factors `scale` and `accepted` (1 for the
    replica in the lower slot of each accepted pair)."""
    L = _capi.lib()
    epot = np.ascontiguousarray(epot, dtype=np.float64)
    n = len(epot)
    beta = np.array(beta, dtype=np.float64)
    temp = np.array(temp, dtype=np.float64)
    nb = 0
    umb = None
    opv = None
    if umbrella is not None:
        umb = np.array(umbrella, dtype=np.float64).reshape(n, -1, 2)
        nb = umb.shape[1]
        umb = np.ascontiguousarray(umb)
        opv = np.ascontiguousarray(op, dtype=np.float64).reshape(n, nb)
    scale = np.ones(n)
    acc = np.zeros(n, dtype=np.int32)
    st = L.g6_exchange_plan(n, int(parity), ctypes.c_uint64(seed), ctypes.c_uint64(counter), dptr(epot), dptr(beta),
                            dptr(temp), nb, dptr(umb), dptr(opv), dptr(scale),
                            acc.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    if st != _capi.G6_OK:
        raise G6Error(st, "g6_exchange_plan: bad arguments")
    return {"beta": beta, "temp": temp, "umbrella": umb, "scale": scale, "accepted": acc}


class ShardedExchange:
    """Replica exchange over the ranks of a torch.distributed process group
    (gloo, or any backend whose all_gather_object works for small host data).
    ``nlocal`` replicas live on this rank; rank r's replicas follow rank r-1's
    in the global order, which is the order of the temperature ladder at the
    start (slots are re-derived from beta at every attempt)."""

    def __init__(self, nlocal: int, group=None):
        import torch.distributed as dist
        self.dist = dist
        self.group = group
        self.rank = dist.get_rank(group)
        self.world = dist.get_world_size(group)
        counts = [None] * self.world
        dist.all_gather_object(counts, int(nlocal), group=group)
        self.counts = [int(c) for c in counts]
        self.offset = int(sum(self.counts[:self.rank]))
        self.nlocal = int(nlocal)
        self.nrep = int(sum(self.counts))

    def gather(self, local) -> np.ndarray:
        """Concatenation over ranks (rank order) of every rank's local rows."""
        parts = [None] * self.world
        self.dist.all_gather_object(parts, np.asarray(local, dtype=np.float64), group=self.group)
        return np.concatenate([np.asarray(p, dtype=np.float64) for p in parts], axis=0)

    def attempt(self, parity, seed, counter, epot, beta, temp, umbrella=None, op=None):
        """One exchange attempt.  epot, beta, temp (and umbrella (nlocal, nb, 2),
        op (nlocal, nb)) are this rank's replicas.  Returns this rank's slice of
        the plan (beta, temp, umbrella, scale, accepted) and the global
        accepted flags."""
        cols = [np.asarray(epot, float), np.asarray(beta, float), np.asarray(temp, float)]
        nb = 0
        if umbrella is not None:
            u = np.asarray(umbrella, float).reshape(self.nlocal, -1, 2)
            nb = u.shape[1]
            cols += [u.reshape(self.nlocal, -1), np.asarray(op, float).reshape(self.nlocal, nb)]
        rows = np.column_stack([c.reshape(self.nlocal, -1) for c in cols])
        g = self.gather(rows)
        ge, gb, gt = g[:, 0], g[:, 1], g[:, 2]
        gu = g[:, 3:3 + 2 * nb].reshape(-1, nb, 2) if nb else None
        go = g[:, 3 + 2 * nb:3 + 3 * nb] if nb else None
        plan = exchange_plan(parity, seed, counter, ge, gb, gt, gu, go)
        sl = slice(self.offset, self.offset + self.nlocal)
        out = {k: (None if v is None else v[sl].copy()) for k, v in plan.items()}
        out["accepted_global"] = plan["accepted"]
        return out


def apply_exchange(system, thermo, result):
    """Apply this rank's slice of an exchange to a RigidWater context and its
    thermostats: velocities scaled (g6_replica_scale), thermostat targets set,
    Nose zeta reset where the temperature changed (Mixture.F90:1626-1653)."""
    scale = np.ascontiguousarray(result["scale"], dtype=np.float64)
    if np.any(scale != 1.0):
        system.replica_scale(scale)
    for r in range(len(scale)):
        if thermo[r].temp != result["temp"][r]:
            thermo[r].temp = float(result["temp"][r])
            for k in range(5):
                thermo[r].zeta[k] = 0.0
