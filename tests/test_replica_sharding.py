"""Replica exchange over several processes, on CPU (gloo).

The decision routine g6_exchange_plan (host code of libg6gpu.so) must follow
replica_exchange_trial (Replica.F90:7-73) as the drivers apply it
(node_in_charge over temperature slots, Mixture.F90:1589-1653;
mc2.F90:950-1001 with umbrellas), restated in the oracle; and an ensemble split
over 2 gloo ranks (ShardedExchange: gather, the same plan on every rank, each
rank keeps its slice) must make exactly the decisions of one process holding
all replicas.  No GPU is needed: the plan is host code."""
import json
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

from genesis6_gb300 import replicas

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import _replica_worker as worker  # noqa: E402


def oracle_attempt(orc, parity, seed, counter, E, beta, temp, umb=None, op=None):
    """One attempt by the oracle's restatement: slots = replicas by decreasing
    beta (node_in_charge), pairs (j, j+1) with j % 2 == parity, uniform of
    Philox (seed; j, counter, 0x52)."""
    beta = beta.copy(); temp = temp.copy()
    umb = None if umb is None else umb.copy()
    n = len(E)
    nic = np.array(sorted(range(n), key=lambda r: (-beta[r], r)), dtype=np.int32)
    acc = np.zeros(n, dtype=np.int32)
    scale = np.ones(n)
    for j in range(parity, n - 1, 2):
        n0, n1 = nic[j], nic[j + 1]
        u = orc.philox_uniform2(seed, j, counter & 0xffffffff, counter >> 32, 0x52)[0]
        a = orc.replica_exchange_trial(j, j + 1, nic, u, E, beta, umb, op)
        acc[n0] = int(a)
        if a:
            scale[n0] = np.sqrt(temp[n1] / temp[n0]); scale[n1] = np.sqrt(temp[n0] / temp[n1])
            temp[n0], temp[n1] = temp[n1], temp[n0]
    return beta, temp, umb, scale, acc


@pytest.mark.parametrize("with_umbrella", [False, True])
def test_plan_follows_replica_trial(orc, with_umbrella):
    rng = np.random.default_rng(3)
    n = 9
    temps = 220.0 * (360.0 / 220.0) ** (np.arange(n) / (n - 1))
    perm = rng.permutation(n)              # a ladder already shuffled by earlier swaps
    temp = temps[perm]
    beta = 1.0 / temp
    umb = np.stack([rng.uniform(0.2, 0.6, (n, 2)), rng.uniform(50.0, 400.0, (n, 2))], axis=2) if with_umbrella else None
    total = 0
    for a in range(40):
        E = rng.normal(-4.0e6, 3.0e4, n)
        op = rng.uniform(0.1, 0.7, (n, 2)) if with_umbrella else None
        p = replicas.exchange_plan(a & 1, 11, (7 << 32) + a, E, beta, temp, umb, op)
        ob, ot, ou, osc, oa = oracle_attempt(orc, a & 1, 11, (7 << 32) + a, E, beta, temp, umb, op)
        assert np.array_equal(p["accepted"], oa)
        assert np.array_equal(p["beta"], ob) and np.array_equal(p["temp"], ot)
        np.testing.assert_allclose(p["scale"], osc, rtol=1e-15)
        if with_umbrella:
            assert np.array_equal(p["umbrella"], ou)
        beta, temp, umb = p["beta"], p["temp"], p["umbrella"]
        total += int(oa.sum())
    assert 5 < total < 40 * (n // 2)      # both outcomes occur


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _run_ranks(tmp_path, counts, attempts):
    out = str(tmp_path / "rank0.json")
    port = _free_port()
    procs = []
    for rank in range(len(counts)):
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE=str(len(counts)), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, os.path.join(HERE, "_replica_worker.py"), out,
                                       ",".join(map(str, counts)), str(attempts)], env=env))
    for p in procs:
        assert p.wait(timeout=300) == 0
    with open(out) as f:
        return json.load(f)


@pytest.mark.parametrize("counts", [[4, 4], [3, 5]])
def test_two_ranks_equal_one_process(tmp_path, counts):
    attempts = 24
    res = _run_ranks(tmp_path, counts, attempts)
    nrep = sum(counts)
    assert res["nrep"] == nrep
    temps, umb, E, op = worker.ladder(nrep, attempts)
    beta, temp, u = 1.0 / temps, temps.copy(), umb.copy()
    for a in range(attempts):
        p = replicas.exchange_plan(a & 1, 77, 1000 + a, E[a], beta, temp, u, op[a])
        assert res["accepted"][a] == p["accepted"].tolist(), a
        beta, temp, u = p["beta"], p["temp"], p["umbrella"]
    final = np.asarray(res["final"])
    assert np.array_equal(final[:, 0], beta) and np.array_equal(final[:, 1], temp)
    assert np.array_equal(final[:, 2:], u.reshape(nrep, -1))
    assert sum(map(sum, res["accepted"])) > 0
