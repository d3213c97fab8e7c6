"""One rank of the sharded replica-exchange check (tests/test_replica_sharding.py).

Run by the test as a separate process with RANK, WORLD_SIZE, MASTER_ADDR and
MASTER_PORT set: joins a gloo group, owns a block of a 220-360 K ladder of
replicas, and performs `attempts` exchange attempts with seeded energies,
umbrellas and order parameters (the same global arrays on every rank, each
rank passing its own slice).  Rank 0 writes the global accepted flags of every
attempt and the final beta/temp/umbrellas as JSON."""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def ladder(nrep, attempts, seed=5):
    """Global inputs: temperatures, umbrellas, and per attempt energies and order parameters."""
    temps = 220.0 * (360.0 / 220.0) ** (np.arange(nrep) / (nrep - 1))
    rng = np.random.default_rng(seed)
    umb = np.stack([rng.uniform(0.2, 0.6, (nrep, 2)), rng.uniform(50.0, 400.0, (nrep, 2))], axis=2)
    E = rng.normal(-4.0e6, 3.0e4, (attempts, nrep))
    op = rng.uniform(0.1, 0.7, (attempts, nrep, 2))
    return temps, umb, E, op


def main():
    import torch.distributed as dist
    from genesis6_gb300 import replicas
    out, counts, attempts = sys.argv[1], [int(c) for c in sys.argv[2].split(",")], int(sys.argv[3])
    dist.init_process_group("gloo")
    rank = dist.get_rank()
    ex = replicas.ShardedExchange(counts[rank])
    temps, umb, E, op = ladder(ex.nrep, attempts)
    sl = slice(ex.offset, ex.offset + ex.nlocal)
    beta, temp, u = 1.0 / temps[sl], temps[sl].copy(), umb[sl].copy()
    acc = []
    for a in range(attempts):
        r = ex.attempt(a & 1, 77, 1000 + a, E[a, sl], beta, temp, u, op[a, sl])
        beta, temp, u = r["beta"], r["temp"], r["umbrella"]
        acc.append(r["accepted_global"].tolist())
    final = ex.gather(np.column_stack([beta, temp, u.reshape(ex.nlocal, -1)]))
    if rank == 0:
        with open(out, "w") as f:
            json.dump({"accepted": acc, "final": final.tolist(), "nrep": ex.nrep, "offsets_ok": True}, f)
    dist.destroy_process_group()


if __name__ == "__main__":
    main()
