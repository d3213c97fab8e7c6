"""Equilibrated start of the 4,096-molecule TIP4P benchmark workload.

Both arms of bench.py (the CUDA library and the CPU restatement of the
reference timed on the host cores) start from this state, so that they time
the same liquid and their first-step energies can be compared.  Workload:
4,096 rigid TIP4P waters at 1.0 g/cm^3 (L = 49.655 A), the seeded lattice
start of genesis6_gb300.config (seed 20261203, Maxwell-Boltzmann 300 K), then
2,000 steps of Gear MD at rc 9 A with the 2 A switch, dt 2 fs, computed in FP64
by the oracle (Mixture.F90:1789-2290 step order, StdForce arithmetic): 1,500
steps in blocks of 50 with the Nose-Hoover thermostat at 300 K (tau 0.1 ps),
the velocities rescaled to 300 K and zeta reset between blocks (the melting
lattice releases ~10 kJ/mol per molecule, which a free Nose-Hoover run turns
into a temperature swing of several hundred K), then 500 free Nose-Hoover
steps at tau 0.5 ps.

Stored (tip4p4096_eq.npz): box edges L (3), centre of mass com (n,3),
quaternion quat (n,4), the first Gear term of the centre of mass d1 (n,3) =
velocity * dt and the body-frame angular velocity w1 (n,3).  The higher Gear
terms start at zero, as in a Genesis6 run started from @NX4A plus velocities.

Run:  python tests/golden/make_equilibrated.py   (about a minute on 8 cores)
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

N, SEED, TEMP, DT, RC, SWITCH, TAU, STEPS = 4096, 20261203, 300.0, 0.002, 9.0, 2.0, 0.5, 2000
OUT = os.path.join(HERE, "tip4p4096_eq.npz")


def main():
    import oracle
    from genesis6_gb300 import config
    info = oracle.model_info("TIP4P")
    b = config.water_box("TIP4P", N, SEED, temp=TEMP, dt=DT, info=info)
    threads = os.cpu_count() or 1
    rec = b["rec"]
    t0 = time.perf_counter()
    for _ in range(1500 // 50):
        th = np.array([1, TEMP * 0.1 ** 2 / DT, 0.0, TEMP, 0, 0, 0, 0, 0, 0], float)
        rec, th, log = oracle.md_run_threaded("TIP4P", rec, b["L"], [RC] * 3, RC - SWITCH, RC, DT, 50, th, threads)
        ekt, ekr = oracle.kinetic("TIP4P", rec, DT)
        temp = 10.0 * 2.0 * (ekt + ekr) / (6.0225e23 * 1.380066e-23 * 6.0 * N)   # I2J 2 Ek / (RGAS dof)
        f = np.sqrt(TEMP / temp)
        rec[:, 3:6] *= f
        rec[:, 18:21] *= f
    th = np.array([1, TEMP * TAU ** 2 / DT, 0.0, TEMP, 0, 0, 0, 0, 0, 0], float)
    rec, th, log = oracle.md_run_threaded("TIP4P", rec, b["L"], [RC] * 3, RC - SWITCH, RC, DT, STEPS - 1500, th,
                                          threads)
    wall = time.perf_counter() - t0
    np.savez_compressed(OUT, L=np.asarray(b["L"], float), com=rec[:, 0:3], quat=rec[:, 33:37], d1=rec[:, 3:6],
                        w1=rec[:, 18:21], dt=np.array(DT))
    print("wrote %s: %d steps in %.1f s; last 500 steps: T %.1f K (last %.1f K), Epot per molecule %.2f kJ/mol"
          % (OUT, STEPS, wall, log[:, 3].mean(), log[-1, 3], log[:, 0].mean() / N * 1e-2))


if __name__ == "__main__":
    main()
