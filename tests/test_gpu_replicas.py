"""Replica ensembles on one GPU: uneven replicas in one context, the
stochastic-collision thermostat, and the replica-exchange acceptance test of
Replica.F90:7-73 with the MD side effects of Mixture.F90:1616-1653."""
import math

import numpy as np
import pytest

import genesis6_gb300 as g6
from genesis6_gb300 import config

pytestmark = pytest.mark.gpu


def _replicas(sizes, temps, seed):
    boxes, recs = [], []
    for k, (n, t) in enumerate(zip(sizes, temps)):
        b = config.water_box("TIP4P", n, seed + k, temp=t, dt=0.002, jitter=0.2)
        boxes.append(b["L"]); recs.append(b["rec"])
    s = g6.RigidWater("TIP4P", sizes, np.array(boxes), path="custom", precision="mixed", rc=8.5)
    s.upload_state(np.concatenate(recs))
    return s


def test_collision_thermostat_reaches_targets():
    temps = [240.0, 300.0, 360.0]
    s = _replicas([216, 300, 260], temps, 7)
    th = s.thermostats(3, "andersen", temp=temps, rate=5.0, seed=11)
    # the lattice start keeps releasing potential energy for a few ps
    s.md_run(0.002, 2500, th, log=False)
    log = s.md_run(0.002, 2500, th)
    T = log[:, :, 3].mean(0)
    for k in range(3):
        assert abs(T[k] - temps[k]) < 0.04 * temps[k], (T, temps)


def test_exchange_follows_replica_trial():
    temps = [280.0, 300.0, 320.0, 340.0]
    s = _replicas([216, 216, 250, 230], temps, 21)
    th = s.thermostats(4, "andersen", temp=temps, rate=2.0, seed=3)
    log = s.md_run(0.002, 50, th)
    E = log[-1, :, 0]
    rec0 = s.download_state()
    beta0 = 1.0 / np.array(temps)
    import oracle
    beta, acc = s.replica_exchange(0, 99, 5, beta0.copy(), th)
    I2J, J2K = 10.0, 0.120273
    for r in (0, 2):
        a0 = -(E[r] * beta0[r] + E[r + 1] * beta0[r + 1]) * I2J * J2K
        a1 = -(E[r] * beta0[r + 1] + E[r + 1] * beta0[r]) * I2J * J2K
        u = oracle.philox_uniform2(99, r, 5, 0, 0x52)[0]
        want = a0 < a1 or u < math.exp(a1 - a0)
        assert bool(acc[r]) == want
        if want:
            assert beta[r] == beta0[r + 1] and beta[r + 1] == beta0[r]
            assert th[r].temp == temps[r + 1] and th[r + 1].temp == temps[r]
            assert th[r].zeta[0] == 0.0
        else:
            assert beta[r] == beta0[r] and th[r].temp == temps[r]
    # velocities of a swapped replica are scaled by sqrt(T'/T) (Rigid_ScaleVelocity)
    rec1 = s.download_state()
    off = np.concatenate([[0], np.cumsum([216, 216, 250, 230])])
    for r in range(4):
        sl = slice(off[r], off[r + 1])
        p = r if r % 2 == 0 else r - 1
        f = math.sqrt(temps[r + 1 if r % 2 == 0 else r - 1] / temps[r]) if acc[p] else 1.0
        assert np.allclose(rec1[sl, 3:6], f * rec0[sl, 3:6], rtol=1e-14, atol=0)
        assert np.allclose(rec1[sl, 18:21], f * rec0[sl, 18:21], rtol=1e-14, atol=0)
