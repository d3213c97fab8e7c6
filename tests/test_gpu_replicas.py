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


def test_umbrella_exchange_follows_replica_trial():
    """Replica.F90:20-62 with two parabolic umbrellas per replica (Umbrella.F90:11-16):
    the umbrella potentials enter both sides of the test and move with beta."""
    temps = [280.0, 300.0, 320.0, 340.0, 360.0, 380.0]
    s = _replicas([216, 230, 216, 240, 220, 216], temps, 41)
    th = s.thermostats(6, "andersen", temp=temps, rate=2.0, seed=5)
    log = s.md_run(0.002, 30, th)
    E = log[-1, :, 0]
    rng = np.random.default_rng(8)
    umb = np.stack([rng.uniform(0.2, 0.6, (6, 2)), rng.uniform(50.0, 400.0, (6, 2))], axis=2)   # (center, coeffi)
    op = rng.uniform(0.1, 0.7, (6, 2))
    beta0 = 1.0 / np.array(temps)
    import oracle
    I2J, J2K = 10.0, 0.120273
    pot = lambda u, o: u[1] * ((o - u[0]) * (o - u[0]))
    for parity in (1, 0):
        beta, acc, umb_new = s.replica_exchange(parity, 77, 9 + parity, beta0.copy(), th, umbrella=umb, op=op)
        for r in range(parity, 5, 2):
            a0, a1 = E[r], E[r + 1]
            for k in range(2):
                a0 = a0 + pot(umb[r, k], op[r, k]); a1 = a1 + pot(umb[r + 1, k], op[r + 1, k])
            acc0 = -(a0 * beta0[r] + a1 * beta0[r + 1]) * I2J * J2K
            b0, b1 = E[r], E[r + 1]
            for k in range(2):
                b0 = b0 + pot(umb[r + 1, k], op[r, k]); b1 = b1 + pot(umb[r, k], op[r + 1, k])
            acc1 = -(b0 * beta0[r + 1] + b1 * beta0[r]) * I2J * J2K
            u = oracle.philox_uniform2(77, r, 9 + parity, 0, 0x52)[0]
            want = acc0 < acc1 or u < math.exp(acc1 - acc0)
            assert bool(acc[r]) == want, (parity, r)
            if want:
                assert np.array_equal(umb_new[r], umb[r + 1]) and np.array_equal(umb_new[r + 1], umb[r])
                assert beta[r] == beta0[r + 1]
            else:
                assert np.array_equal(umb_new[r], umb[r]) and beta[r] == beta0[r]
        # the exchange changed temperatures; restore them for the other parity's check
        for r in range(6):
            th[r].temp = temps[r]
