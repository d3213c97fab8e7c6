"""Start velocities: rigid_vreset2 (RigidModule.F90:1016-1053) with
Random_Normal (RandomModule.F90:28-36).

The host restatement in genesis6_gb300.config must give the reference's
numbers for a given stream of uniforms (the oracle restates the same two
routines in C++), and the seeded Maxwell-Boltzmann draw used for synthetic
configurations must have the reference's per-axis variances kT/m and kT/I_k."""
import numpy as np

from genesis6_gb300 import config

MODELS = ["TIP4P", "TIP5P", "ST2", "SPCE"]


def test_vreset2_follows_reference_restatement(orc):
    rng = np.random.default_rng(5)
    for model in MODELS:
        info = orc.model_info(model)
        n = 500
        u = 1.0 - rng.random((n, 12))          # Random_GetNext = 1 - x, in (0, 1]
        for temp, dt in ((300.0, 0.002), (260.0, 0.001)):
            d1, w1 = config.rigid_vreset2(temp, info["mass"], info["inertia"], u, dt)
            d1o, w1o = orc.vreset2(model, n, temp, dt, u)
            np.testing.assert_allclose(d1, d1o, rtol=1e-13, atol=0)
            np.testing.assert_allclose(w1, w1o, rtol=1e-13, atol=0)


def test_maxwell_boltzmann_variances(orc):
    n = 200_000
    for model in MODELS:
        info = orc.model_info(model)
        kT = 300.0 * config.RGAS * config.J2I
        v, w = config.maxwell_boltzmann(n, 300.0, info["mass"], info["inertia"], np.random.default_rng(7))
        # the variance of a variance estimate from n normals is 2 var^2 / n: 5 sigma
        tol = 5.0 * np.sqrt(2.0 / n)
        np.testing.assert_allclose(v.var(axis=0), kT / info["mass"], rtol=tol)
        np.testing.assert_allclose(w.var(axis=0), kT / np.asarray(info["inertia"]), rtol=tol)
        assert np.abs(v.mean(axis=0)).max() < 1e-12 * np.sqrt(kT / info["mass"])   # net momentum removed
        # the same variances as the reference formula on a uniform stream
        u = 1.0 - np.random.default_rng(9).random((n, 12))
        d1, w1 = config.rigid_vreset2(300.0, info["mass"], info["inertia"], u, 1.0)
        np.testing.assert_allclose(d1.var(axis=0), kT / info["mass"], rtol=tol)
        np.testing.assert_allclose(w1.var(axis=0), kT / np.asarray(info["inertia"]), rtol=tol)
