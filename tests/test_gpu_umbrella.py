"""Umbrella Monte Carlo on the device (g6_order_parameter, g6_mc_run_umbrella)
against the oracle: the order parameters of a state (local Q6, Q6Local.F90;
triangle-angle divergence, Triangle.F90), FP64 chains that replay the CPU
chain trial by trial with the umbrella in the Metropolis test (mc2.F90:684-722),
and the incrementally updated order parameter of long chains against a
computation from scratch (the reference's own DEBUG3 check, mc2.F90:745-760)."""
import math

import numpy as np
import pytest

import genesis6_gb300 as g6
from genesis6_gb300 import _capi, config

pytestmark = pytest.mark.gpu

BCC_Q6 = 0.628539361054709
KIND = {"ep": 0, "q6": 1, "triangle": 2}
REF = np.random.default_rng(1).uniform(0.5, 2.0, 21)


def _chains(model, nrep, n, seed, prec="fp64", jitter=0.45):
    recs = [config.water_box(model, n, seed + r, jitter=jitter) for r in range(nrep)]
    L = recs[0]["L"][0]
    rc = 0.5 * L
    s = g6.RigidWater(model, [n] * nrep, np.array([b["L"] for b in recs]), path="custom", precision=prec, rc=rc,
                      skin=0.0)
    s.upload_state(np.concatenate([b["rec"] for b in recs]))
    return s, recs, rc


@pytest.mark.parametrize("kind", ["q6", "triangle"])
def test_order_parameter_matches_oracle(orc, kind):
    s, recs, rc = _chains("TIP4P", 3, 343, 21)
    op = s.order_parameter(kind, refhist=REF)
    for c, b in enumerate(recs):
        want = orc.order_parameter(KIND[kind], b["com"], b["L"], ref=REF)[0]
        assert op[c] == pytest.approx(want, rel=1e-12)
    if kind == "triangle":
        op_log = s.order_parameter(kind, refhist=REF, logarithmic=True)
        assert np.allclose(op_log, np.log(op), rtol=1e-14)


def _crystal_system(basis, a, m):
    basis = np.asarray(basis, float)
    cells = np.array([[i, j, k] for i in range(m) for j in range(m) for k in range(m)], float)
    com = ((cells[:, None, :] + basis[None, :, :]) * a).reshape(-1, 3)
    n = len(com)
    rng = np.random.default_rng(3)
    info = _capi.model_info("TIP4P")
    quat = config.random_quaternions(n, rng)
    v, w = config.maxwell_boltzmann(n, 300.0, info["mass"], info["inertia"], rng)
    L = np.full(3, a * m)
    s = g6.RigidWater("TIP4P", [n], L[None, :], path="custom", precision="fp64", rc=0.45 * L[0], skin=0.0)
    s.upload_state(config.rigid_records(com, quat, v, w, 0.002))
    return s


def test_order_parameter_of_a_bcc_crystal():
    s = _crystal_system([[0, 0, 0], [0.5, 0.5, 0.5]], 3.2, 6)   # 8 bonds at 2.77 A per molecule
    assert s.order_parameter("q6")[0] == pytest.approx(BCC_Q6, abs=1e-12)


def test_more_bonds_than_the_reference_holds_is_reported():
    # fcc with nearest neighbours at 2.8 A: 12 bonds per molecule, MAXBOND is 10 (Q6Local.F90:32)
    s = _crystal_system([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]], 2.8 * math.sqrt(2), 4)
    with pytest.raises(_capi.G6Error) as e:
        s.order_parameter("q6")
    assert e.value.status == _capi.G6_ERR_CAPACITY


@pytest.mark.parametrize("kind", ["ep", "q6", "triangle"])
def test_fp64_umbrella_chain_replays_oracle(orc, kind):
    s, recs, rc = _chains("TIP4P", 2, 216, 31)
    beta = 1.0 / 260.0
    ntrial = 200
    E0 = [orc.compute("TIP4P", "custom", b["com"], b["quat"], b["L"], [rc] * 3, rc - 2.0, rc)[2] for b in recs]
    op0 = s.order_parameter(kind, refhist=REF)
    # an umbrella that decides a share of the trials: centre below the current value
    shift, coeff = {"ep": (300.0, 2.0e-3), "q6": (0.02, 3.0e7), "triangle": (0.05, 2.0e5)}[kind]
    center = op0 - shift
    res = s.mc_run_umbrella(ntrial, 99, 0, beta, kind, center, coeff, refhist=REF, trace=True)
    rec_g = s.download_state()
    differs = False
    for c, b in enumerate(recs):
        o0 = E0[c] if kind == "ep" else orc.order_parameter(KIND[kind], b["com"], b["L"], ref=REF)[0]
        com, quat, e, o, tr = orc.mc_umbrella_run("TIP4P", "custom", b["com"], b["quat"], b["L"], rc - 2.0, rc, beta,
                                                  0.15, 0.15, ntrial, 99, c, 0, KIND[kind], center[c], coeff, E0[c],
                                                  o0, ref=REF)
        t = res["trace"][c]
        assert np.array_equal(t[:, 3], tr[:, 3])   # same targets
        assert np.array_equal(t[:, 2], tr[:, 2])   # same decisions
        assert np.abs(t[:, 4] - tr[:, 4]).max() <= 1e-10 * max(1.0, np.abs(tr[:, 4]).max())
        assert res["op"][c] == pytest.approx(o, rel=1e-10)
        assert res["energy"][c] == pytest.approx(e, rel=1e-10)
        sl = rec_g[216 * c:216 * (c + 1)]
        assert np.abs(sl[:, :3] - com).max() < 1e-10
        assert np.abs(sl[:, 33:37] - quat).max() < 1e-10
        _, _, _, plain = orc.mc_run("TIP4P", "custom", b["com"], b["quat"], b["L"], rc - 2.0, rc, beta, 0.15, 0.15,
                                    ntrial, 99, c, 0, E0[c])
        differs |= not np.array_equal(plain[:, 2], tr[:, 2])
    assert differs   # the umbrella changed some decisions


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("kind", ["q6", "triangle"])
def test_incremental_order_parameter_equals_fresh(orc, kind, prec):
    s, recs, rc = _chains("TIP4P", 4, 343, 41, prec=prec)
    op0 = s.order_parameter(kind, refhist=REF)
    res = s.mc_run_umbrella(3000, 5, 0, 1.0 / 260.0, kind, op0, 1.0e3, refhist=REF, sample_every=500)
    assert (res["accepted"] > 300).all()
    fresh = s.order_parameter(kind, refhist=REF)
    tol = 1e-10 if kind == "q6" else 1e-14
    assert np.abs(res["op"] - fresh).max() <= tol * np.abs(fresh).max()
    assert np.array_equal(res["op_samples"][:, -1], res["op"])
    rec = s.download_state()
    for c, b in enumerate(recs):
        want = orc.order_parameter(KIND[kind], rec[343 * c:343 * (c + 1), :3], b["L"], ref=REF)[0]
        assert res["op"][c] == pytest.approx(want, rel=tol * 10)
