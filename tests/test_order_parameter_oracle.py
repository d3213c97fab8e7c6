"""Order parameters of umbrella Monte Carlo in the oracle: local Q6
(Q6Local.F90 sq6system_prepareall :98-223, q6.F90 qlm/ylm/plgndr), the
triangle-angle histogram and its Kullback divergence (Triangle.F90
sTriangle_prepareall :53-100, DistribModule.F90 histogram_accumulate and
kullback_div :304-326), and the umbrella chain (mc2.F90:684-722).

Pins that do not come from the oracle's own arithmetic: Steinhardt's q6 of the
fcc (12 directions) and bcc (8 directions) nearest-neighbour shells, which the
local Q6 of a perfect crystal must equal at every molecule (each neighbourhood
is symmetric under the cubic point group, so its bond directions are one
orbit), recomputed here from scipy's spherical harmonics when scipy is
present; and the hand-counted angle histogram of an orthorhombic lattice with
its divergence in closed form."""
import math

import numpy as np
import pytest

from genesis6_gb300 import config

FCC_Q6 = 0.5745242597140697   # Steinhardt q6 of the 12 <110> directions
BCC_Q6 = 0.628539361054709    # Steinhardt q6 of the 8 <111> directions


def _crystal(basis, a, m):
    basis = np.asarray(basis, float)
    cells = np.array([[i, j, k] for i in range(m) for j in range(m) for k in range(m)], float)
    return ((cells[:, None, :] + basis[None, :, :]) * a).reshape(-1, 3), np.full(3, a * m)


def test_q6_closed_forms_from_spherical_harmonics():
    special = pytest.importorskip("scipy.special")
    import itertools

    def q6(dirs):
        d = np.asarray(dirs, float)
        d /= np.linalg.norm(d, axis=1)[:, None]
        th, ph = np.arccos(d[:, 2]), np.arctan2(d[:, 1], d[:, 0])
        if hasattr(special, "sph_harm_y"):
            y = [special.sph_harm_y(6, m, th, ph) for m in range(-6, 7)]
        else:   # older scipy: sph_harm(m, l, azimuth, polar)
            y = [special.sph_harm(m, 6, ph, th) for m in range(-6, 7)]
        return math.sqrt(4 * math.pi / 13 * sum(abs(np.mean(v)) ** 2 for v in y))

    bcc = list(itertools.product([-1, 1], repeat=3))
    fcc = [v for v in itertools.product([-1, 0, 1], repeat=3) if sum(map(abs, v)) == 2]
    assert q6(fcc) == pytest.approx(FCC_Q6, abs=1e-13)
    assert q6(bcc) == pytest.approx(BCC_Q6, abs=1e-13)


@pytest.mark.parametrize("lattice", ["fcc", "bcc"])
def test_q6_of_perfect_crystals(orc, lattice):
    if lattice == "fcc":   # nearest neighbours at 2.8 A (bonds), next shell at 3.96 A
        com, L = _crystal([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]], 2.8 * math.sqrt(2), 5)
        want = FCC_Q6
    else:                  # nearest neighbours at 2.77 A (bonds), next shell at 3.2 A
        com, L = _crystal([[0, 0, 0], [0.5, 0.5, 0.5]], 3.2, 6)
        want = BCC_Q6
    op, q6, _ = orc.order_parameter(orc.OP_Q6, com, L)
    assert np.abs(q6 - want).max() < 1e-12
    assert op == pytest.approx(want, abs=1e-12)


def test_q6_bond_along_z_is_undefined_as_in_the_reference(orc):
    # a simple cubic crystal has bonds with x = y = 0: e^{i phi} = 0/0 (q6.F90:38)
    com, L = _crystal([[0, 0, 0]], 2.8, 6)
    op, _, _ = orc.order_parameter(orc.OP_Q6, com, L)
    assert math.isnan(op)


def test_triangle_of_an_orthorhombic_lattice(orc):
    sp = np.array([2.6, 2.8, 3.2])
    m = 6
    com = np.array([[i, j, k] for i in range(m) for j in range(m) for k in range(m)], float) * sp
    n = len(com)
    ref = np.ones(21)
    op, _, hist = orc.order_parameter(orc.OP_TRIANGLE, com, sp * m, ref=ref)
    # 4 nearest: +-x (2.6 A) and +-y (2.8 A): two angles of cos -1 (bin 0), four of cos 0 (bin 10)
    want = np.zeros(21)
    want[0], want[10] = 2 * n, 4 * n
    assert np.array_equal(hist, want)
    assert op == pytest.approx(math.log(7) / 3 + 2 * math.log(14) / 3, rel=1e-14)
    op_log, _, _ = orc.order_parameter(orc.OP_TRIANGLE, com, sp * m, ref=ref, logarithmic=True)
    assert op_log == pytest.approx(math.log(op), rel=1e-14)
    # an empty reference bin takes p in place of q (kullback_div :319): those bins add nothing
    ref2 = ref.copy()
    ref2[10] = 0.0
    op2, _, _ = orc.order_parameter(orc.OP_TRIANGLE, com, sp * m, ref=ref2)
    assert op2 == pytest.approx(math.log(20 / 3) / 3, rel=1e-14)


def _liquidish(orc, n, seed):
    b = config.water_box("TIP4P", n, seed, jitter=0.45, info=orc.model_info("TIP4P"))
    return b["com"], b["L"]


def test_order_parameters_do_not_depend_on_labels_or_origin(orc):
    com, L = _liquidish(orc, 343, 11)
    rng = np.random.default_rng(2)
    perm = rng.permutation(len(com))
    shift = np.array([0.31, -0.77, 1.13])
    ref = rng.uniform(0.5, 2.0, 21)
    for kind in (orc.OP_Q6, orc.OP_TRIANGLE):
        op0, q0, h0 = orc.order_parameter(kind, com, L, ref=ref)
        op1, q1, h1 = orc.order_parameter(kind, com[perm], L, ref=ref)
        op2, q2, h2 = orc.order_parameter(kind, com + shift, L, ref=ref)
        assert np.isfinite(op0)
        assert op1 == pytest.approx(op0, rel=1e-12) and op2 == pytest.approx(op0, rel=1e-12)
        if kind == orc.OP_TRIANGLE:
            assert np.array_equal(h0, h1) and np.array_equal(h0, h2)
        else:
            assert np.abs(q1 - q0[perm]).max() < 1e-12


def test_umbrella_chain_without_bias_is_the_plain_chain(orc):
    com, L = _liquidish(orc, 125, 5)
    quat = config.random_quaternions(len(com), np.random.default_rng(4))
    rc = 0.5 * L[0]
    E0 = orc.compute("TIP4P", "custom", com, quat, L, [rc] * 3, rc - 2.0, rc)[2]
    _, _, e_p, tr_p = orc.mc_run("TIP4P", "custom", com, quat, L, rc - 2.0, rc, 1 / 260.0, 0.15, 0.15, 60, 7, 0, 0, E0)
    for kind in (orc.OP_EP, orc.OP_Q6):
        op0 = E0 if kind == orc.OP_EP else orc.order_parameter(kind, com, L)[0]
        _, _, e_u, o_u, tr_u = orc.mc_umbrella_run("TIP4P", "custom", com, quat, L, rc - 2.0, rc, 1 / 260.0, 0.15,
                                                   0.15, 60, 7, 0, 0, kind, 0.0, 0.0, E0, op0)
        assert np.array_equal(tr_u[:, :4], tr_p)
        assert e_u == e_p
        if kind == orc.OP_EP:
            assert np.array_equal(tr_u[:, 4], tr_u[:, 1])   # the energy order parameter is the running energy


def test_umbrella_term_enters_the_metropolis_test(orc):
    com, L = _liquidish(orc, 125, 5)
    quat = config.random_quaternions(len(com), np.random.default_rng(4))
    rc = 0.5 * L[0]
    E0 = orc.compute("TIP4P", "custom", com, quat, L, [rc] * 3, rc - 2.0, rc)[2]
    op0 = orc.order_parameter(orc.OP_Q6, com, L)[0]
    # a steep umbrella centred far below the current Q6 rejects every move that raises Q6
    c2, q2, e2, o2, tr = orc.mc_umbrella_run("TIP4P", "custom", com, quat, L, rc - 2.0, rc, 1 / 260.0, 0.15, 0.15, 80,
                                             9, 0, 0, orc.OP_Q6, op0 - 0.5, 1.0e12, E0, op0)
    ops = np.concatenate([[op0], tr[:, 4]])
    assert (np.diff(ops) <= 1e-12).all()
    acc = tr[:, 2] == 1
    assert acc.any()
    # every accepted order parameter is the configuration's own
    assert o2 == pytest.approx(orc.order_parameter(orc.OP_Q6, c2, L)[0], rel=1e-13)
