"""CPU checks of the FP64 learned-proposal reference (oracle/mlp.py): the
analytic gradient of the training loss against central finite differences."""
import numpy as np
import pytest

from oracle import mlp


def _records(rng, n=64):
    rec = np.zeros((n, mlp.RECORD))
    rec[:, :2 * mlp.NIN] = rng.uniform(0, 3, (n, 2 * mlp.NIN))
    rec[:, 2 * mlp.NIN] = rng.chisquare(3, n) * 0.15 ** 2       # |d|^2 at sigma0 = 0.15
    rec[:, 2 * mlp.NIN + 1] = rng.chisquare(3, n) * 0.15 ** 2
    rec[:, 2 * mlp.NIN + 2] = rng.normal(0.5, 1.5, n)           # beta * dE
    return rec


@pytest.mark.parametrize("w_move,w_energy", [(1.0, 0.0), (1.0, 0.5), (0.0, 1.0)])
def test_gradient_matches_finite_differences(w_move, w_energy):
    rng = np.random.default_rng(0)
    p = rng.normal(0, 0.3, mlp.NPARAM)
    rec = _records(rng)
    mean = rec[:, :mlp.NIN].mean(0); istd = 1 / rec[:, :mlp.NIN].std(0)
    loss, g = mlp.loss_and_grad(p, rec, mean, istd, 0.15, 0.15, w_move, w_energy)
    h = 1e-6
    for k in rng.choice(mlp.NPARAM, 40, replace=False).tolist() + [mlp.B3, mlp.B3 + 1]:
        pp = p.copy(); pp[k] += h
        pm = p.copy(); pm[k] -= h
        fd = (mlp.loss_and_grad(pp, rec, mean, istd, 0.15, 0.15, w_move, w_energy)[0] -
              mlp.loss_and_grad(pm, rec, mean, istd, 0.15, 0.15, w_move, w_energy)[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(g).max())


def test_constant_network_gives_sigma0():
    p = np.zeros(mlp.NPARAM)
    p0 = (1.0 - mlp.SMIN) / mlp.SSPAN      # the initial output bias of g6_mlp_train
    p[mlp.B3:] = np.log(p0 / (1.0 - p0))
    z, _ = mlp.forward(p, np.zeros((3, mlp.NIN)))
    st, sr = mlp.widths(z, 0.15, 0.2)
    assert np.allclose(st, 0.15) and np.allclose(sr, 0.2)
