"""FP64 NumPy reference of the learned-proposal pieces (test infrastructure).

The device computes local-environment features, the 24-64-64-2 tanh network,
its training loss and gradients in FP32 kernels (genesis6_gb300/csrc/g6_mlp.cuh,
g6_train.cu).  This module restates each in FP64 so the tests can check the
kernels: the gradient here is checked against finite differences of the loss
here, and the device gradient against this one.
"""
from __future__ import annotations

import numpy as np

NIN, NH, NOUT = 24, 64, 2
W1, B1 = 0, NH * NIN
W2 = B1 + NH
B2 = W2 + NH * NH
W3 = B2 + NH
B3 = W3 + NOUT * NH
NPARAM = B3 + NOUT
RECORD = 2 * NIN + 3
SMIN, SSPAN = 0.1, 2.9          # sigma = sigma0 * (SMIN + SSPAN * sigmoid(z))


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return (p[W1:B1].reshape(NH, NIN), p[B1:W2], p[W2:B2].reshape(NH, NH), p[B2:W3], p[W3:B3].reshape(NOUT, NH),
            p[B3:NPARAM])


def features(com_all, L, t, com, off_charged):
    """Features of molecule t placed at `com` with lab offsets of its charged sites (NQ,3)."""
    f = np.zeros(NIN)
    u = np.zeros((4, 3))
    for s in range(min(4, len(off_charged))):
        u[s] = off_charged[s] / np.linalg.norm(off_charged[s])
    for j in range(len(com_all)):
        if j == t:
            continue
        d = com_all[j] - com
        d = d - np.round(d / L) * L
        r2 = d @ d
        if r2 >= 6.0 ** 2 or r2 <= 0:
            continue
        r = np.sqrt(r2)
        f[:16] += np.exp(-((r - (2.4 + 0.225 * np.arange(16))) * 4.0) ** 2)
        g1 = np.exp(-((r - 2.9) / 0.35) ** 2)
        g2 = np.exp(-((r - 4.5) * 2.0) ** 2)
        c = np.maximum(u @ d / r, 0.0)
        f[16:20] += g1 * c ** 4
        f[20:24] += g2 * c ** 4
    return f


def forward(p, x):
    """x (B,24) normalised -> z (B,2), with activations for backprop."""
    w1, b1, w2, b2, w3, b3 = unpack(p)
    h1 = np.tanh(x @ w1.T + b1)
    h2 = np.tanh(h1 @ w2.T + b2)
    z = h2 @ w3.T + b3
    return z, (x, h1, h2)


def widths(z, s0t, s0r):
    s = 1.0 / (1.0 + np.exp(-z))
    return s0t * (SMIN + SSPAN * s[..., 0]), s0r * (SMIN + SSPAN * s[..., 1])


def loss_and_grad(p, rec, mean, istd, s0t, s0r, w_move=1.0, w_energy=0.0):
    """Mean over records of -J (g6_train.cu) and its gradient w.r.t. the parameters.

    J = min(q(x'|x), exp(-beta dE) q(x|x')) / q0(x'|x) * (w_move * D + w_energy * (beta dE)^2):
    the expected jump of an accepted move under the network's proposal, estimated
    from moves drawn with the fixed widths s0t, s0r."""
    rec = np.asarray(rec, dtype=np.float64)
    B = rec.shape[0]
    xo = (rec[:, :NIN] - mean) * istd
    xn = (rec[:, NIN:2 * NIN] - mean) * istd
    d2, r2, bde = rec[:, 2 * NIN], rec[:, 2 * NIN + 1], rec[:, 2 * NIN + 2]
    zo, ao = forward(p, xo)
    zn, an = forward(p, xn)
    sg_o = 1.0 / (1.0 + np.exp(-zo))
    sg_n = 1.0 / (1.0 + np.exp(-zn))
    so = np.stack([s0t * (SMIN + SSPAN * sg_o[:, 0]), s0r * (SMIN + SSPAN * sg_o[:, 1])], 1)
    sn = np.stack([s0t * (SMIN + SSPAN * sg_n[:, 0]), s0r * (SMIN + SSPAN * sg_n[:, 1])], 1)

    def logq(s):
        return -3 * np.log(s[:, 0]) - d2 / (2 * s[:, 0] ** 2) - 3 * np.log(s[:, 1]) - r2 / (2 * s[:, 1] ** 2)

    lq0 = -3 * np.log(s0t) - d2 / (2 * s0t ** 2) - 3 * np.log(s0r) - r2 / (2 * s0r ** 2)
    lf = logq(so) - lq0
    lr = logq(sn) - bde - lq0
    use_o = lf <= lr
    l = np.where(use_o, lf, lr)
    D = w_move * (d2 / s0t ** 2 + r2 / s0r ** 2) + w_energy * bde ** 2
    J = np.exp(np.minimum(l, 30.0)) * D
    loss = -J.mean()
    s_act = np.where(use_o[:, None], so, sn)
    sg_act = np.where(use_o[:, None], sg_o, sg_n)
    dls = np.stack([-3 / s_act[:, 0] + d2 / s_act[:, 0] ** 3, -3 / s_act[:, 1] + r2 / s_act[:, 1] ** 3], 1)
    dsdz = np.stack([s0t, s0r])[None, :] * SSPAN * sg_act * (1 - sg_act)
    gz = (-J[:, None] * dls * dsdz) / B
    gzo = np.where(use_o[:, None], gz, 0.0)
    gzn = np.where(use_o[:, None], 0.0, gz)
    g = np.zeros(NPARAM)
    w1, b1, w2, b2, w3, b3 = unpack(p)
    for gzs, (x, h1, h2) in ((gzo, ao), (gzn, an)):
        g[W3:B3] += (gzs.T @ h2).ravel()
        g[B3:NPARAM] += gzs.sum(0)
        d2h = (gzs @ w3) * (1 - h2 ** 2)
        g[W2:B2] += (d2h.T @ h1).ravel()
        g[B2:W3] += d2h.sum(0)
        d1h = (d2h @ w2) * (1 - h1 ** 2)
        g[W1:B1] += (d1h.T @ x).ravel()
        g[B1:W2] += d1h.sum(0)
    return loss, g


def mc_run_learned(orc, model, path, com, quat, L, rin, rc, beta, p, mean, istd, s0t, s0r, ntrial, seed, chain,
                   counter):
    """Monte Carlo chain with learned widths on the CPU, the device's G6_MC_LEARNED
    trial in FP64: the widths at the old pose from the features of the current
    configuration, Gaussian rotation vector and translation scaled by them (same
    Philox draws as the device: counter = chain, trial, draw), the widths at the
    new pose, and the Metropolis-Hastings test
    log u < -beta dE + log q(x|x') - log q(x'|x) with the isotropic Gaussian
    densities of the two widths.  `orc` is the oracle module (energies, draws,
    site placement).  Returns com, quat and a trace (ntrial, 4): dE, accepted,
    target, log Hastings ratio."""
    com = np.array(com, dtype=np.float64)
    quat = np.array(quat, dtype=np.float64)
    n = com.shape[0]
    K = orc.constants()
    conv = K["I2J"] * K["J2K"]
    p = np.asarray(p, dtype=np.float64)
    mean = np.asarray(mean, dtype=np.float64)
    istd = np.asarray(istd, dtype=np.float64)
    # the charged sites, in site order: their directions are the direction features
    charged = np.nonzero(orc.model_info(model)["param"][:, 0] != 0.0)[0]

    def widths_at(t, c, q):
        intra = orc.place_sites(model, c[None, :], q[None, :])[3][0]
        f = features(com, L, t, c, intra[charged][:4])
        z, _ = forward(p, ((f - mean) * istd)[None, :])
        st, sr = widths(z, s0t, s0r)
        return float(st[0]), float(sr[0])

    def logq(st, sr, d2, r2):
        return -3.0 * (np.log(st) + np.log(sr)) - d2 / (2 * st * st) - r2 / (2 * sr * sr)

    trace = np.zeros((ntrial, 4))
    for k in range(ntrial):
        trial = counter + k
        lo, hi = trial & 0xffffffff, trial >> 32
        u0 = orc.philox_uniform2(seed, chain, lo, hi, 0)
        t = min(int(u0[0] * n), n - 1)
        g = []
        for d in range(6):
            a = orc.philox_uniform2(seed, chain, lo, hi, 1 + d)
            g.append(np.sqrt(-2.0 * np.log(a[0])) * np.sin(2.0 * np.pi * a[1]))
        st, sr = widths_at(t, com[t], quat[t])
        rot = np.array(g[:3]) * sr
        dx = np.array(g[3:]) * st
        qr = np.array([1.0, rot[0], rot[1], rot[2]])
        qr = qr / np.sqrt(qr @ qr)
        a_, b_, c_, d_ = qr
        qo = quat[t]
        qn = np.array([a_ * qo[0] - b_ * qo[1] - c_ * qo[2] - d_ * qo[3], a_ * qo[1] + b_ * qo[0] + c_ * qo[3] - d_ * qo[2],
                       a_ * qo[2] + c_ * qo[0] - b_ * qo[3] + d_ * qo[1], a_ * qo[3] + d_ * qo[0] + b_ * qo[2] - c_ * qo[1]])
        if qn[0] < 0:
            qn = -qn
        cn = com[t] + dx
        st2, sr2 = widths_at(t, cn, qn)
        d2, r2 = float(dx @ dx), float(rot @ rot)
        logh = logq(st2, sr2, d2, r2) - logq(st, sr, d2, r2)
        eo = orc.molecule_energy(model, path, com, quat, t, com[t], quat[t], L, rin, rc)
        en = orc.molecule_energy(model, path, com, quat, t, cn, qn, L, rin, rc)
        dE = en - eo
        x = -(dE * conv) * beta + logh
        acc = x >= 0.0 or np.log(u0[1]) < x
        if acc:
            com[t] = cn
            quat[t] = qn
        trace[k] = (dE, 1.0 if acc else 0.0, t, logh)
    return com, quat, trace
