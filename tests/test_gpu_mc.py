"""GPU Monte Carlo and learned proposal widths against the CPU references.

- plain MC in FP64 replays the oracle's chain (same Philox draws) trial by trial;
- the running energy stays equal to a full recomputation (the reference's
  incremental-vs-full check, mc2.F90:489-505);
- training records carry the features of the reference formulas (oracle/mlp.py);
- the device gradient of the training loss matches the FP64 reference;
- training lowers the loss and the learned sampler keeps the energy consistent.
"""
import numpy as np
import pytest

import genesis6_gb300 as g6
from genesis6_gb300 import _capi, config
from genesis6_gb300._capi import dptr, fptr
from oracle import mlp

pytestmark = pytest.mark.gpu


def _chains(model, nrep, n, seed, prec="fp64", jitter=0.3):
    boxes, recs = [], []
    for r in range(nrep):
        b = config.water_box(model, n, seed + r, jitter=jitter)
        boxes.append(b["L"]); recs.append(b)
    L = boxes[0][0]
    rc = 0.5 * L
    s = g6.RigidWater(model, [n] * nrep, np.array(boxes), path="custom", precision=prec, rc=rc, skin=0.0)
    s.upload_state(np.concatenate([b["rec"] for b in recs]))
    return s, recs, rc


def _mc(s, ntrial, seed, counter, beta, st, sr, mode=_capi.MC_PLAIN, sample_every=0):
    R = s.nrep
    beta = np.full(R, beta); st = np.full(R, st); sr = np.full(R, sr)
    counts = np.zeros(2 * R, np.int64); energy = np.zeros(R); trace = np.zeros((R, ntrial, 4))
    nsm = ntrial // sample_every if sample_every else 0
    samples = np.zeros((R, max(nsm, 1)))
    import ctypes
    s._check(s.L.g6_mc_run(s.ctx, ntrial, seed, counter, dptr(beta), dptr(st), dptr(sr), mode, sample_every,
                           dptr(samples) if nsm else None,
                           counts.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), dptr(energy), dptr(trace)))
    return counts.reshape(R, 2), energy, trace, samples


@pytest.mark.parametrize("model", ["ST2", "TIP4P", "SPCE"])
def test_mc_fp64_replays_oracle(orc, model):
    s, recs, rc = _chains(model, 2, 216, 40)
    beta = 1.0 / 260.0
    ntrial = 300
    counts, energy, trace, _ = _mc(s, ntrial, 99, 0, beta, 0.15, 0.15)
    rec_g = s.download_state()
    for c, b in enumerate(recs):
        L = b["L"]
        E0 = orc.compute(model, "custom", b["com"], b["quat"], L, [rc] * 3, rc - 2.0, rc)[2]
        com, quat, e, tr = orc.mc_run(model, "custom", b["com"], b["quat"], L, rc - 2.0, rc, beta, 0.15, 0.15, ntrial,
                                      99, c, 0, E0)
        assert np.array_equal(trace[c, :, 3], tr[:, 3])          # same targets
        assert np.array_equal(trace[c, :, 2], tr[:, 2])          # same decisions
        assert np.abs(trace[c, :, 0] - tr[:, 0]).max() <= 1e-9 * np.abs(tr[:, 0]).max()
        assert energy[c] == pytest.approx(e, rel=1e-10)
        sl = rec_g[216 * c:216 * (c + 1)]
        assert np.abs(sl[:, :3] - com).max() < 1e-10
        assert np.abs(sl[:, 33:37] - quat).max() < 1e-10
        assert counts[c, 1] == ntrial and counts[c, 0] == int(tr[:, 2].sum())


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_mc_running_energy_matches_full(prec):
    s, recs, rc = _chains("ST2", 4, 343, 50, prec=prec)
    counts, energy, trace, samples = _mc(s, 1500, 5, 0, 1.0 / 260.0, 0.15, 0.15, sample_every=100)
    F, tau, ep, vir = s.force()
    tol = 1e-10 if prec == "fp64" else 2e-5
    for c in range(4):
        assert energy[c] == pytest.approx(ep[c], rel=tol, abs=tol * 1e3)
        assert samples[c, -1] == energy[c]
    acc = counts[:, 0] / counts[:, 1]
    assert (acc > 0.2).all() and (acc < 0.95).all()


def test_collect_records_hold_reference_features(orc):
    s, recs, rc = _chains("ST2", 1, 216, 60)
    b = recs[0]
    _mc(s, 1, 3, 0, 1.0 / 260.0, 0.15, 0.15, mode=_capi.MC_COLLECT)
    rec = np.zeros((4, mlp.RECORD), np.float32)
    import ctypes
    cnt = ctypes.c_int64()
    s._check(s.L.g6_mlp_records(s.ctx, fptr(rec), 4, ctypes.byref(cnt)))
    assert cnt.value == 1
    # target and move from the same Philox draws as the device
    u = orc.philox_uniform2(3, 0, 0, 0, 0)
    t = min(int(u[0] * 216), 215)
    sx, sy, sz, intra, tmat = orc.place_sites("ST2", b["com"], b["quat"])
    fo = mlp.features(b["com"], b["L"], t, b["com"][t], intra[t, 1:5])
    assert np.allclose(rec[0, :mlp.NIN], fo, rtol=2e-4, atol=2e-4)
    rot = []; dx = []
    for k in range(3):
        a = orc.philox_uniform2(3, 0, 0, 0, 1 + k)
        rot.append(np.sqrt(-2 * np.log(a[0])) * np.sin(2 * np.pi * a[1]) * 0.15)
    for k in range(3):
        a = orc.philox_uniform2(3, 0, 0, 0, 4 + k)
        dx.append(np.sqrt(-2 * np.log(a[0])) * np.sin(2 * np.pi * a[1]) * 0.15)
    assert rec[0, 2 * mlp.NIN] == pytest.approx(np.sum(np.square(dx)), rel=1e-5)
    assert rec[0, 2 * mlp.NIN + 1] == pytest.approx(np.sum(np.square(rot)), rel=1e-5)


def test_feature_cache_follows_the_chain(orc):
    """Records carry the target's features from the device cache, which accepted
    moves update term by term; they must equal a fresh evaluation at the state
    the FP64 oracle chain reaches after the same number of trials."""
    s, recs, rc = _chains("ST2", 1, 216, 61)
    b = recs[0]
    beta, K = 1.0 / 260.0, 400
    counts, energy, trace, _ = _mc(s, K, 17, 0, beta, 0.15, 0.15, mode=_capi.MC_COLLECT)
    assert counts[0, 0] > 50                      # enough accepted moves to exercise the updates
    rec = np.zeros((K, mlp.RECORD), np.float32)
    import ctypes
    cnt = ctypes.c_int64()
    s._check(s.L.g6_mlp_records(s.ctx, fptr(rec), K, ctypes.byref(cnt)))
    assert cnt.value == K
    E0 = orc.compute("ST2", "custom", b["com"], b["quat"], b["L"], [rc] * 3, rc - 2.0, rc)[2]
    for k in (120, 260, K - 1):
        com, quat, _, tr = orc.mc_run("ST2", "custom", b["com"], b["quat"], b["L"], rc - 2.0, rc, beta, 0.15, 0.15,
                                      k, 17, 0, 0, E0)
        assert np.array_equal(tr[:, 2], trace[0, :k, 2])
        t = int(trace[0, k, 3])
        sx, sy, sz, intra, tmat = orc.place_sites("ST2", com, quat)
        fo = mlp.features(com, b["L"], t, com[t], intra[t, 1:5])
        assert np.allclose(rec[k, :mlp.NIN], fo, rtol=2e-4, atol=2e-4), k


def test_network_widths_match_reference():
    s, recs, rc = _chains("ST2", 1, 216, 71)
    rng = np.random.default_rng(5)
    p = rng.normal(0, 0.3, mlp.NPARAM).astype(np.float32)
    feat = rng.uniform(0, 3, (300, mlp.NIN)).astype(np.float32)
    mean = feat.mean(0).astype(np.float32); istd = (1 / feat.std(0)).astype(np.float32)
    s._check(s.L.g6_mlp_set(s.ctx, fptr(p), fptr(mean), fptr(istd), 0.15, 0.2))
    st = np.zeros(300); sr = np.zeros(300)
    s._check(s.L.g6_mlp_widths(s.ctx, fptr(feat), 300, dptr(st), dptr(sr)))
    z, _ = mlp.forward(p.astype(np.float64), (feat.astype(np.float64) - mean) * istd)
    wt, wr = mlp.widths(z, 0.15, 0.2)
    assert np.allclose(st, wt, rtol=1e-5) and np.allclose(sr, wr, rtol=1e-5)


def test_learned_chain_is_reproducible():
    s, recs, rc = _chains("ST2", 4, 216, 81, prec="mixed")
    _mc(s, 1500, 11, 0, 1.0 / 260.0, 0.15, 0.15, mode=_capi.MC_COLLECT)
    s._check(s.L.g6_mlp_train(s.ctx, 3, 256, 3e-3, 7, 0.15, 0.15, None))
    rec0 = s.download_state()
    out = []
    for _ in range(2):
        s.upload_state(rec0)
        counts, energy, trace, _ = _mc(s, 800, 12, 10 ** 6, 1.0 / 260.0, 0.15, 0.15, mode=_capi.MC_LEARNED)
        out.append((counts.copy(), energy.copy(), trace.copy()))
    assert np.array_equal(out[0][2], out[1][2])
    assert np.array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("w_move,w_energy", [(1.0, 0.0), (1.0, 0.5)])
def test_mlp_gradient_matches_reference(w_move, w_energy):
    s, recs, rc = _chains("ST2", 1, 216, 70)
    s._check(s.L.g6_mlp_objective(s.ctx, w_move, w_energy))
    rng = np.random.default_rng(1)
    n = 512
    rec = np.zeros((n, mlp.RECORD))
    rec[:, :2 * mlp.NIN] = rng.uniform(0, 3, (n, 2 * mlp.NIN))
    rec[:, 2 * mlp.NIN] = rng.chisquare(3, n) * 0.15 ** 2
    rec[:, 2 * mlp.NIN + 1] = rng.chisquare(3, n) * 0.15 ** 2
    rec[:, 2 * mlp.NIN + 2] = rng.normal(0.5, 1.5, n)
    p = rng.normal(0, 0.2, mlp.NPARAM).astype(np.float32)
    mean = rec[:, :mlp.NIN].mean(0).astype(np.float32); istd = (1 / rec[:, :mlp.NIN].std(0)).astype(np.float32)
    s._check(s.L.g6_mlp_set(s.ctx, fptr(p), fptr(mean), fptr(istd), 0.15, 0.15))
    rec32 = rec.astype(np.float32)
    g = np.zeros(mlp.NPARAM, np.float32)
    loss = np.zeros(1)
    s._check(s.L.g6_mlp_grad(s.ctx, fptr(rec32), n, fptr(g), dptr(loss)))
    lref, gref = mlp.loss_and_grad(p.astype(np.float64), rec32.astype(np.float64), mean.astype(np.float64),
                                   istd.astype(np.float64), 0.15, 0.15, w_move, w_energy)
    assert loss[0] == pytest.approx(lref, rel=1e-4)
    assert np.abs(g - gref).max() <= 2e-3 * np.abs(gref).max()


def test_training_lowers_loss_and_learned_chain_is_consistent():
    s, recs, rc = _chains("ST2", 8, 216, 80, prec="mixed")
    _mc(s, 2000, 11, 0, 1.0 / 260.0, 0.15, 0.15, mode=_capi.MC_COLLECT)
    loss = np.zeros(6)
    s._check(s.L.g6_mlp_train(s.ctx, 6, 256, 3e-3, 7, 0.15, 0.15, dptr(loss)))
    assert np.isfinite(loss).all()
    assert loss[-1] < loss[0]
    counts, energy, trace, _ = _mc(s, 1000, 12, 10 ** 6, 1.0 / 260.0, 0.15, 0.15, mode=_capi.MC_LEARNED)
    F, tau, ep, vir = s.force()
    for c in range(8):
        assert energy[c] == pytest.approx(ep[c], rel=2e-5, abs=0.05)
    assert (counts[:, 0] > 0).all()


@pytest.mark.parametrize("model", ["ST2", "TIP4P", "SPCE"])
def test_learned_fp64_chain_replays_reference(orc, model):
    """The FP64 learned-width chain (widths at both poses, Hastings term) follows
    the CPU restatement trial by trial: same targets, same decisions, same end
    state.  The network is random, so the widths vary from molecule to molecule
    and from pose to pose."""
    s, recs, rc = _chains(model, 2, 216, 90)
    rng = np.random.default_rng(9)
    p = rng.normal(0, 0.3, mlp.NPARAM).astype(np.float32)
    mean = np.full(mlp.NIN, 0.5, np.float32); istd = np.full(mlp.NIN, 1.0, np.float32)
    s._check(s.L.g6_mlp_set(s.ctx, fptr(p), fptr(mean), fptr(istd), 0.1, 0.1))
    beta, ntrial = 1.0 / 260.0, 250
    counts, energy, trace, _ = _mc(s, ntrial, 31, 0, beta, 0.1, 0.1, mode=_capi.MC_LEARNED)
    rec_g = s.download_state()
    for c, b in enumerate(recs):
        com, quat, tr = mlp.mc_run_learned(orc, model, "custom", b["com"], b["quat"], b["L"], rc - 2.0, rc, beta,
                                           p, mean, istd, 0.1, 0.1, ntrial, 31, c, 0)
        assert np.array_equal(trace[c, :, 3], tr[:, 2])          # same targets
        assert np.array_equal(trace[c, :, 2], tr[:, 1])          # same decisions
        assert 0 < tr[:, 1].sum() < ntrial
        # the widths come from FP32 features and an FP32 network on the device
        # (about 1e-6 relative), so the moves and their dE differ at that level
        assert np.abs(trace[c, :, 0] - tr[:, 0]).max() <= 2e-5 * np.abs(tr[:, 0]).max()
        sl = rec_g[216 * c:216 * (c + 1)]
        assert np.abs(sl[:, :3] - com).max() < 1e-5
        assert np.abs(sl[:, 33:37] - quat).max() < 1e-5


def test_feature_pool_overflow_is_reported():
    """More than 64 molecules within 6 A of a pose (a compressed cluster) ends the
    run with G6_ERR_CAPACITY instead of silently dropping feature neighbours."""
    b = config.water_box("ST2", 216, 70, jitter=0.0)
    rec = b["rec"].copy()
    c0 = rec[:100, 0:3].mean(axis=0)
    rec[:100, 0:3] = c0 + (rec[:100, 0:3] - c0) * 0.3      # 100 molecules squeezed into a few A
    s = g6.RigidWater("ST2", 216, b["L"], path="custom", precision="mixed", rc=0.5 * b["L"][0] - 0.05, skin=0.0)
    s.upload_state(rec)
    with pytest.raises(g6.G6Error) as e:
        _mc(s, 64, 5, 0, 1.0 / 260.0, 0.15, 0.15, mode=_capi.MC_COLLECT)
    assert e.value.status == _capi.G6_ERR_CAPACITY
    assert "within 6 A" in str(e.value)
