"""GPU parity: libg6gpu.so (through its C ABI) against the FP64 oracle.

Bars:
  - cell ids and the within-cutoff pair set: bit-exact, including the image
    offsets and the switch values hh/dh of every pair;
  - plain FP64 mode: total energy and virial to 1e-12 relative, per-molecule
    force/torque to 1e-12 of the RMS force/torque;
  - mixed mode: relative RMS force error <= 1e-5 (torques <= 1e-5).
"""
import numpy as np
import pytest

import genesis6_gb300 as g6
from genesis6_gb300 import _capi, config
from genesis6_gb300.interaction import Interaction, Sites, force, pair_potential, site_positions

pytestmark = pytest.mark.gpu

CASES = [("TIP4P", "custom"), ("TIP4P", "std"), ("TIP5P", "std"), ("ST2", "custom"), ("ST2", "std"), ("SPCE", "std")]


def _system(model, path, n, seed, prec="fp64", rc=8.5, jitter=0.4, skin=1.0, cell_edge=0.0):
    b = config.water_box(model, n, seed, jitter=jitter)
    s = g6.RigidWater(model, n, b["L"], path=path, precision=prec, rc=rc, skin=skin, cell_edge=cell_edge)
    s.upload_state(b["rec"])
    return s, b


def _canon(p):
    a = np.minimum(p["i"], p["j"]); b = np.maximum(p["i"], p["j"])
    key = a.astype(np.int64) * 10 ** 7 + b
    return key


@pytest.mark.parametrize("n,rc", [(256, 8.5), (4096, 9.0), (1000, 7.0), (32768, 9.0)])
def test_cells_bitexact(orc, n, rc):
    s, b = _system("TIP4P", "custom", n, 11 + n, rc=rc, jitter=3.0)
    cell_gpu = s.cells()
    cell_orc, _ = orc.pairsearch(b["com"], b["L"], [rc] * 3, rc - 2.0, rc)
    assert np.array_equal(cell_gpu, cell_orc)


@pytest.mark.parametrize("n,rc", [(256, 8.5), (4096, 9.0), (512, 9.5), (32768, 9.0)])
def test_pairset_bitexact(orc, n, rc):
    s, b = _system("TIP4P", "custom", n, 3 + n, rc=rc, jitter=3.0)
    pg = s.pairsearch()
    _, po = orc.pairsearch(b["com"], b["L"], [rc] * 3, rc - 2.0, rc)
    kg, ko = _canon(pg), _canon(po)
    assert len(kg) == len(ko) == len(np.unique(kg))
    og, oo = np.argsort(kg), np.argsort(ko)
    assert np.array_equal(kg[og], ko[oo])
    # orientation of each pair may differ; image offsets flip sign with it
    sg = np.where(pg["i"][og] < pg["j"][og], 1.0, -1.0)
    so = np.where(po["i"][oo] < po["j"][oo], 1.0, -1.0)
    for k in ("ox", "oy", "oz"):
        assert np.array_equal(pg[k][og] * sg, po[k][oo] * so)
    for k in ("hh", "dh"):
        assert np.array_equal(pg[k][og], po[k][oo])   # bit-exact switch values


@pytest.mark.parametrize("model,path", CASES)
def test_force_fp64_matches_oracle(orc, model, path):
    n = 256 if model == "TIP4P" else 343
    L = config.box_edge(n)
    rc = min(8.5, 0.5 * L - 0.05)
    s, b = _system(model, path, n, 21, rc=rc)
    F, tau, ep, vir = s.force()
    Fo, to, Eo, Vo, _ = orc.compute(model, path, b["com"], b["quat"], b["L"], [rc] * 3, rc - 2.0, rc)
    assert ep[0] == pytest.approx(Eo, rel=1e-12)
    assert np.abs(vir[0] - Vo).max() <= 1e-12 * np.abs(Vo).max()
    frms = np.sqrt((Fo ** 2).sum(1).mean()); trms = np.sqrt((to ** 2).sum(1).mean())
    assert np.abs(F - Fo).max() <= 1e-12 * frms
    assert np.abs(tau - to).max() <= 1e-12 * trms


@pytest.mark.parametrize("n,seed", [(4096, 4), (32768, 17)])
def test_force_fp64_large(orc, n, seed):
    """TIP4P-4096 and TIP4P-32768 (ndiv 11 at rc 9 A): FP64 energy, virial and
    per-molecule force/torque against the oracle's full force path."""
    s, b = _system("TIP4P", "custom", n, seed, rc=9.0)
    F, tau, ep, vir = s.force()
    Fo, to, Eo, Vo, npair = orc.compute("TIP4P", "custom", b["com"], b["quat"], b["L"], [9.0] * 3, 7.0, 9.0)
    assert ep[0] == pytest.approx(Eo, rel=1e-12)
    assert np.abs(vir[0] - Vo).max() <= 1e-12 * np.abs(Vo).max()
    frms = np.sqrt((Fo ** 2).sum(1).mean()); trms = np.sqrt((to ** 2).sum(1).mean())
    assert np.abs(F - Fo).max() <= 1e-12 * frms
    assert np.abs(tau - to).max() <= 1e-12 * trms


@pytest.mark.parametrize("model,path", CASES)
def test_force_mixed_rms_error(orc, model, path):
    n = 512
    L = config.box_edge(n)
    rc = min(9.0, 0.5 * L - 0.05)
    s, b = _system(model, path, n, 31, prec="mixed", rc=rc)
    F, tau, ep, vir = s.force()
    Fo, to, Eo, Vo, _ = orc.compute(model, path, b["com"], b["quat"], b["L"], [rc] * 3, rc - 2.0, rc)
    ef = np.sqrt(((F - Fo) ** 2).sum() / (Fo ** 2).sum())
    et = np.sqrt(((tau - to) ** 2).sum() / (to ** 2).sum())
    assert ef <= 1e-5, ef
    assert et <= 1e-5, et
    assert ep[0] == pytest.approx(Eo, rel=1e-5)


@pytest.mark.parametrize("model,path,half", [("TIP4P", "custom", 1), ("TIP4P", "custom", 0), ("TIP4P", "std", 1),
                                            ("TIP5P", "custom", 1), ("ST2", "custom", 1), ("ST2", "std", 1),
                                            ("SPCE", "std", 1)])
def test_md_step_forces_rms_error(orc, model, path, half):
    """The forces of the mixed MD step's pair kernel itself (g6_step_forces:
    half list with the partner's share by float atomics, or the full list)
    against the FP64 oracle: relative RMS force and torque error <= 1e-5."""
    import ctypes
    n = 512
    L = config.box_edge(n)
    rc = min(9.0, 0.5 * L - 0.05)
    s, b = _system(model, path, n, 33, prec="mixed", rc=rc)
    sh = _capi.Shape(lpi=8, step_lpi=8, step_mpw=4, skin=1.0, cap=0, step_ms=0.0, step_half=half)
    s._check(s.L.g6_set_shape(s.ctx, ctypes.byref(sh)))
    F, tau, ep = s.step_forces()
    Fo, to, Eo, Vo, _ = orc.compute(model, path, b["com"], b["quat"], b["L"], [rc] * 3, rc - 2.0, rc)
    ef = np.sqrt(((F - Fo) ** 2).sum() / (Fo ** 2).sum())
    et = np.sqrt(((tau - to) ** 2).sum() / (to ** 2).sum())
    assert ef <= 1e-5, ef
    assert et <= 1e-5, et
    assert ep[0] == pytest.approx(Eo, rel=1e-5)
    # the step's forces also agree with the force-only entry's mixed forces
    F2, tau2, ep2, _ = s.force()
    assert np.sqrt(((F - F2) ** 2).sum() / (F2 ** 2).sum()) <= 1e-5


def test_md_step_forces_then_md_run():
    """A half-row list left by g6_step_forces is rebuilt in full form for a
    full-list run, and the run follows the same run on a fresh context."""
    import ctypes
    n = 343
    b = config.water_box("TIP4P", n, 14, temp=300.0, dt=0.002, jitter=0.2)
    runs = []
    for first in (True, False):
        s = g6.RigidWater("TIP4P", n, b["L"], path="custom", precision="mixed", rc=8.5)
        s.upload_state(b["rec"])
        if first:
            s.step_forces()   # half rows (the default list form)
        sh = _capi.Shape(lpi=8, step_lpi=8, step_mpw=4, skin=1.0, cap=0, step_ms=0.0, step_half=0)
        s._check(s.L.g6_set_shape(s.ctx, ctypes.byref(sh)))
        runs.append((s.md_run(0.002, 10), s.download_state()))
        s.close()
    assert np.array_equal(runs[0][0][:, 0, 6], runs[1][0][:, 0, 6])   # pairs within rc
    assert np.array_equal(runs[0][1], runs[1][1])


def test_half_list_shape_is_set_and_reported():
    """g6_set_shape accepts the half or the full list in both precisions,
    reports the list form back and refuses any other value."""
    import ctypes
    for prec in ("fp64", "mixed"):
        m, _ = _system("TIP4P", "custom", 216, 4, prec=prec, rc=8.0)
        sh = _capi.Shape(lpi=8, step_lpi=8, step_mpw=8, skin=1.0, cap=0, step_ms=0.0, step_half=1)
        assert m.L.g6_set_shape(m.ctx, ctypes.byref(sh)) == _capi.G6_OK
        got = _capi.Shape()
        m._check(m.L.g6_get_shape(m.ctx, ctypes.byref(got)))
        assert got.step_half == 1
        sh.step_half = 2
        assert m.L.g6_set_shape(m.ctx, ctypes.byref(sh)) == _capi.G6_ERR_ARG


def test_step_forces_refuses_fp64():
    s, b = _system("TIP4P", "custom", 216, 3, prec="fp64", rc=8.0)
    with pytest.raises(g6.G6Error) as e:
        s.step_forces()
    assert e.value.status == _capi.G6_ERR_STATE


@pytest.mark.parametrize("model,path", CASES)
def test_force_sites_entry_matches_reference_call(orc, model, path):
    """g6_force_sites / g6_pair_potential mirror force()/PairPotential() on the caller's pair list."""
    n = 216
    L = config.box_edge(n)
    rc = min(8.5, 0.5 * L - 0.05)
    b = config.water_box(model, n, 41, jitter=0.4)
    s = g6.RigidWater(model, n, b["L"], path=path, rc=rc)
    x, y, z = orc.place_sites(model, b["com"], b["quat"])[:3]
    _, p = orc.pairsearch(b["com"], b["L"], [rc] * 3, rc - 2.0, rc)
    site = Sites.of(x, y, z)
    iv = Interaction.from_pairs(p)
    ep, vr = force(s, site, iv)
    fx, fy, fz, epo, vro = orc.force_sites(model, path, x, y, z, p)
    fs = np.abs(np.concatenate([fx, fy, fz])).max()
    assert np.abs(site.fx - fx).max() <= 1e-12 * fs
    assert np.abs(site.fy - fy).max() <= 1e-12 * fs
    assert np.abs(site.fz - fz).max() <= 1e-12 * fs
    assert np.abs(ep - epo).max() <= 1e-12 * np.abs(epo).max()
    assert np.abs(vr - vro).max() <= 1e-12 * np.abs(vro).max()
    e2 = pair_potential(s, site, iv)
    e2o = orc.pair_potential(model, path, x, y, z, p)
    assert np.abs(e2 - e2o).max() <= 1e-12 * np.abs(e2o).max()
    # host-side site placement agrees with the oracle's
    hx, hy, hz = site_positions(model, b["com"], b["quat"])
    assert np.abs(hx - x).max() < 1e-12


@pytest.mark.parametrize("model,path,half", [("TIP4P", "custom", 0), ("TIP4P", "std", 0), ("TIP5P", "custom", 0),
                                             ("ST2", "custom", 0), ("SPCE", "std", 0), ("ST2", "std", 0),
                                             ("TIP4P", "custom", 1), ("TIP4P", "std", 1), ("TIP5P", "custom", 1),
                                             ("ST2", "custom", 1), ("SPCE", "std", 1)])
def test_md_fp64_follows_oracle(orc, model, path, half):
    """Short Gear MD: the device trajectory tracks the oracle's step by step,
    with the full list (the default) and with the half list (each pair once,
    the partner's share by FP64 atomics, then a separate integrator kernel)."""
    import ctypes
    n = 256
    b = config.water_box(model, n, 5, temp=300.0, dt=0.002, jitter=0.2)
    L = b["L"]
    s = g6.RigidWater(model, n, L, path=path, rc=8.5, skin=1.0)
    if half:
        sh = _capi.Shape(lpi=8, step_lpi=8, step_mpw=8, skin=1.0, cap=0, step_ms=0.0, step_half=1)
        s._check(s.L.g6_set_shape(s.ctx, ctypes.byref(sh)))
    s.upload_state(b["rec"])
    log = s.md_run(0.002, 20)
    rec_g = s.download_state()
    rec_o, _, log_o = orc.md_run(model, path, b["rec"], L, [8.5] * 3, 6.5, 8.5, 0.002, 20, np.zeros(10))
    assert np.abs(log[:, 0, 0] - log_o[:, 0]).max() <= 1e-9 * np.abs(log_o[:, 0]).max()
    assert np.abs(log[:, 0, 5] - log_o[:, 5]).max() <= 1e-9 * np.abs(log_o[:, 5]).max()
    # kinetic energies, temperature and pressure (rigid_ek, Rigid_PressureTensor; Mixture.F90:2251-2264)
    for c in (1, 2, 3):
        assert np.abs(log[:, 0, c] - log_o[:, c]).max() <= 1e-9 * np.abs(log_o[:, c]).max(), c
    assert np.abs(log[:, 0, 4] - log_o[:, 4]).max() <= 1e-8 * np.abs(log_o[:, 4]).max()
    assert np.abs(rec_g[:, :3] - rec_o[:, :3]).max() < 1e-9
    assert np.abs(rec_g[:, 33:37] - rec_o[:, 33:37]).max() < 1e-9
    assert np.array_equal(log[:, 0, 6], log_o[:, 6])   # pairs within rc, every step


@pytest.mark.parametrize("half", [0, 1])
def test_md_nose_follows_oracle(orc, half):
    import ctypes
    n = 216
    b = config.water_box("TIP4P", n, 6, temp=350.0, dt=0.002, jitter=0.2)
    L = b["L"]
    q = 300.0 * 0.1 ** 2 / 0.002
    s = g6.RigidWater("TIP4P", n, L, path="custom", rc=8.5)
    if half:
        sh = _capi.Shape(lpi=16, step_lpi=16, step_mpw=8, skin=1.0, cap=0, step_ms=0.0, step_half=1)
        s._check(s.L.g6_set_shape(s.ctx, ctypes.byref(sh)))
    s.upload_state(b["rec"])
    th = s.thermostats(1, "nose", temp=300.0, q=q, dump=0.0)
    log = s.md_run(0.002, 25, th)
    t_o = np.array([1, q, 0.0, 300.0, 0, 0, 0, 0, 0, 0], float)
    _, t_o, log_o = orc.md_run("TIP4P", "custom", b["rec"], L, [8.5] * 3, 6.5, 8.5, 0.002, 25, t_o)
    assert np.abs(log[:, 0, 7] - log_o[:, 7]).max() <= 1e-9 * max(1e-30, np.abs(log_o[:, 7]).max())
    assert np.abs(log[:, 0, 5] - log_o[:, 5]).max() <= 1e-9 * np.abs(log_o[:, 5]).max()
    assert th[0].zeta[0] == pytest.approx(t_o[4], rel=1e-8)


@pytest.mark.parametrize("model,mpw,half", [("TIP4P", 4, 0), ("TIP4P", 8, 0), ("TIP4P", 16, 0), ("TIP4P", 32, 0),
                                            ("ST2", 4, 0), ("ST2", 16, 0), ("TIP4P", 4, 1), ("TIP4P", 8, 1),
                                            ("TIP4P", 32, 1), ("ST2", 4, 1), ("ST2", 16, 1), ("TIP5P", 4, 1)])
def test_md_mixed_integrators_follow_oracle(orc, model, mpw, half):
    """Mixed-precision Gear MD with each integrator kernel (one lane per molecule
    with 8, 16 or 32 molecules per warp; four lanes per molecule for step_mpw 4)
    and either list form (half: each pair once, the other molecule's force and
    torque by atomics; full: each pair from both sides) under a Nose-Hoover
    thermostat tracks the oracle's FP64 trajectory for 20 steps within the
    error of FP32 site forces."""
    import ctypes
    n = 256
    b = config.water_box(model, n, 7, temp=320.0, dt=0.002, jitter=0.2)
    L = b["L"]
    q = 300.0 * 0.1 ** 2 / 0.002
    s = g6.RigidWater(model, n, L, path="custom", precision="mixed", rc=8.5, skin=1.0)
    s.upload_state(b["rec"])
    sh = _capi.Shape(lpi=8, step_lpi=8, step_mpw=mpw, skin=1.0, cap=0, step_ms=0.0, step_half=half)
    s._check(s.L.g6_set_shape(s.ctx, ctypes.byref(sh)))
    th = s.thermostats(1, "nose", temp=300.0, q=q, dump=0.0)
    log = s.md_run(0.002, 20, th)
    rec_g = s.download_state()
    t_o = np.array([1, q, 0.0, 300.0, 0, 0, 0, 0, 0, 0], float)
    rec_o, t_o, log_o = orc.md_run(model, "custom", b["rec"], L, [8.5] * 3, 6.5, 8.5, 0.002, 20, t_o)
    assert np.abs(rec_g[:, :3] - rec_o[:, :3]).max() < 1e-5
    assert np.abs(rec_g[:, 33:37] - rec_o[:, 33:37]).max() < 1e-5
    assert np.abs(rec_g[:, 3:6] - rec_o[:, 3:6]).max() < 1e-6          # d1 = v dt
    assert np.abs(rec_g[:, 18:21] - rec_o[:, 18:21]).max() < 1e-5 * np.abs(rec_o[:, 18:21]).max()
    for c in (0, 1, 2, 3, 5):   # Epot, Ekt, Ekr, T, H
        assert np.abs(log[:, 0, c] - log_o[:, c]).max() <= 2e-5 * np.abs(log_o[:, c]).max(), c
    assert np.array_equal(log[:, 0, 6], log_o[:, 6])   # pairs within rc
    assert th[0].zeta[0] == pytest.approx(t_o[4], rel=1e-4, abs=1e-9)


def test_md_mixed_quad_integrator_collisions():
    """The four-lane integrator draws the stochastic collisions of the
    one-lane integrator (same Philox counters per molecule and step): the two
    trajectories agree within FP32 rounding."""
    import ctypes
    n = 343
    b = config.water_box("TIP4P", n, 9, temp=300.0, dt=0.002, jitter=0.2)
    out = []
    for mpw in (4, 8):
        s = g6.RigidWater("TIP4P", n, b["L"], path="custom", precision="mixed", rc=8.5, skin=1.0)
        s.upload_state(b["rec"])
        sh = _capi.Shape(lpi=8, step_lpi=8, step_mpw=mpw, skin=1.0, cap=0, step_ms=0.0)
        s._check(s.L.g6_set_shape(s.ctx, ctypes.byref(sh)))
        th = s.thermostats(1, "andersen", temp=300.0, rate=20.0, seed=77)
        log = s.md_run(0.002, 30, th)
        out.append((s.download_state(), log))
    (ra, la), (rb, lb) = out
    assert np.abs(ra[:, :3] - rb[:, :3]).max() < 1e-5
    assert np.abs(ra[:, 3:6] - rb[:, 3:6]).max() < 1e-6
    assert np.abs(la[:, 0, 3] - lb[:, 0, 3]).max() < 1e-4 * lb[:, 0, 3].max()


def test_md_mixed_conserves_energy():
    n = 512
    b = config.water_box("TIP4P", n, 8, temp=300.0, dt=0.001, jitter=0.2)
    s = g6.RigidWater("TIP4P", n, b["L"], path="custom", precision="mixed", rc=9.0)
    s.upload_state(b["rec"])
    s.md_run(0.001, 200)        # relax the lattice start
    log = s.md_run(0.001, 400)
    H = log[:, 0, 5]
    ek = (log[:, 0, 1] + log[:, 0, 2]).mean() * 10.0   # J/mol
    assert np.isfinite(H).all()
    assert np.ptp(H) < 0.02 * ek


@pytest.mark.parametrize("prec,pinned,half", [("fp64", False, 0), ("mixed", False, 0), ("mixed", True, 0),
                                              ("mixed", False, 1), ("mixed", True, 1)])
def test_host_buffer_step_equals_device_step(prec, pinned, half):
    """g6_md_step_host (state in a host buffer, copied in and out; a page-locked
    buffer takes the cached-graph route) gives the same state, log and
    thermostat as one device-resident step from the same state, on two calls in
    a row: bit for bit with the full list, within FP32 rounding with the half
    list (its atomics sum in a varying order)."""
    import ctypes
    n = 343
    b = config.water_box("TIP4P", n, 12, temp=300.0, dt=0.002, jitter=0.2)
    s = g6.RigidWater("TIP4P", n, b["L"], path="custom", precision=prec, rc=8.5)
    if prec == "mixed":
        sh = _capi.Shape()
        s._check(s.L.g6_get_shape(s.ctx, ctypes.byref(sh)))
        sh.lpi = sh.lpi or 8
        sh.step_lpi = sh.step_lpi or 8
        sh.step_mpw = sh.step_mpw or 4
        sh.step_half = half
        s._check(s.L.g6_set_shape(s.ctx, ctypes.byref(sh)))
    s.upload_state(b["rec"])
    s.md_run(0.002, 50, s.thermostats(1, "nose", temp=300.0, q=300.0 * 0.25 / 0.002))
    rec = s.download_state()
    th_a = s.thermostats(1, "nose", temp=300.0, q=300.0 * 0.25 / 0.002)
    th_b = s.thermostats(1, "nose", temp=300.0, q=300.0 * 0.25 / 0.002)
    if pinned:
        import torch
        host = torch.empty(rec.shape, dtype=torch.float64, pin_memory=True).numpy()
        host[:] = rec
    else:
        host = rec.copy()
    for _ in range(2):
        ref_in = host.copy()
        s.upload_state(ref_in)
        log_a = s.md_run(0.002, 1, th_a)
        want = s.download_state()
        lg = np.zeros(10)
        s.md_step_host(0.002, host, th_b, lg)
        if half:
            assert np.abs(host[:, :3] - want[:, :3]).max() < 1e-9
            assert np.abs(host - want).max() <= 1e-5 * np.abs(want).max()
            assert np.abs(lg - log_a[0, 0]).max() <= 1e-6 * np.abs(log_a[0, 0]).max()
            assert lg[6] == log_a[0, 0, 6]
            host[:] = want      # the next call starts from the same state on both routes
            ctypes.memmove(ctypes.byref(th_b[0]), ctypes.byref(th_a[0]), ctypes.sizeof(th_a[0]))
        else:
            assert np.array_equal(host, want)
            assert np.array_equal(lg, log_a[0, 0])
            assert list(th_a[0].zeta) == list(th_b[0].zeta)


@pytest.mark.parametrize("half", [0, 1])
def test_consecutive_host_steps_follow_a_device_run(half):
    """Twenty g6_md_step_host calls in a row on a page-locked buffer (two
    replicas, a short skin so that the keep-the-list test of the records-in
    kernel triggers rebuilds) end where one 20-step device run ends: state,
    per-replica log rows and Nose thermostats (the control words travel through
    the page-locked block, not through copies)."""
    import ctypes
    import torch
    sizes = [216, 250]
    boxes, recs = [], []
    for k, n in enumerate(sizes):
        b = config.water_box("TIP4P", n, 40 + k, temp=300.0, dt=0.002, jitter=0.2)
        boxes.append(b["L"]); recs.append(b["rec"])
    s = g6.RigidWater("TIP4P", sizes, np.array(boxes), path="custom", precision="mixed", rc=8.0)
    sh = _capi.Shape()
    s._check(s.L.g6_get_shape(s.ctx, ctypes.byref(sh)))
    sh.lpi = sh.lpi or 8
    sh.step_lpi = sh.step_lpi or 8
    sh.step_mpw = sh.step_mpw or 4
    sh.step_half = half
    sh.skin = 0.3
    s._check(s.L.g6_set_shape(s.ctx, ctypes.byref(sh)))
    rec0 = np.concatenate(recs)
    nose = lambda: s.thermostats(2, "nose", temp=[300.0, 330.0], q=300.0 * 0.25 / 0.002)
    s.upload_state(rec0)
    s.md_run(0.002, 30, nose())
    start = s.download_state()
    th_a, th_b = nose(), nose()
    s.upload_state(start)
    log_a = s.md_run(0.002, 20, th_a)
    want = s.download_state()
    host = torch.empty(start.shape, dtype=torch.float64, pin_memory=True).numpy()
    host[:] = start
    s.upload_state(start)
    logs = []
    for _ in range(20):
        lg = np.zeros((2, 10))
        s.md_step_host(0.002, host, th_b, lg)
        logs.append(lg)
    logs = np.array(logs)
    assert logs[:, :, 8].sum() >= 2          # the list was rebuilt on the way
    # the two routes may rebuild the rows at different steps, which changes the
    # FP32 summation order of the forces (~1e-6 relative): positions move ~0.2 A
    # under the forces in 20 steps, so they agree to ~1e-7 A
    assert np.abs(host[:, :3] - want[:, :3]).max() < 2e-6
    assert np.abs(host - want).max() <= 1e-5 * np.abs(want).max()
    for r in range(2):
        for col in (0, 1, 2, 3, 5, 7):
            a, b_ = log_a[:, r, col], logs[:, r, col]
            assert np.abs(a - b_).max() <= 1e-5 * np.abs(a).max() + 1e-12
        # every pair within rc was in the rows at every step on both routes; a
        # pair within ~1e-7 A of rc may fall on either side on the two routes
        dn = np.abs(logs[:, r, 6] - log_a[:, r, 6])
        assert dn.max() <= 2 and (dn > 0).sum() <= 2
        assert th_b[r].zeta[0] == pytest.approx(th_a[r].zeta[0], rel=1e-5, abs=1e-12)
        assert th_b[r].zetasum == pytest.approx(th_a[r].zetasum, rel=1e-5)


def test_replicas_equal_separate_systems(orc):
    sizes = [216, 300, 250]
    boxes, recs = [], []
    for k, n in enumerate(sizes):
        b = config.water_box("TIP4P", n, 100 + k, jitter=0.3)
        boxes.append(b["L"]); recs.append(b)
    s = g6.RigidWater("TIP4P", sizes, np.array(boxes), path="custom", rc=8.5)
    s.upload_state(np.concatenate([b["rec"] for b in recs]))
    F, tau, ep, vir = s.force()
    off = np.concatenate([[0], np.cumsum(sizes)])
    for k, b in enumerate(recs):
        Fo, to, Eo, Vo, _ = orc.compute("TIP4P", "custom", b["com"], b["quat"], b["L"], [8.5] * 3, 6.5, 8.5)
        assert ep[k] == pytest.approx(Eo, rel=1e-12)
        frms = np.sqrt((Fo ** 2).sum(1).mean())
        assert np.abs(F[off[k]:off[k + 1]] - Fo).max() <= 1e-12 * frms


@pytest.mark.parametrize("half", [0, 1])
def test_fp64_md_replicas_equal_separate_runs(half):
    """Ten FP64 MD steps of three uneven replicas in one context (Nose at three
    temperatures) end where three separate single-replica runs end, with the
    full list and with the half list (whose j-side FP64 atomics and 32-molecule
    integrator blocks straddle replica boundaries)."""
    import ctypes
    sizes, temps = [216, 300, 250], [260.0, 300.0, 340.0]
    boxes, recs = [], []
    for k, n in enumerate(sizes):
        b = config.water_box("TIP4P", n, 70 + k, temp=temps[k], dt=0.002, jitter=0.2)
        boxes.append(b["L"]); recs.append(b["rec"])
    q = 300.0 * 0.1 ** 2 / 0.002

    def shaped(sys_):
        sh = _capi.Shape(lpi=8, step_lpi=8, step_mpw=8, skin=1.0, cap=0, step_ms=0.0, step_half=half)
        sys_._check(sys_.L.g6_set_shape(sys_.ctx, ctypes.byref(sh)))
        return sys_

    s = shaped(g6.RigidWater("TIP4P", sizes, np.array(boxes), path="custom", rc=8.5))
    s.upload_state(np.concatenate(recs))
    log = s.md_run(0.002, 10, s.thermostats(3, "nose", temp=temps, q=q))
    got = s.download_state()
    off = np.concatenate([[0], np.cumsum(sizes)])
    for k, n in enumerate(sizes):
        one = shaped(g6.RigidWater("TIP4P", n, boxes[k], path="custom", rc=8.5))
        one.upload_state(recs[k])
        log1 = one.md_run(0.002, 10, one.thermostats(1, "nose", temp=temps[k], q=q))
        want = one.download_state()
        assert np.abs(got[off[k]:off[k + 1]] - want).max() <= 1e-10 * np.abs(want).max()
        for c in (0, 3, 5, 7):
            assert np.abs(log[:, k, c] - log1[:, 0, c]).max() <= 1e-10 * np.abs(log1[:, 0, c]).max() + 1e-14
        assert np.array_equal(log[:, k, 6], log1[:, 0, 6])


def test_nonfinite_state_is_reported():
    b = config.water_box("TIP4P", 256, 1)
    s = g6.RigidWater("TIP4P", 256, b["L"], rc=8.5)
    rec = b["rec"].copy()
    rec[7, 3:6] = np.nan      # a velocity that turns the COM into NaN after predict
    s.upload_state(rec)
    with pytest.raises(g6.G6Error) as e:
        s.md_run(0.002, 3)
    assert e.value.status == g6._capi.G6_ERR_NONFINITE


@pytest.mark.parametrize("half", [0, 1])
def test_host_buffer_step_recovers_row_overflow(half):
    """Host-buffer steps on a page-locked buffer with rows too short for the
    list: the overflow flag comes back through the pinned block, the step is
    repeated from the kept input records with a larger capacity, and three
    steps end where three steps of a context that never overflowed end (bit
    for bit with the full list, within FP32 summation order with the half)."""
    import ctypes
    import torch
    from genesis6_gb300 import _capi
    n = 512
    b = config.water_box("TIP4P", n, 44, temp=300.0, dt=0.002, jitter=0.2)
    q = 300.0 * 0.25 / 0.002
    out = []
    for cap in (0, 64):   # about 140 full-row or 70 half-row entries at rc + skin = 10 A
        s = g6.RigidWater("TIP4P", n, b["L"], path="custom", precision="mixed", rc=9.0)
        s.upload_state(b["rec"])
        sh = _capi.Shape(lpi=16, step_lpi=16, step_mpw=8, skin=1.0, cap=cap, step_ms=0.0, step_half=half)
        s._check(s.L.g6_set_shape(s.ctx, ctypes.byref(sh)))
        th = s.thermostats(1, "nose", temp=300.0, q=q)
        host = torch.empty((n, 53), dtype=torch.float64, pin_memory=True).numpy()
        host[:] = b["rec"]
        logs = []
        for _ in range(3):
            lg = np.zeros(10)
            s.md_step_host(0.002, host, th, lg)
            logs.append(lg)
        if cap:
            got = _capi.Shape()
            s._check(s.L.g6_get_shape(s.ctx, ctypes.byref(got)))
            assert got.cap > cap
        out.append((host.copy(), np.array(logs), list(th[0].zeta)))
    (ha, la, za), (hb, lb, zb) = out
    if half:
        assert np.abs(ha - hb).max() <= 1e-5 * np.abs(ha).max()
        cols = [0, 1, 2, 3, 5, 7]
        assert np.abs(la[:, cols] - lb[:, cols]).max() <= 1e-6 * np.abs(la[:, cols]).max()
        assert np.abs(la[:, 6] - lb[:, 6]).max() <= 2   # a pair at rc may fall on either side
    else:
        assert np.array_equal(ha, hb)
        assert np.array_equal(la[:, [0, 1, 2, 3, 4, 5, 6, 7, 9]], lb[:, [0, 1, 2, 3, 4, 5, 6, 7, 9]])
        assert za == zb


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_row_overflow_is_recovered(prec):
    """Neighbour-list rows longer than the capacity: g6_md_run puts the state
    back to the run's start, raises the capacity and repeats the run, so the
    result is the trajectory of a run that never overflowed; g6_md_end on its
    own reports G6_ERR_CAPACITY with the start state restored."""
    from genesis6_gb300 import _capi
    import ctypes
    n = 512
    b = config.water_box("TIP4P", n, 44, temp=300.0, dt=0.002, jitter=0.2)

    def make(cap):
        s = g6.RigidWater("TIP4P", n, b["L"], path="custom", precision=prec, rc=9.0)
        s.upload_state(b["rec"])
        sh = _capi.Shape(lpi=16, step_lpi=16, step_mpw=8, skin=1.0, cap=cap, step_ms=0.0)
        s._check(s.L.g6_set_shape(s.ctx, ctypes.byref(sh)))
        return s

    q = 300.0 * 0.25 / 0.002
    a = make(0)
    th_a = a.thermostats(1, "nose", temp=300.0, q=q)
    log_a = a.md_run(0.002, 20, th_a)
    s = make(64)                       # about 140 entries per row at rc + skin = 10 A
    th_s = s.thermostats(1, "nose", temp=300.0, q=q)
    log_s = s.md_run(0.002, 20, th_s)
    assert np.array_equal(a.download_state(), s.download_state())
    assert np.array_equal(log_a, log_s)
    assert list(th_a[0].zeta) == list(th_s[0].zeta)
    got = _capi.Shape()
    s._check(s.L.g6_get_shape(s.ctx, ctypes.byref(got)))
    assert got.cap > 64
    # the three-phase API: the overflow is reported and the start state restored
    t = make(64)
    th_t = t.thermostats(1, "nose", temp=300.0, q=q)
    assert t.L.g6_md_begin(t.ctx, 0.002, 5, th_t, 0) == _capi.G6_OK
    assert t.L.g6_md_advance(t.ctx, 5) == _capi.G6_OK
    assert t.L.g6_md_end(t.ctx, th_t, None) == _capi.G6_ERR_CAPACITY
    assert np.array_equal(t.download_state(), b["rec"])
    assert th_t[0].zeta[0] == 0.0
