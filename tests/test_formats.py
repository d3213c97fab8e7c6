"""Genesis6 file formats (genesis6_gb300/formats.py).

The binary restart is checked against files packed here record by record in
the order and layout the reference writes them (Mixture.F90:2526-2598,
RigidModule.F90:801-828, NoseModule.F90:148-155, BoxModule.F90:147-154,
CutoffModule.F90:85-90, GridModule.F90:246-252, TimeModule.F90:16-23); the text
configuration against the list-directed layouts of RigidModule.F90:694-727 and
830-884.  The GPU test resumes an MD run from a restart file.
"""
import struct

import numpy as np
import pytest

from genesis6_gb300 import config, formats as F


def rec(body):
    return struct.pack("<i", len(body)) + body + struct.pack("<i", len(body))


def random_records(n, seed):
    rng = np.random.default_rng(seed)
    r = rng.normal(size=(n, F.REC))
    q = rng.normal(size=(n, 4))
    r[:, 33:37] = q / np.linalg.norm(q, axis=1, keepdims=True)
    return r


def reference_wtg2_columns(r, dt):
    """The implied-do order of Rigid_WriteBinaryWTG2 written out longhand:
    com x, y, z; ((dx(s), i), s); dy; dz; ((quat(s)%vec(c), i), s) for c = 1..4;
    ((wx(s), i), s); wy; wz -- with w in the external unit w * dt."""
    n = len(r)
    com, d, w, q = r[:, 0:3], r[:, 3:18].reshape(n, 5, 3), r[:, 18:33].reshape(n, 5, 3), r[:, 33:53].reshape(n, 5, 4)
    out = [com[:, 0], com[:, 1], com[:, 2]]
    for k in range(3):
        out += [d[:, s, k] for s in range(5)]
    for c in range(4):
        out += [q[:, s, c] for s in range(5)]
    for k in range(3):
        out += [w[:, s, k] * dt for s in range(5)]
    return np.concatenate(out)


def reference_restart_bytes(r, dt, L, rc, sw, voxa, nose, nstep, nloop, nlog, mol_id):
    """A TRAJOUT file as Mixture.F90:2526-2598 writes it for one rigid component
    (cutoff, box, grid, @NLOG, @DTPS, @ASTP, @NOS2 with q/dt, @TEST, @MDLP, @NCMP,
    then @FIXC, @ID08, @WTG2)."""
    b = b""
    b += rec(b"@RCOA") + rec(struct.pack("<2d", rc, sw))
    b += rec(b"@BOX3") + rec(struct.pack("<3d", *L))
    b += rec(b"@VOXA") + rec(struct.pack("<3d", *voxa))
    b += rec(b"@NLOG") + rec(struct.pack("<i", nlog))
    b += rec(b"@DTPS") + rec(struct.pack("<d", dt))
    b += rec(b"@ASTP") + rec(struct.pack("<i", nstep))
    temp, q, dump, zeta, zsum = nose
    b += rec(b"@NOS2") + rec(struct.pack("<9d", temp, q / dt, dump, *zeta, zsum))
    b += rec(b"@TEST")
    b += rec(b"@MDLP") + rec(struct.pack("<i", nloop))
    b += rec(b"@NCMP") + rec(struct.pack("<i", 1))
    b += rec(b"@FIXC") + rec(struct.pack("<i", 0))
    b += rec(b"@ID08") + rec(mol_id.encode())
    b += rec(b"@WTG2") + rec(struct.pack("<i", len(r)))
    b += rec(reference_wtg2_columns(r, dt).astype("<f8").tobytes())
    return b


NOSE = (300.0, 1.25e3, 0.0, (1e-3, -2e-5, 3e-7, -4e-9, 5e-11), 0.125)


def test_fortran_records_round_trip_and_reject_bad_markers():
    bodies = [b"@BOX3", struct.pack("<3d", 1.0, 2.0, 3.0), b"", b"x" * 1000]
    data = b"".join(rec(x) for x in bodies)
    assert F.read_records(data) == bodies
    bad = bytearray(data)
    bad[4 + 5] ^= 1   # trailing marker of the first record
    with pytest.raises(F.FormatError):
        F.read_records(bytes(bad))
    with pytest.raises(F.FormatError):
        F.read_records(data[:-2])


def test_read_restart_written_in_reference_layout():
    r = random_records(37, 1)
    dt = 0.002
    data = reference_restart_bytes(r, dt, (19.7, 19.8, 19.9), 8.5, 2.0, (3.0, 3.0, 3.0), NOSE, 1234, 1000, 10,
                                   "TIP4P   ")
    st = F.read_restart(data)
    assert np.array_equal(st.box, [19.7, 19.8, 19.9])
    assert (st.rc, st.switch, st.dt, st.nstep, st.nloop, st.nlog) == (8.5, 2.0, dt, 1234, 1000, 10)
    assert np.array_equal(st.voxa, [3.0, 3.0, 3.0])
    assert st.nose.temp == 300.0 and st.nose.zeta == NOSE[3] and st.nose.zetasum == 0.125
    assert st.nose.q == pytest.approx(NOSE[1], rel=1e-15)   # q/dt on file, q*dt... back to the run's q
    (c,) = st.components
    assert c.model == "TIP4P" and not c.fixed
    np.testing.assert_allclose(c.rec, r, rtol=1e-15, atol=0)   # w stacks: /dt of (w*dt)


def test_write_restart_is_the_reference_layout_and_round_trips():
    r = random_records(16, 2)
    dt = 0.001
    st = F.State(box=np.array([20.0, 20.0, 20.0]), rc=9.0, switch=2.0, voxa=np.array([4.5, 4.5, 4.5]), dt=dt,
                 nstep=77, nloop=500, nlog=5, nose=F.Nose(NOSE[0], NOSE[1], NOSE[2], NOSE[3], NOSE[4]),
                 components=[F.Component("ST2_____", r)])
    data = F.write_restart(st)
    ref = reference_restart_bytes(r, dt, (20.0, 20.0, 20.0), 9.0, 2.0, (4.5, 4.5, 4.5), NOSE, 77, 500, 5, "ST2_____")
    assert data == ref
    back = F.read_restart(data)
    np.testing.assert_allclose(back.components[0].rec, r, rtol=1e-15, atol=0)
    assert back.components[0].model == "ST2"


def test_read_restart_skips_unknown_and_old_nose_unit():
    r = random_records(3, 3)
    b = rec(b"@DTPS") + rec(struct.pack("<d", 0.002)) + rec(b"@XXXX") + rec(b"opaque")
    b += rec(b"@NOSE") + rec(struct.pack("<8d", 250.0, 2.0, 0.0, 0, 0, 0, 0, 0))
    b += rec(b"@ID08") + rec(b"TIP5P   ") + rec(b"@WTG2") + rec(struct.pack("<i", 3))
    b += rec(reference_wtg2_columns(r, 0.002).astype("<f8").tobytes())
    st = F.read_restart(b)
    assert st.components[0].model == "TIP5P"
    assert st.nose.q == pytest.approx(2.0 * F.NOSE_OLD_UNIT ** 2 * 0.002)   # NoseModule.F90:101, Mixture.F90:1206
    with pytest.raises(F.FormatError):   # a short @WTG2 record
        F.read_restart(b[:-20] + struct.pack("<i", 0))


def test_fortran_e17_10():
    # list of (value, what Fortran's e17.10 edit descriptor prints)
    for x, s in ((1.0, "   0.1000000000E+01"), (-2.5, "  -0.2500000000E+01"), (123.456789012345, "   0.1234567890E+03"),
                 (1e-7, "   0.1000000000E-06"), (0.0, "   0.0000000000E+00"), (9.99999999995, "   0.1000000000E+02")):
        assert F._e17(x) == s[-17:]


def test_text_configuration_nx4a_wtg3_and_round_trip():
    text = """@DTPS
0.002
@BOX3
 19.7 19.7 19.7
@RCOA
 8.5 2.0
@NOS2
 300.0 1.0e3 0.0 0 0 0 0 0 0
@MDLP
 1000
@XTRA comment kept
 1 2 3
@ID08
TIP4P
@NX4A
 2
 0.1E+01 0.2E+01 0.3E+01 1.0 0.0 0.0 0.0
 4.0 5.0 6.0
 0.0 1.0 0.0 0.0
"""
    st = F.read_config(text)
    assert st.dt == 0.002 and st.rc == 8.5 and st.switch == 2.0 and st.nloop == 1000
    assert st.nose.q == pytest.approx(1.0e3 * 0.002)
    (c,) = st.components
    assert c.model == "TIP4P"
    np.testing.assert_array_equal(c.rec[:, 0:3], [[1, 2, 3], [4, 5, 6]])
    np.testing.assert_array_equal(c.rec[:, 33:37], [[1, 0, 0, 0], [0, 1, 0, 0]])
    assert not c.rec[:, 3:33].any() and not c.rec[:, 37:].any()
    assert ("@XTRA", [" 1 2 3"]) in st.other
    back = F.read_config(F.write_config(st))
    np.testing.assert_allclose(back.components[0].rec, c.rec, rtol=1e-10)
    assert back.nose.q == pytest.approx(st.nose.q) and back.rc == 8.5
    # @WTG3: velocities in A/ps and angular velocities in rad/ps (RigidModule.F90:849-863)
    r = random_records(5, 4)
    wtg3 = "@DTPS\n0.002\n" + F.write_wtg3(F.Component("ST2_____", r), 0.002)
    c3 = F.read_config(wtg3).components[0]
    np.testing.assert_allclose(c3.rec[:, 0:6], r[:, 0:6], rtol=1e-9, atol=1e-12)   # 10 digits on file
    np.testing.assert_allclose(c3.rec[:, 18:21], r[:, 18:21], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(c3.rec[:, 33:37], r[:, 33:37], rtol=1e-9, atol=1e-12)


def test_logd_line_layout():
    log = np.array([-1000.0, 300.0, 290.0, 301.5, 12.0, -4.0e3, 0, 1e-3, 0, 5])
    line = F.logd_line(10, log, 256, 19.7 ** 3, 1.0e3, 0.002)
    head, body = line.splitlines()
    assert head == "@LOGD"
    assert len(body) == 10 + 15 * 25 and body[:10] == "%10d" % 10
    vals = [float(x) for x in body[10:].split()]
    assert vals[0] == 301.5 and vals[1] == 12.0 and vals[11] == -4.0e3 and vals[13] == -4.0e3
    # the Nose terms close the balance H = (Ep + Ek) I2J + nose_ep + nose_ek
    assert (vals[3] + vals[4]) / 1e-3 + (vals[7] + vals[8]) / 1e-3 == pytest.approx(-4.0e3)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_md_resumes_from_a_restart_file(precision):
    """A run split by a binary restart (write, read, new context) continues as
    the unsplit run: the file carries the Gear stacks and the Nose state."""
    import genesis6_gb300 as g6
    b = config.water_box("TIP4P", 256, 11, temp=300.0, dt=0.002, jitter=0.2)
    L = b["L"]
    dt, q = 0.002, 300.0 * 0.25 ** 2 / 0.002
    st0 = F.State(box=np.asarray(L, dtype=np.float64), rc=8.5, switch=2.0, dt=dt, nstep=0, nloop=40, nlog=1,
                  nose=F.Nose(300.0, q), components=[F.Component("TIP4P   ", b["rec"])])
    # unsplit: 40 steps
    s, th = F.system_from_state(F.read_restart(F.write_restart(st0)), precision=precision)
    log_a = s.md_run(dt, 40, th)
    rec_a = s.download_state()
    s.close()
    # split: 25 steps, restart file, new context, 15 steps
    s, th = F.system_from_state(F.read_restart(F.write_restart(st0)), precision=precision)
    s.md_run(dt, 25, th)
    mid = F.write_restart(F.state_from_system(s, th, st0, nstep=25))
    s.close()
    st1 = F.read_restart(mid)
    assert st1.nstep == 25
    s, th = F.system_from_state(st1, precision=precision)
    log_b = s.md_run(dt, 15, th)
    rec_b = s.download_state()
    s.close()
    # mixed: the split run builds its own neighbour list (another order of the
    # pair sums) and the half list adds the other molecule's share with atomics
    # in a varying order; 40 steps of a liquid amplify those FP32 roundings
    tol = 1e-9 if precision == "fp64" else 1e-4
    np.testing.assert_allclose(rec_b[:, 0:3], rec_a[:, 0:3], rtol=0, atol=tol)
    np.testing.assert_allclose(rec_b[:, 33:37], rec_a[:, 33:37], rtol=0, atol=tol)
    np.testing.assert_allclose(log_b[-1, 0, 5], log_a[-1, 0, 5], rtol=tol)   # H, with the Nose terms


def test_json_form_round_trips_through_the_restart():
    r = random_records(9, 6)
    st = F.State(box=np.array([20.0, 21.0, 22.0]), rc=9.0, switch=2.0, dt=0.002, nstep=5, nloop=100, nlog=2,
                 nose=F.Nose(300.0, 2.5, 0.0, (1e-3, 0, 0, 0, 0), 0.5), components=[F.Component("TIP5P   ", r)])
    back = F.read_restart(F.write_restart(F.state_from_json(F.state_to_json(st))))
    np.testing.assert_allclose(back.components[0].rec, r, rtol=1e-15, atol=0)
    assert back.components[0].model == "TIP5P" and back.nose.q == pytest.approx(2.5) and back.nstep == 5
    poses = F.state_from_json(F.state_to_json(st, poses_only=True)).components[0].rec
    assert np.array_equal(poses[:, 0:3], r[:, 0:3]) and np.array_equal(poses[:, 33:37], r[:, 33:37])
    assert not poses[:, 3:33].any()
