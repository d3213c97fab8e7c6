"""Genesis6 on-disk formats: the tagged text configuration and the binary
restart file, so that a Genesis6 run can continue on this library and back.

Text configuration (read from stdin by Mixture.F90:586-760 and mc2): a line
whose first five characters are a tag, then the tag's values on the following
lines, read list-directed.  Tags handled here:

    @ID08  molecule type of the next component (8 characters)
    @NX4A  n, then n lines com(3) quat(4)              (RigidModule.F90:694-727, 866-884)
    @WTG3  n, then n lines com(3) quat(4) v(3) [A/ps] w(3) [rad/ps]
                                                        (RigidModule.F90:830-863)
    @BOX3  box edges (BoxModule.F90:109-135)
    @RCOA  rc, switch width (CutoffModule.F90:73-98)
    @VOXA  requested cell edges (GridModule.F90:210-223)
    @DTPS  dt [ps] (TimeModule.F90:25-53)
    @NOS2  temp q dump zeta0..zeta4 zetasum (NoseModule.F90:120-173)
    @NOSE  temp q dump zeta0..zeta4, q in the old unit (NoseModule.F90:90-103)
    @MDLP, @NLOG, @SNPO, @SNPV, @NCMP, @FAST, @FIXC   one value each
Other tags are kept with their text lines until the next tag, so a
configuration survives a read/write round trip.

Binary restart (TRAJIN/TRAJOUT, Fortran unformatted sequential records with
4-byte little-endian length markers): a 5-character tag record followed by the
tag's data records (Mixture.F90:383-560 reads, 2526-2598 writes).  @WTG2 holds
n and then one record of 53 n doubles in column order: com x, y, z; dx, dy, dz
stacks (5 each); quaternion stacks per component; wx, wy, wz stacks
(RigidModule.F90:635-663, 801-828), with the angular stacks in the external
unit w * dt (RigidModule.F90:1639-1667).  The Nose mass is written as q / dt
(Mixture.F90:2545) and held as q * dt during a run (Mixture.F90:1206).

The per-molecule record of this library (53 doubles: com, d[5][3], w[5][3],
q[5][4]) holds the reference's internal units, so conversion is only the dt
factors above.
"""
from __future__ import annotations

import dataclasses
import io
import struct
from typing import Dict, List, Optional, Tuple

import numpy as np

REC = 53
NOSE_OLD_UNIT = 21.8852721616497249235   # NoseModule.F90:101 (@NOSE q scale, squared)
MODEL_IDS = {"TIP4P": "TIP4P   ", "TIP5P": "TIP5P   ", "ST2": "ST2_____", "SPCE": "SPC_E   "}   # RigidSetup.F90:33-58; SPCEModule.F90:19
ID_MODELS = {v.strip("_ ").upper(): k for k, v in MODEL_IDS.items()}


class FormatError(ValueError):
    pass


# ---------------------------------------------------------------------------
# Fortran unformatted sequential records
# ---------------------------------------------------------------------------
def read_records(data: bytes) -> List[bytes]:
    """Split a gfortran unformatted sequential file into its records."""
    out, pos = [], 0
    while pos < len(data):
        if pos + 4 > len(data):
            raise FormatError("truncated record marker at byte %d" % pos)
        (n,) = struct.unpack_from("<i", data, pos)
        if n < 0 or pos + 8 + n > len(data):
            raise FormatError("bad record length %d at byte %d" % (n, pos))
        body = data[pos + 4:pos + 4 + n]
        (m,) = struct.unpack_from("<i", data, pos + 4 + n)
        if m != n:
            raise FormatError("record markers differ (%d, %d) at byte %d" % (n, m, pos))
        out.append(body)
        pos += 8 + n
    return out


def pack_record(body: bytes) -> bytes:
    return struct.pack("<i", len(body)) + body + struct.pack("<i", len(body))


# ---------------------------------------------------------------------------
# Conversion between the reference's stacks and this library's record
# ---------------------------------------------------------------------------
def record_from_columns(cols: np.ndarray, dt: float) -> np.ndarray:
    """(53, n) in @WTG2 order (external unit) -> (n, 53) records (internal unit)."""
    n = cols.shape[1]
    rec = np.zeros((n, REC))
    rec[:, 0:3] = cols[0:3].T
    for k in range(3):                      # dx, dy, dz stacks: rows 3 + 5k + s
        for s in range(5):
            rec[:, 3 + 3 * s + k] = cols[3 + 5 * k + s]
    for c in range(4):                      # quaternion component c, stack s: rows 18 + 5c + s
        for s in range(5):
            rec[:, 33 + 4 * s + c] = cols[18 + 5 * c + s]
    for k in range(3):                      # wx, wy, wz stacks: rows 38 + 5k + s, w * dt on file
        for s in range(5):
            rec[:, 18 + 3 * s + k] = cols[38 + 5 * k + s] / dt
    return rec


def columns_from_record(rec: np.ndarray, dt: float) -> np.ndarray:
    rec = np.asarray(rec, dtype=np.float64)
    n = rec.shape[0]
    cols = np.zeros((REC, n))
    cols[0:3] = rec[:, 0:3].T
    for k in range(3):
        for s in range(5):
            cols[3 + 5 * k + s] = rec[:, 3 + 3 * s + k]
    for c in range(4):
        for s in range(5):
            cols[18 + 5 * c + s] = rec[:, 33 + 4 * s + c]
    for k in range(3):
        for s in range(5):
            cols[38 + 5 * k + s] = rec[:, 18 + 3 * s + k] * dt
    return cols


def record_from_poses(com, quat, vel=None, omega=None, dt: float = 1.0) -> np.ndarray:
    """Records with zero higher derivatives from poses (and, for @WTG3, the COM
    velocity [A/ps] and body angular velocity [rad/ps]: dx(1) = v dt, w(1) = w)."""
    com = np.asarray(com, dtype=np.float64).reshape(-1, 3)
    quat = np.asarray(quat, dtype=np.float64).reshape(-1, 4)
    rec = np.zeros((len(com), REC))
    rec[:, 0:3] = com
    rec[:, 33:37] = quat
    if vel is not None:
        rec[:, 3:6] = np.asarray(vel, dtype=np.float64).reshape(-1, 3) * dt
    if omega is not None:
        rec[:, 18:21] = np.asarray(omega, dtype=np.float64).reshape(-1, 3)
    return rec


# ---------------------------------------------------------------------------
# Restart state
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class Component:
    id: str                      # 8-character molecule type (@ID08)
    rec: np.ndarray              # (n, 53) records in internal units
    fixed: bool = False          # @FIXC

    @property
    def model(self) -> str:
        key = self.id.strip("_ ").upper()
        if key not in ID_MODELS:
            raise FormatError("molecule type %r is not a rigid water model of this library" % self.id)
        return ID_MODELS[key]


@dataclasses.dataclass
class Nose:
    temp: float
    q: float                     # as held during a run (internal form)
    dump: float = 0.0
    zeta: Tuple[float, ...] = (0.0, 0.0, 0.0, 0.0, 0.0)
    zetasum: float = 0.0


@dataclasses.dataclass
class State:
    box: Optional[np.ndarray] = None          # @BOX3
    rc: Optional[float] = None                # @RCOA rc
    switch: Optional[float] = None            # @RCOA rc - r_in
    voxa: Optional[np.ndarray] = None         # @VOXA
    dt: Optional[float] = None                # @DTPS [ps]
    nstep: Optional[int] = None               # @ASTP
    nloop: Optional[int] = None               # @MDLP
    nlog: Optional[int] = None                # @NLOG
    nose: Optional[Nose] = None               # @NOS2 / @NOSE
    components: List[Component] = dataclasses.field(default_factory=list)
    # tags carried through unchanged: (tag, [data records]) for binary files,
    # (tag, [text lines]) for text files
    other: List[Tuple[str, list]] = dataclasses.field(default_factory=list)
    scalars: Dict[str, int] = dataclasses.field(default_factory=dict)   # @SNPO, @SNPV, @NCMP, @FAST ...


def _dt_or_fail(st: State) -> float:
    if not st.dt:
        raise FormatError("@DTPS is needed to convert the angular stacks and the Nose mass")
    return st.dt


# ---------------------------------------------------------------------------
# Binary restart
# ---------------------------------------------------------------------------
# data records that follow a tag, and their layouts (Fortran default integer = int32)
_BIN_SIMPLE = {
    "@NLOG": "<i", "@ASTP": "<i", "@MDLP": "<i", "@NCMP": "<i", "@FIXC": "<i",
    "@BOX3": "<3d", "@BXLA": "<d", "@RCOA": "<2d", "@VOXA": "<3d", "@VOXN": "<3i",
    "@DTPS": "<d", "@DTSC": "<d", "@NOS2": "<9d", "@NOSE": "<8d", "@VCNT": "<id",
    "@BOOK": "<id", "@IVSC": "<iid",
}
_BIN_OPAQUE_ONE = {"@PCN5", "@NORT", "@VSTR"}   # one data record each, carried through


def read_restart(data: bytes) -> State:
    """Parse a binary restart (the bytes of a TRAJOUT file)."""
    recs = read_records(data)
    st = State()
    raw: Dict[str, tuple] = {}
    pending_id, pending_fixed = None, False
    i = 0
    while i < len(recs):
        tag = recs[i][:5].decode("latin-1") if len(recs[i]) >= 5 else ""
        i += 1
        if tag in _BIN_SIMPLE:
            fmt = _BIN_SIMPLE[tag]
            if i >= len(recs) or len(recs[i]) < struct.calcsize(fmt):
                raise FormatError("%s: missing or short data record" % tag)
            raw[tag] = struct.unpack_from(fmt, recs[i])
            i += 1
            if tag == "@FIXC":
                pending_fixed = raw[tag][0] != 0
            elif tag == "@IVSC" or tag == "@BOOK" or tag == "@VCNT" or tag == "@VOXN" or tag == "@DTSC":
                st.other.append((tag, [recs[i - 1]]))
        elif tag == "@ID08":
            if i >= len(recs):
                raise FormatError("@ID08: missing data record")
            pending_id = recs[i][:8].decode("latin-1")
            i += 1
        elif tag == "@WTG2":
            if i + 1 >= len(recs):
                raise FormatError("@WTG2: missing data records")
            (n,) = struct.unpack_from("<i", recs[i])
            body = recs[i + 1]
            if len(body) != 8 * REC * n:
                raise FormatError("@WTG2: %d bytes for %d molecules (expected %d)" % (len(body), n, 8 * REC * n))
            i += 2
            cols = np.frombuffer(body, dtype="<f8").reshape(REC, n).copy()
            st.components.append(Component(pending_id or "", cols, pending_fixed))   # converted below
            pending_id, pending_fixed = None, False
        elif tag == "@TIE4":
            (nt,) = struct.unpack_from("<i", recs[i])
            st.other.append((tag, recs[i:i + 1 + max(nt, 0)]))
            i += 1 + max(nt, 0)
        elif tag in _BIN_OPAQUE_ONE:
            st.other.append((tag, [recs[i]]))
            i += 1
        elif tag == "@TEST":
            st.other.append((tag, []))
        # any other record is skipped, as the reference's loop does (Mixture.F90:383-560)
    if "@DTPS" in raw:
        st.dt = raw["@DTPS"][0]
    elif "@DTSC" in raw:
        st.dt = raw["@DTSC"][0] * 1e12   # TimeModule.F90:55-64
    if "@BOX3" in raw:
        st.box = np.array(raw["@BOX3"])
    elif "@BXLA" in raw:
        st.box = np.full(3, raw["@BXLA"][0])
    if "@RCOA" in raw and raw["@RCOA"][0] > 0:
        st.rc, st.switch = raw["@RCOA"]
    if "@VOXA" in raw and raw["@VOXA"][0] > 0:
        st.voxa = np.array(raw["@VOXA"])
    for tag, key in (("@NLOG", "nlog"), ("@ASTP", "nstep"), ("@MDLP", "nloop")):
        if tag in raw:
            setattr(st, key, raw[tag][0])
    if "@NCMP" in raw:
        st.scalars["@NCMP"] = raw["@NCMP"][0]
    if st.components:
        dt = _dt_or_fail(st)
        for c in st.components:
            c.rec = record_from_columns(c.rec, dt)
    if "@NOS2" in raw or "@NOSE" in raw:
        dt = _dt_or_fail(st)
        if "@NOS2" in raw:
            v = raw["@NOS2"]
            q, zsum = v[1], v[8]
        else:
            v = raw["@NOSE"]
            q, zsum = v[1] * NOSE_OLD_UNIT ** 2, 0.0
        if v[0] >= 0.0:   # a negative temperature switches the thermostat off (NoseModule.F90:130)
            st.nose = Nose(v[0], q * dt, v[2], tuple(v[3:8]), zsum)
    return st


def write_restart(st: State) -> bytes:
    """Binary restart in the order Mixture.F90:2526-2598 writes it."""
    out = io.BytesIO()

    def tag(t):
        out.write(pack_record(t.encode("latin-1")))

    def rec(fmt, *v):
        out.write(pack_record(struct.pack(fmt, *v)))

    other = dict((t, r) for t, r in st.other)
    if st.rc:
        tag("@RCOA"); rec("<2d", st.rc, st.switch)
    if st.box is not None:
        tag("@BOX3"); rec("<3d", *np.asarray(st.box, dtype=np.float64))
    if "@BOOK" in other:
        tag("@BOOK"); out.write(pack_record(other["@BOOK"][0]))
    if st.voxa is not None:
        tag("@VOXA"); rec("<3d", *np.asarray(st.voxa, dtype=np.float64))
    elif "@VOXN" in other:
        tag("@VOXN"); out.write(pack_record(other["@VOXN"][0]))
    if "@VCNT" in other:
        tag("@VCNT"); out.write(pack_record(other["@VCNT"][0]))
    tag("@NLOG"); rec("<i", int(st.nlog or 0))
    dt = _dt_or_fail(st)
    tag("@DTPS"); rec("<d", dt)
    tag("@ASTP"); rec("<i", int(st.nstep or 0))
    if st.nose is not None:
        n = st.nose
        tag("@NOS2"); rec("<9d", n.temp, n.q / dt, n.dump, *n.zeta, n.zetasum)
    if "@PCN5" in other:
        tag("@PCN5"); out.write(pack_record(other["@PCN5"][0]))
    tag("@TEST")
    tag("@MDLP"); rec("<i", int(st.nloop or 0))
    tag("@NCMP"); rec("<i", len(st.components))
    if "@TIE4" in other:
        tag("@TIE4")
        for r in other["@TIE4"]:
            out.write(pack_record(r))
    for c in st.components:
        tag("@FIXC"); rec("<i", 1 if c.fixed else 0)
        tag("@ID08"); out.write(pack_record(c.id.ljust(8)[:8].encode("latin-1")))
        tag("@WTG2"); rec("<i", len(c.rec))
        out.write(pack_record(columns_from_record(c.rec, dt).astype("<f8").tobytes()))
    for t, r in st.other:
        if t == "@IVSC":
            tag("@IVSC"); out.write(pack_record(r[0]))
    return out.getvalue()


# ---------------------------------------------------------------------------
# Text configuration
# ---------------------------------------------------------------------------
_TEXT_SCALARS = ("@MDLP", "@NLOG", "@SNPO", "@SNPV", "@NCMP", "@FAST", "@PTSO", "@MDVW", "@ASTP")


def _floats(lines: List[str], need: int, start: int, tag: str) -> Tuple[List[float], int]:
    vals: List[float] = []
    k = start
    while len(vals) < need:
        if k >= len(lines):
            raise FormatError("%s: expected %d values" % (tag, need))
        vals.extend(float(x.replace("D", "E").replace("d", "e")) for x in lines[k].split())
        k += 1
    return vals[:need], k


def read_config(text: str) -> State:
    """Parse a tagged text configuration (list-directed values after each tag)."""
    lines = text.splitlines()
    st = State()
    pending_id, pending_fixed = None, False
    k = 0
    while k < len(lines):
        tag = lines[k][:5]
        k += 1
        if tag == "@ID08":
            pending_id = lines[k].split()[0].strip("'\"") if lines[k].split() else ""
            pending_id = pending_id.ljust(8)[:8]
            k += 1
        elif tag in ("@NX4A", "@WTG3"):
            n = int(lines[k].split()[0])
            k += 1
            width = 7 if tag == "@NX4A" else 13
            v, k = _floats(lines, width * n, k, tag)
            a = np.array(v).reshape(n, width)
            if tag == "@NX4A":
                rec = record_from_poses(a[:, 0:3], a[:, 3:7])
            else:
                rec = record_from_poses(a[:, 0:3], a[:, 3:7], a[:, 7:10], a[:, 10:13], _dt_or_fail(st))
            st.components.append(Component(pending_id or "", rec, pending_fixed))
            pending_id, pending_fixed = None, False
        elif tag == "@BOX3":
            v, k = _floats(lines, 3, k, tag)
            st.box = np.array(v)
        elif tag == "@RCOA":
            v, k = _floats(lines, 2, k, tag)
            if v[0] > 0:
                st.rc, st.switch = v
        elif tag == "@VOXA":
            v, k = _floats(lines, 3, k, tag)
            st.voxa = np.array(v) if v[0] > 0 else None
        elif tag == "@DTPS":
            v, k = _floats(lines, 1, k, tag)
            st.dt = v[0]
        elif tag in ("@NOS2", "@NOSE"):
            nv = 9 if tag == "@NOS2" else 8
            v, k = _floats(lines, nv, k, tag)
            q = v[1] if tag == "@NOS2" else v[1] * NOSE_OLD_UNIT ** 2
            # the run multiplies q by dt after the whole configuration is read (Mixture.F90:1206)
            st.nose = Nose(v[0], q, v[2], tuple(v[3:8]), v[8] if nv == 9 else 0.0) if v[0] >= 0.0 else None
            st.scalars["_nose_q_per_dt"] = 1
        elif tag == "@FIXC":
            pending_fixed = lines[k].strip().upper().lstrip(".").startswith("T")
            k += 1
        elif tag in _TEXT_SCALARS:
            v = int(lines[k].split()[0])
            k += 1
            {"@MDLP": lambda: setattr(st, "nloop", v), "@NLOG": lambda: setattr(st, "nlog", v),
             "@ASTP": lambda: setattr(st, "nstep", v)}.get(tag, lambda: st.scalars.__setitem__(tag, v))()
        elif tag.startswith("@"):
            body = []
            while k < len(lines) and not lines[k].startswith("@"):
                body.append(lines[k])
                k += 1
            st.other.append((tag, body))
    if st.nose is not None and st.scalars.pop("_nose_q_per_dt", 0):
        st.nose.q *= _dt_or_fail(st)
    return st


def _fe(x: float, w: int, d: int) -> str:
    """Fortran Ew.d: [-]0.<d digits>E+XX, right-aligned in w columns."""
    if x == 0.0:
        return ("0." + "0" * d + "E+00").rjust(w)
    mant, exp = ("%.*e" % (d - 1, abs(x))).split("e")   # the d significant digits, rounded
    return ("%s0.%sE%+03d" % ("-" if x < 0 else "", mant.replace(".", ""), int(exp) + 1)).rjust(w)


def _e17(x: float) -> str:
    return _fe(x, 17, 10)


def write_config(st: State) -> str:
    """Text configuration: the tags this module understands, then the others."""
    out: List[str] = []
    if st.dt is not None:
        out += ["@DTPS", " %.17g" % st.dt]
    if st.box is not None:
        out += ["@BOX3", " " + " ".join("%.17g" % x for x in st.box)]
    if st.rc:
        out += ["@RCOA", " %.17g %.17g" % (st.rc, st.switch)]
    if st.voxa is not None:
        out += ["@VOXA", " " + " ".join("%.17g" % x for x in st.voxa)]
    if st.nose is not None:
        n = st.nose
        q = n.q / _dt_or_fail(st)
        out += ["@NOS2", " " + " ".join("%.17g" % x for x in (n.temp, q, n.dump, *n.zeta, n.zetasum))]
    for tag, key in (("@MDLP", "nloop"), ("@NLOG", "nlog"), ("@ASTP", "nstep")):
        if getattr(st, key) is not None:
            out += [tag, " %d" % getattr(st, key)]
    for tag, v in st.scalars.items():
        out += [tag, " %d" % v]
    for c in st.components:
        if c.fixed:
            out += ["@FIXC", " T"]
        out += ["@ID08", c.id.ljust(8)[:8], "@NX4A", " %d" % len(c.rec)]
        for r in c.rec:
            out.append(" ".join(_e17(x) for x in (*r[0:3], *r[33:37])))
    for tag, body in st.other:
        if isinstance(body, list) and all(isinstance(b, str) for b in body):
            out += [tag] + body
    return "\n".join(out) + "\n"


def write_wtg3(component: Component, dt: float) -> str:
    """@WTG3 snapshot of one component (Rigid_WriteWTG3, RigidModule.F90:830-863)."""
    out = ["@ID08", component.id.ljust(8)[:8], "@WTG3", " %d" % len(component.rec)]
    for r in component.rec:
        vals = (*r[0:3], *r[33:37], *(r[3:6] / dt), *r[18:21])
        out.append(" ".join(_e17(x) for x in vals))
    return "\n".join(out) + "\n"


def logd_line(nstep: int, log: np.ndarray, nmol: int, volume: float, thermo_q: float, dt: float) -> str:
    """One @LOGD record (Mixture.F90:2429-2489) of a single rigid component from a
    per-step log row of this library ([0] Ep, [1] Ekt, [2] Ekr (internal), [3] T,
    [4] P, [5] H [J/mol], [7] zeta0): T, P, V, Ep and Ek of the component [kJ/mol],
    Ep and Ek per molecule, Nose potential and kinetic terms, the Andersen terms
    (0), H, the external energy (0), H again and the monitor energy (0)."""
    I2J, X2KX, RGAS = 10.0, 1e-3, 6.0225e23 * 1.380066e-23
    ep, ek = float(log[0]), float(log[1] + log[2])
    temp, press, h, z0 = float(log[3]), float(log[4]), float(log[5]), float(log[7])
    dof = 2.0 * I2J * ek / (RGAS * temp) if temp > 0 else 0.0
    nose_ek = z0 * z0 * thermo_q * dt * dof * 0.5 * RGAS
    nose_ep = h - (ep + ek) * I2J - nose_ek
    vals = [temp, press, volume, ep * I2J * X2KX, ek * I2J * X2KX, ep * I2J / nmol * X2KX, ek * I2J / nmol * X2KX,
            nose_ep * X2KX, nose_ek * X2KX, 0.0, 0.0, h, 0.0, h, 0.0]
    return "@LOGD\n%10d%s\n" % (nstep, "".join(" " + _fe(v, 24, 17) for v in vals))


# ---------------------------------------------------------------------------
# Systems from and to restart states
# ---------------------------------------------------------------------------
def system_from_state(st: State, *, path: str = "custom", precision: str = "mixed", skin: float = 1.0,
                      device: int = 0):
    """A RigidWater of the state's single rigid-water component with its box,
    cutoff and Gear stacks, plus the thermostat list for md_run."""
    from .system import RigidWater
    if len(st.components) != 1:
        raise FormatError("one rigid-water component is supported, found %d" % len(st.components))
    if st.box is None or not st.rc:
        raise FormatError("@BOX3 and @RCOA are needed")
    c = st.components[0]
    s = RigidWater(c.model, len(c.rec), st.box, path=path, precision=precision, rc=st.rc, switch=st.switch,
                   skin=skin, device=device)
    s.upload_state(c.rec)
    if st.nose is not None:
        th = RigidWater.thermostats(1, "nose", temp=st.nose.temp, q=st.nose.q, dump=st.nose.dump)
        for k in range(5):
            th[0].zeta[k] = st.nose.zeta[k]
        th[0].zetasum = st.nose.zetasum
    else:
        th = RigidWater.thermostats(1)
    return s, th


def state_from_system(s, thermo, st: State, nstep: Optional[int] = None) -> State:
    """The restart state after a run: st with the system's records, the
    thermostat's Nose state and the step counter."""
    rec = s.download_state()
    out = dataclasses.replace(st, components=[dataclasses.replace(st.components[0], rec=rec)])
    if nstep is not None:
        out.nstep = nstep
    if st.nose is not None and thermo is not None:
        t = thermo[0]
        out.nose = Nose(t.temp, t.q, t.dump, tuple(t.zeta[k] for k in range(5)), t.zetasum)
    return out


# ---------------------------------------------------------------------------
# JSON form of a configuration: one key per tag, the tag's values as on file
# ---------------------------------------------------------------------------
def state_to_json(st: State, poses_only: bool = False) -> str:
    """{"DTPS": dt, "BOX3": [...], "RCOA": [rc, width], "VOXA": [...], "NOS2": [temp, q/dt, dump,
    zeta0..4, zetasum], "MDLP"/"NLOG"/"ASTP": n, "components": [{"ID08": id, "FIXC": bool,
    "NX4A": [[com, quat], ...]} or {..., "WTG2": [[53 values], ...]}]}: the values the text and
    binary forms carry, with the records in this library's internal units (poses_only keeps
    com and quaternion only)."""
    import json
    d: Dict[str, object] = {}
    if st.dt is not None:
        d["DTPS"] = st.dt
    if st.box is not None:
        d["BOX3"] = [float(x) for x in st.box]
    if st.rc:
        d["RCOA"] = [st.rc, st.switch]
    if st.voxa is not None:
        d["VOXA"] = [float(x) for x in st.voxa]
    if st.nose is not None:
        n = st.nose
        d["NOS2"] = [n.temp, n.q / _dt_or_fail(st), n.dump, *n.zeta, n.zetasum]
    for tag, key in (("MDLP", "nloop"), ("NLOG", "nlog"), ("ASTP", "nstep")):
        if getattr(st, key) is not None:
            d[tag] = int(getattr(st, key))
    comps = []
    for c in st.components:
        e: Dict[str, object] = {"ID08": c.id.strip(), "FIXC": bool(c.fixed)}
        if poses_only:
            e["NX4A"] = np.concatenate([c.rec[:, 0:3], c.rec[:, 33:37]], axis=1).tolist()
        else:
            e["WTG2"] = np.asarray(c.rec).tolist()
        comps.append(e)
    d["components"] = comps
    return json.dumps(d)


def state_from_json(text: str) -> State:
    import json
    d = json.loads(text)
    st = State()
    st.dt = d.get("DTPS")
    if "BOX3" in d:
        st.box = np.asarray(d["BOX3"], dtype=np.float64)
    if "RCOA" in d and d["RCOA"][0] > 0:
        st.rc, st.switch = (float(v) for v in d["RCOA"])
    if "VOXA" in d and d["VOXA"][0] > 0:
        st.voxa = np.asarray(d["VOXA"], dtype=np.float64)
    if "NOS2" in d and d["NOS2"][0] >= 0:
        v = d["NOS2"]
        st.nose = Nose(v[0], v[1] * _dt_or_fail(st), v[2], tuple(v[3:8]), v[8])
    st.nloop, st.nlog, st.nstep = d.get("MDLP"), d.get("NLOG"), d.get("ASTP")
    for e in d.get("components", []):
        if "WTG2" in e:
            rec = np.asarray(e["WTG2"], dtype=np.float64).reshape(-1, REC)
        else:
            a = np.asarray(e["NX4A"], dtype=np.float64).reshape(-1, 7)
            rec = record_from_poses(a[:, 0:3], a[:, 3:7])
        st.components.append(Component(str(e["ID08"]).ljust(8)[:8], rec, bool(e.get("FIXC", False))))
    return st
