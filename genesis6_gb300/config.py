"""Seeded synthetic configurations of rigid water.

The reference reads an @NX4A block (COM + quaternion per molecule,
RigidModule.F90:694-727) and draws Maxwell-Boltzmann velocities with
rigid_vreset2 (RigidModule.F90:1016-1053).  This module builds the same
content without input files: molecules on a simple-cubic lattice (the first n
sites in lexicographic order), uniformly random unit quaternions (normalised
4-D Gaussians), COM velocities N(0, kT/m) per axis and body-frame angular
velocities N(0, kT/I_k), net momentum removed.  Units are the reference's:
Angstrom, ps, amu, energy in 10 J/mol (kT = T * RGAS * J2I).
"""
from __future__ import annotations

import numpy as np

from . import _capi

RGAS = 6.0225e23 * 1.380066e-23   # PhysConst.F90:21-26
J2I = 0.1
DENSITY = 0.033456                 # molecules / A^3 at 1.0 g/cm^3 (M = 18)
REC = 53


def box_edge(n: int, density: float = DENSITY) -> float:
    return (n / density) ** (1.0 / 3.0)


def lattice(n: int, L: float) -> np.ndarray:
    m = int(np.ceil(n ** (1.0 / 3.0) - 1e-9))
    a = L / m
    idx = np.arange(m)
    g = np.stack(np.meshgrid(idx, idx, idx, indexing="ij"), -1).reshape(-1, 3)[:n]
    return (g + 0.5) * a - 0.5 * L


def random_quaternions(n: int, rng: np.random.Generator) -> np.ndarray:
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    return q


def rigid_records(com, quat, vel=None, omega=None, dt=0.002) -> np.ndarray:
    """Per-molecule 53-double records: com, d[5][3] (d[0] = v*dt), w[5][3], q[5][4]."""
    n = com.shape[0]
    rec = np.zeros((n, REC))
    rec[:, 0:3] = com
    if vel is not None:
        rec[:, 3:6] = vel * dt
    if omega is not None:
        rec[:, 18:21] = omega
    rec[:, 33:37] = quat
    return rec


def maxwell_boltzmann(n: int, temp: float, mass: float, inertia, rng: np.random.Generator):
    """Seeded Maxwell-Boltzmann velocities with rigid_vreset2's per-axis
    variances (RigidModule.F90:1016-1053): COM velocity N(0, kT/m), body-frame
    angular velocity N(0, kT/I_k), kT = temp * RGAS * J2I, from numpy's
    normal generator; the net COM momentum is removed.  Returns v, w (n,3)."""
    kT = temp * RGAS * J2I
    v = rng.standard_normal((n, 3)) * np.sqrt(kT / mass)
    v -= v.mean(axis=0, keepdims=True)
    w = rng.standard_normal((n, 3)) * np.sqrt(kT / np.asarray(inertia))[None, :]
    return v, w


def rigid_vreset2(temp: float, mass: float, inertia, u, dt: float):
    """Velocities exactly as rigid_vreset2 (RigidModule.F90:1016-1053) draws
    them from a given stream of uniforms u (n, 12) in (0, 1] (the values of
    Random_GetNext): per molecule the COM terms dx(1), dy(1), dz(1) =
    N(0, kT/m) * dt, then the body-frame wx(1), wy(1), wz(1) = N(0, kT/I_k),
    each normal from two consecutive numbers by Random_Normal
    (RandomModule.F90:28-36: sqrt(-2 log r1) sin(2 pi r2) sqrt(var)).  The
    reference does not remove the net momentum here.  Returns d1 (n,3), w1 (n,3)."""
    u = np.asarray(u, float).reshape(-1, 12)
    kT = temp * RGAS * J2I
    var = np.array([kT / mass] * 3 + [kT / float(i) for i in inertia])
    r1, r2 = u[:, 0::2], u[:, 1::2]
    z = np.sqrt(-2.0 * np.log(r1)) * np.sin(2.0 * 3.1415926535897932 * r2) * np.sqrt(var)[None, :]
    return z[:, :3] * dt, z[:, 3:].copy()


def water_box(model: str, n: int, seed: int, temp: float = 300.0, dt: float = 0.002, density: float = DENSITY,
              jitter: float = 0.0, info=None):
    """Seeded lattice configuration.  Returns dict(L=(3,), com, quat, rec).

    ``info`` (a dict with "mass" and "inertia") supplies the model's mass and
    principal moments; without it they come from g6_model_info in
    libg6gpu.so.  A caller that must not load the library (a CPU-only timing
    of the same workload) passes its own tables."""
    if info is None:
        info = _capi.model_info(model)
    rng = np.random.default_rng(seed)
    L = box_edge(n, density)
    com = lattice(n, L)
    if jitter > 0:
        com = com + rng.uniform(-jitter, jitter, com.shape)
    quat = random_quaternions(n, rng)
    v, w = maxwell_boltzmann(n, temp, info["mass"], info["inertia"], rng)
    return {"L": np.array([L, L, L]), "com": com, "quat": quat, "rec": rigid_records(com, quat, v, w, dt),
            "mass": info["mass"], "inertia": info["inertia"]}


def load_start(path: str, dt: float):
    """A stored starting state (npz with L, com, quat, d1 = v * dt_file, w1 and
    dt_file) as 53-double records for time step dt; the higher Gear terms are
    zero.  Returns dict(L=(3,), com, quat, rec)."""
    z = np.load(path)
    vel = z["d1"] / float(z["dt"])
    rec = rigid_records(z["com"], z["quat"], vel, z["w1"], dt)
    return {"L": np.asarray(z["L"], float), "com": rec[:, 0:3].copy(), "quat": rec[:, 33:37].copy(), "rec": rec}


def replica_sizes(nrep: int, lo: int, hi: int, seed: int) -> np.ndarray:
    """Replica sizes drawn log-uniformly in [lo, hi] (rounded)."""
    rng = np.random.default_rng(seed)
    return np.rint(np.exp(rng.uniform(np.log(lo), np.log(hi), nrep))).astype(np.int32)
