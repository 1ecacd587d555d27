"""Batched test-particle tracing workload of the cutoff-rigidity calculation
(srcEarth/gridless/CutoffRigidityGridless.cpp): protons started on a sphere of
radius 1.1 R_E with isotropic directions and rigidities log-uniform in a band,
traced in a dipole plus a uniform field until they hit the Earth (r < 1 R_E),
escape (r > 10 R_E) or exhaust the step budget."""
import numpy as np

from .ecsim import trace_dipole

R_E = 6371.2e3
Q_P = 1.602176634e-19
M_P = 1.007276466621 * 1.66053906660e-27
C_LIGHT = 299792458.0


def sphere_starts(n, seed, r0=1.1, rig_gv=(0.1, 20.0)):
    """n protons on r = r0 R_E, isotropic directions, rigidity log-uniform (GV)."""
    rng = np.random.default_rng(seed)
    mu = rng.uniform(-1, 1, n)
    ph = rng.uniform(0, 2 * np.pi, n)
    pos = np.stack([np.sqrt(1 - mu ** 2) * np.cos(ph), np.sqrt(1 - mu ** 2) * np.sin(ph), mu], 1)
    mu2 = rng.uniform(-1, 1, n)
    ph2 = rng.uniform(0, 2 * np.pi, n)
    d = np.stack([np.sqrt(1 - mu2 ** 2) * np.cos(ph2), np.sqrt(1 - mu2 ** 2) * np.sin(ph2), mu2], 1)
    R = 10 ** rng.uniform(np.log10(rig_gv[0] * 1e9), np.log10(rig_gv[1] * 1e9), n)
    x = np.ascontiguousarray(r0 * R_E * pos)
    p = np.ascontiguousarray((R * Q_P / C_LIGHT)[:, None] * d)
    return x, p


def trace_cutoff(n, seed=7, precision=0, max_steps=100000, b_eq=3.1e-5, b_south=5e-9,
                 device=0, starts=None):
    """Runs the workload (on `starts` = (x, p) when given, else n seeded starts);
    returns (x, p, status, steps, total_steps, kernel_ms)."""
    if starts is None:
        x, p = sphere_starts(n, seed)
    else:
        x, p = (np.ascontiguousarray(a[:n], np.float64).copy() for a in starts)
    st, steps, tot, ms = trace_dipole(x, p, Q_P, M_P, b_eq, R_E,
                                      np.array([0.0, 0.0, -b_south]), R_E, 10.0 * R_E, max_steps,
                                      0.15, 10.0, precision, device)
    return x, p, st, steps, tot, ms
