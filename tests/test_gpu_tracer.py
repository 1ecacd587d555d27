"""GPU relativistic test-particle tracing against the FP64 oracle and the
golden trajectories of the reference build (dipole + uniform southward field).

FP64 kernel: same status and step count as the oracle, end points within 1e-6
relative (rounding differs: the kernel runs in normalised units).
FP32 kernel: statuses agree for >= 90% of particles, step totals within 10%.
"""
import json
import os

import numpy as np
import pytest

import amps_gb300 as A
from tests import oracle_lib as O

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def golden():
    g = json.load(open(os.path.join(GOLD, "gridless_boris.json")))
    return g, np.array(g["x0"]), np.array(g["p0"])


def run(g, x0, p0, precision):
    x, p = x0.copy(), p0.copy()
    st, steps, tot, ms = A.trace_dipole(x, p, g["q"], g["m0"], g["b_eq"], g["r_e"],
                                        np.array(g["b_ext"]), g["r_in"], g["r_out"],
                                        g["max_steps"], g["dphi"], g["dt_max"], precision)
    return x, p, st, steps, tot


def test_fp64_tracer_matches_reference_golden():
    g, x0, p0 = golden()
    x, p, st, steps, tot = run(g, x0, p0, 0)
    np.testing.assert_array_equal(st, np.array(g["status"]))
    np.testing.assert_array_equal(steps, np.array(g["steps"]))
    assert tot == int(np.sum(steps))
    gx = np.array(g["x"])
    assert (np.linalg.norm(x - gx, axis=1) / np.linalg.norm(gx, axis=1)).max() < 1e-6


def sphere_starts(n, seed):
    rng = np.random.default_rng(seed)
    re_m = 6371.2e3
    q = 1.602176634e-19
    m0 = 1.007276466621 * 1.66053906660e-27
    c = 299792458.0
    mu = rng.uniform(-1, 1, n); ph = rng.uniform(0, 2 * np.pi, n)
    pos = np.stack([np.sqrt(1 - mu**2) * np.cos(ph), np.sqrt(1 - mu**2) * np.sin(ph), mu], 1)
    mu2 = rng.uniform(-1, 1, n); ph2 = rng.uniform(0, 2 * np.pi, n)
    d = np.stack([np.sqrt(1 - mu2**2) * np.cos(ph2), np.sqrt(1 - mu2**2) * np.sin(ph2), mu2], 1)
    R = 10 ** rng.uniform(8, np.log10(2e10), n)
    x = np.ascontiguousarray(1.1 * re_m * pos)
    p = np.ascontiguousarray((R * q / c)[:, None] * d)
    return x, p, q, m0, re_m


def test_fp64_tracer_matches_oracle_many_lifetimes():
    x0, p0, q, m0, re_m = sphere_starts(2000, 11)
    ext = np.array([0.0, 0.0, -5e-9])
    xo, po, so, sto, toto = O.trace(x0, p0, q, m0, 3.1e-5, re_m, ext, re_m, 10 * re_m, 4000,
                                    0.15, 10.0)
    x, p = x0.copy(), p0.copy()
    st, steps, tot, ms = A.trace_dipole(x, p, q, m0, 3.1e-5, re_m, ext, re_m, 10 * re_m, 4000,
                                        precision=0, dt_max=10.0)
    agree = (st == so) & (steps == sto)
    # marginal trajectories may cross a boundary one step apart after thousands
    # of steps (rounding differs between SI and normalised units)
    assert agree.mean() > 0.98, agree.mean()
    assert tot == int(steps.sum())
    ok = agree & (st != 0)
    rel = np.linalg.norm(x[ok] - xo[ok], axis=1) / np.linalg.norm(xo[ok], axis=1)
    # most trajectories agree to rounding; a few chaotic ones amplify it
    assert np.median(rel) < 1e-12 and np.quantile(rel, 0.95) < 1e-6
    # lifetimes are uneven (the point of the persistent kernel)
    assert steps.min() < 50 and steps.max() == 4000


def test_fp32_tracer_tracks_fp64():
    x0, p0, q, m0, re_m = sphere_starts(4000, 12)
    ext = np.array([0.0, 0.0, -5e-9])
    out = {}
    for prec in (0, 1):
        x, p = x0.copy(), p0.copy()
        out[prec] = A.trace_dipole(x, p, q, m0, 3.1e-5, re_m, ext, re_m, 10 * re_m, 3000,
                                   precision=prec, dt_max=10.0) + (x,)
    s64, n64, t64 = out[0][0], out[0][1], out[0][2]
    s32, n32, t32 = out[1][0], out[1][1], out[1][2]
    assert (s64 == s32).mean() > 0.9
    assert abs(t32 - t64) / t64 < 0.1


def test_tracer_argument_errors():
    x = np.zeros((1, 3)); p = np.zeros((1, 3))
    with pytest.raises(A.AmpsGpuError) as e:
        A.trace_dipole(x, p, 1.0, 1.0, 3.1e-5, 6.4e6, np.zeros(3), 6.4e6, 6.4e6, 10)
    assert e.value.status == 1
    st, steps, tot, ms = A.trace_dipole(np.zeros((0, 3)), np.zeros((0, 3)), 1.0, 1.0, 3.1e-5,
                                        6.4e6, np.zeros(3), 6.4e6, 6.4e7, 10)
    assert tot == 0
