"""Injection through open faces (the OpenFlow boundary) against the FP64
oracle: with the same counter-based random streams the device and the oracle
inject the same particles (count, positions after the partial push, velocities)
on two faces of an open axis with drifting Maxwellians of two species, and the
deposited moments of the stepped plasma agree; the injected particles continue
the id sequence and survive later steps; a rate sanity check against the
analytic Maxwellian flux."""
import ctypes as C

import numpy as np
import pytest

from tests import gpu_cases as G
from tests import oracle_lib as O
from tests.oracle_lib import p

pytestmark = pytest.mark.gpu


@pytest.fixture
def lib():
    L = O.load()
    yield L
    L.orc_set_open_axes(0)


def sources(wl):
    e, i = wl.species
    # (face, species, density, vth, drift): ~2 particles per boundary cell face
    return [(0, 0, 2000.0 * e.weight, e.vth, (0.02, 0.0, 0.0)),
            (1, 1, 2000.0 * i.weight, i.vth, (-0.004, 0.001, 0.0))]


def oracle_injection(lib, st, srcs, seed, step):
    out_x, out_v = [], []
    for s, (face, spec, dens, vth, drift) in enumerate(srcs):
        cap = 200000
        xo, vo = np.zeros((cap, 3)), np.zeros((cap, 3))
        blk, cel = np.zeros(cap, np.int32), np.zeros(cap, np.int32)
        dr = np.array(drift, np.float64)
        k = lib.orc_inject(C.byref(st.m), face, spec, dens, p(dr), vth, seed, step, s, p(st.E_half),
                           p(st.Bprev), cap, p(xo), p(vo), p(blk, C.c_int32), p(cel, C.c_int32))
        assert 0 <= k <= cap
        out_x.append(xo[:k]); out_v.append(vo[:k])
    return np.concatenate(out_x), np.concatenate(out_v), [len(a) for a in out_x]


def match(gx, ox):
    """index into ox of the nearest oracle particle to each device particle
    (positions and velocities are compared through this pairing, which must
    be one to one)"""
    d2 = ((gx[:, None, :] - ox[None, :, :]) ** 2).sum(axis=2)
    m = np.argmin(d2, axis=1)
    assert len(np.unique(m)) == len(m)
    return m


def test_injection_matches_oracle(lib):
    wl, ic, x, f = G.make_case(nb=(2, 2, 2), ppc=8, seed=51)
    srcs = sources(wl)
    lib.orc_set_open_axes(1)
    with G.gpu_ctx(wl, ic, x, f) as ctx:
        ctx.set_open_axes(True, False, False)
        ctx.set_injection_seed(77)
        for face, spec, dens, vth, drift in srcs:
            ctx.add_injection(face, spec, dens, vth, drift)
        n0 = ctx.num_particles()
        ctx.push_deposit()
        st = G.oracle_state(wl, ic, x, f)
        st.push()
        xi, vi, per = oracle_injection(lib, st, srcs, 77, 0)
        assert min(per) > 50
        ninj = ctx.injected_particles()
        assert ninj == len(xi)
        alive = st.block >= 0
        assert ctx.num_particles() == n0 - (~alive).sum() + ninj
        g = G.by_id(ctx.export_particles())
        new = g["id"] >= n0
        assert new.sum() == ninj
        np.testing.assert_array_equal(np.sort(g["id"][new]), n0 + np.arange(ninj))
        gx, gv = g["x"][new], g["v"][new]
        m = match(gx, xi)
        assert np.abs(gx - xi[m]).max() <= 4e-6
        assert np.abs(gv - vi[m]).max() <= 2e-5 * np.abs(vi).max()
        # moments of the stepped plasma: survivors and injected particles
        keep = st.block >= 0
        spec_new = np.concatenate([np.full(k, srcs[s][1], np.uint8) for s, k in enumerate(per)])
        o2 = O.OracleState(wl, np.concatenate([st.x[keep], xi]), np.concatenate([st.v[keep], vi]),
                           np.concatenate([st.spec[keep], spec_new]), f)
        o2.Bcur[:] = st.Bcur
        o2.deposit()
        J, M = ctx.export_moments()
        assert G.rel_err(J, o2.J) <= 1e-5 and G.rel_err(M, o2.M) <= 1e-5
        # a second step: new stream, ids continue
        ctx.push_deposit()
        assert ctx.injected_particles() > ninj


def test_injection_rate_follows_the_maxwellian_flux(lib):
    wl, ic, x, f = G.make_case(nb=(2, 2, 2), ppc=4, seed=52, e_amp=0.0, b_amp=0.0)
    e = wl.species[0]
    with G.gpu_ctx(wl, ic, x, f) as ctx:
        ctx.set_open_axes(False, False, True)
        ctx.add_injection(4, 0, 3000.0 * e.weight, e.vth)
        tot = 0
        for _ in range(5):
            before = ctx.injected_particles()
            ctx.push_deposit()
            tot += ctx.injected_particles() - before
    area = (16 * wl.mesh.dx) ** 2
    expected = 5 * 3000.0 * e.vth / np.sqrt(2 * np.pi) * area * wl.dt
    assert abs(tot - expected) < 5 * np.sqrt(expected), (tot, expected)
