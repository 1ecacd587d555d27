"""The FP64 restatement of the div E correction (oracle/amps_oracle_dive.c,
ECSIM::divECorrection, src/pic/pic_field_solver_ecsim.cpp:4341-4364) checked by
the properties its steps must have: the discrete divergence of a sinusoidal
corner field, charge conservation of the cell-centred deposit, the Poisson
solve's residual, and a smaller Gauss-law residual after the correction.  (The
reference exits when the correction is switched on, :6168-6170: no reference
output exists.)"""
import ctypes as C

import numpy as np

from tests import gpu_cases as G
from tests import oracle_lib as O


def setup(seed=5):
    wl, ic, x, f = G.make_case(nb=(2, 2, 2), ppc=8, seed=seed)
    st = O.OracleState(wl, x, ic["v"].astype(np.float64), ic["spec"], f)
    return wl, st


def test_div_e_of_a_sinusoidal_field():
    wl, st = setup()
    NX, NY, NZ = wl.mesh.shape
    k = 2 * np.pi / (NX * wl.mesh.dx)
    h = np.arange(NX * NY * NZ)            # global corner order I + NX (J + NY K)
    xc = np.stack([h % NX, (h // NX) % NY, h // (NX * NY)], 1) * wl.mesh.dx
    E = np.zeros((len(xc), 3))
    E[:, 0] = np.sin(k * xc[:, 0])
    dive = np.zeros(len(xc))
    st.lib.orc_div_e(C.byref(st.m), O.p(E), O.p(dive))
    # the average of four edge differences of a field that varies along x only
    expect = (np.sin(k * (xc[:, 0] + wl.mesh.dx)) - np.sin(k * xc[:, 0])) / wl.mesh.dx
    np.testing.assert_allclose(dive, expect, atol=1e-12)


def test_net_charge_is_conserved():
    wl, st = setup()
    rho = np.zeros(wl.mesh.ncells)
    st.lib.orc_net_charge(C.byref(st.m), len(st.spec), O.p(st.x), O.p(st.spec, C.c_uint8), None,
                          O.p(st.block, C.c_int32), O.p(rho))
    q = np.array([s.charge * s.weight for s in wl.species])[st.spec]
    assert abs(rho.sum() * wl.mesh.dx ** 3 - q.sum()) <= 1e-12 * np.abs(q).sum()


def test_poisson_cg_reaches_its_tolerance():
    wl, st = setup()
    rng = np.random.default_rng(3)
    rhs = rng.standard_normal(wl.mesh.ncells)
    phi = np.zeros_like(rhs)
    rel = C.c_double()
    it = st.lib.orc_poisson_cg(C.byref(st.m), O.p(rhs), O.p(phi), 1e-10, 2000, C.byref(rel))
    assert rel.value <= 1e-10 and it < 2000
    # Laplacian(phi) = rhs - mean(rhs), checked with the 7-point formula
    NX, NY, NZ = wl.mesh.shape
    grid = phi.reshape(NZ, NY, NX)          # global cell order I + NX (J + NY K)
    lap = sum(np.roll(grid, s, a) for a in range(3) for s in (-1, 1)) - 6 * grid
    lap = lap.ravel() / wl.mesh.dx ** 2
    r = lap - (rhs - rhs.mean())
    assert np.linalg.norm(r) <= 1e-9 * np.linalg.norm(rhs - rhs.mean())


def test_correction_reduces_the_gauss_residual():
    wl, st = setup()
    st.step(tol=1e-10, maxit=200, precond=0)
    n_e = int((st.spec == 0).sum())
    for _ in range(2):
        r = st.div_e_correction(tol=1e-10, maxit=500)
        assert r["rel_residual"] <= 1e-10 and r["moved"] == n_e
        assert r["gauss_after"] < 0.5 * r["gauss_before"], r
