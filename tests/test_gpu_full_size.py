"""Parity at full size: the periodic ECSIM plasma of 32^3 cells as 4^3 blocks
of 8^3 cells, electrons and protons at 64 particles per cell per species
(4,194,304 particles, seeded Maxwellian, v_th,e = 0.05c, B0 along z with
omega_pe/omega_ce = 2, dt = 0.1/omega_pe), two full ECSIM time steps
(UpdateJMassMatrix, field solve with Jacobi GMRES to 1e-8, push + deposit) on
the GPU through the C ABI and in the FP64 oracle from the same particles.

Tolerances, relative to the largest reference entry:
  E^n, E^{n+theta}, B (perturbation), corner J, corner M   1e-5
  particle energy 1e-6, wave energy 1e-5
  positions 4e-6 cell, velocities 2e-5 of max|v|
  block / cell ids: identical except particles whose two positions straddle a
  cell face within ULP_BOUND FP32 ulps of an offset in [4, 8) (tests/parity.py);
  the mismatch count is printed.
"""
import os

import numpy as np
import pytest

import amps_gb300 as A
from tests import gpu_cases as G
from tests import oracle_lib as O
from tests import parity as P

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("b_center", [False, True], ids=["corner_B", "centre_B"])
def test_uniform_plasma_two_steps_full_size(b_center):
    """b_center: the particles see B from the cell centres (the reference's
    default configuration) on the GPU and in the oracle"""
    wl = A.WORKLOADS["ecsim_32c_64ppc"]()
    ic = A.make_initial_condition(wl, nthreads=os.cpu_count() or 4)
    x = A.physical_positions(wl.mesh, ic["u"], ic["block"])
    v = ic["v"].astype(np.float64)
    f = A.initial_fields(wl)
    n = wl.nparticles
    assert n == 4194304
    ctx = A.EcsimContext(wl, capacity=n, track_ids=True)
    try:
        ctx.import_particles(x, v, ic["spec"])
        ctx.import_fields(**f)
        ctx.set_b_center(b_center)
        st = O.OracleState(wl, x, v, ic["spec"], f, b_center=b_center)
        eg = ctx.UpdateJMassMatrix()
        eo = st.deposit()
        assert eg == pytest.approx(eo, rel=1e-6)
        for step in range(2):
            s = ctx.PicTimeStep(tol=wl.tol, maxit=400, precond=1)
            it, diag = st.step(tol=wl.tol, maxit=400, precond=1)
            assert s.solve.converged == 1 and s.solve.rel_residual <= wl.tol
            assert s.particle_energy == pytest.approx(diag[0], rel=1e-6)
            assert s.solve.wave_energy == pytest.approx(diag[1], rel=1e-5)
            print("step %d: GMRES iterations gpu %d oracle %d" % (step, s.solve.iterations, it))
        out = ctx.export_fields()
        b0 = np.array(wl.b0)
        errs = {
            "E_n": G.rel_err(out["E_n"], st.E_n),
            "E_half": G.rel_err(out["E_half"], st.E_half),
            "B_center": G.rel_err(out["B_center"] - b0, st.Bcen - b0),
            "B_corner_cur": G.rel_err(out["B_corner_cur"] - b0, st.Bcur - b0),
        }
        J, M = ctx.export_moments()
        errs["J"] = G.rel_err(J, st.J)
        errs["M"] = G.rel_err(M, st.M)
        print("relative errors:", {k: "%.2e" % e for k, e in errs.items()})
        for k, e in errs.items():
            assert e <= 1e-5, (k, e)
        g = G.by_id(ctx.export_particles())
        np.testing.assert_array_equal(g["id"], np.arange(n))
        np.testing.assert_array_equal(g["spec"], st.spec)
        Ld = np.array(wl.mesh.shape, float) * wl.mesh.dx
        dxp = np.abs(g["x"] - st.x)
        dxp = np.minimum(dxp, np.abs(dxp - Ld))
        assert dxp.max() <= 4e-6, dxp.max()
        assert np.abs(g["v"] - st.v).max() <= 2e-5 * np.abs(st.v).max()
        nb = wl.mesh.nblocks
        rep = P.mismatch_report(g["x"], g["block"], g["cell"], st.x, st.block, st.cell,
                                A.block_origins(wl.mesh, np.arange(nb)),
                                np.full(nb, wl.mesh.dx), Ld)
        print("block/cell mismatches: %d of %d (largest position difference %.2f ulp of [4,8))"
              % (rep["mismatches"], n, rep["max_offset_ulps"]))
        assert rep["face_rule_holds"], rep["violations"]
        assert rep["mismatches"] <= 1e-5 * n
    finally:
        ctx.close()
