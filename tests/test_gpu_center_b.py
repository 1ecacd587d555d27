"""GPU parity of the centre-B configuration (_PIC_FIELD_SOLVER_B_CENTER_BASED_,
the reference's default build) against the FP64 oracle, through the C ABI.

The particles see B interpolated from the cell centres with CellCentered::
Linear's trilinear stencil (pic_interpolation_routines.cpp:820-905): the push
(Lapenta2017, pic_mover_boris.cpp:979) reads centre B^n, the deposit
(ProcessCell, pic_field_solver_ecsim.cpp:2050-2117) centre B^{n+1}; E stays at
the corners.  The test fields give B_center its own perturbation, unrelated to
the corner B slots, so a kernel that read the corner B would fail.

Tolerances are those of the corner-B parity tests: positions 4e-6 cell,
velocities 2e-5 max|v|, J and M 1e-5 of max|ref|, energies 1e-6.
"""
import numpy as np
import pytest

import amps_gb300 as A
from tests import gpu_cases as G
from tests import oracle_lib as O
from tests.test_gpu_ecsim import compare_particles

pytestmark = pytest.mark.gpu


def centre_case(vscale=1.0, nb=(2, 2, 2), ppc=8, chunk=None):
    wl, ic, x, f = G.make_case(nb=nb, ppc=ppc, vscale=vscale)
    ctx = G.gpu_ctx(wl, ic, x, f)
    ctx.set_b_center(True)
    if chunk:
        ctx.set_arrivals_chunk(chunk)
    st = O.OracleState(wl, x, ic["v"].astype(np.float64), ic["spec"], f, b_center=True)
    return wl, ic, x, f, ctx, st


def check_moments(ctx, st, eg, eo):
    J, M = ctx.export_moments()
    assert G.rel_err(J, st.J) <= 1e-5, G.rel_err(J, st.J)
    assert G.rel_err(M, st.M) <= 1e-5, G.rel_err(M, st.M)
    assert eg == pytest.approx(eo, rel=1e-6)
    return J, M


def test_center_b_deposit_matches_oracle():
    """the full deposit (UpdateJMassMatrix) with B^{n+1} at the cell centres;
    the corner-B moments of the same particles differ well beyond the tolerance"""
    wl, ic, x, f, ctx, st = centre_case()
    eg = ctx.UpdateJMassMatrix()
    eo = st.deposit()
    J, M = check_moments(ctx, st, eg, eo)
    corner = G.oracle_state(wl, ic, x, f)
    corner.deposit()
    assert G.rel_err(M, corner.M) > 1e-3


@pytest.mark.parametrize("vscale", [1.0, 8.0, 40.0])
def test_center_b_fused_push_deposit_matches_oracle(vscale):
    """one fused push + deposit; at vscale 40 most particles change cell and
    the per-cell slack overflows (vacated-slot placement and the relayout
    deposit from the centre stencil too)"""
    wl, ic, x, f, ctx, st = centre_case(vscale=vscale)
    eg = ctx.push_deposit()
    st.push()
    eo = st.deposit()
    compare_particles(ctx, st)
    check_moments(ctx, st, eg, eo)


@pytest.mark.parametrize("chunk", [16, 32])
def test_center_b_arrivals_chunks(chunk):
    wl, ic, x, f, ctx, st = centre_case(vscale=8.0, chunk=chunk)
    eg = ctx.push_deposit()
    st.push()
    eo = st.deposit()
    compare_particles(ctx, st)
    check_moments(ctx, st, eg, eo)


def test_center_b_push_only_matches_oracle():
    wl, ic, x, f, ctx, st = centre_case(vscale=4.0)
    assert ctx.MoveParticles() == 0
    assert st.push() == 0
    compare_particles(ctx, st)


def test_center_b_full_steps_match_oracle():
    """three ECSIM steps (field solve, then push with centre B^n and deposit
    with centre B^{n+1}); the particle-step graphs are replayed across the
    swaps of the centre-B buffers"""
    wl, ic, x, f, ctx, st = centre_case(nb=(2, 2, 2), ppc=8)
    st.deposit()
    for _ in range(3):
        s = ctx.PicTimeStep(tol=1e-10, maxit=400, precond=1)
        it, diag = st.step(tol=1e-10, maxit=400, precond=1)
        assert s.solve.converged == 1
        assert s.particle_energy == pytest.approx(diag[0], rel=1e-6)
        assert s.solve.wave_energy == pytest.approx(diag[1], rel=1e-5)
    out = ctx.export_fields()
    for k, ref in (("E_n", st.E_n), ("E_half", st.E_half)):
        assert G.rel_err(out[k], ref) <= 1e-4, (k, G.rel_err(out[k], ref))
    assert G.rel_err(out["B_center"], st.Bcen) <= 1e-5
    J, M = ctx.export_moments()
    assert G.rel_err(J, st.J) <= 1e-5 and G.rel_err(M, st.M) <= 1e-5
    compare_particles(ctx, st, pos_tol=2e-5)


def test_center_b_switch_back_to_corners():
    """turning centre B off again restores the corner-B results"""
    wl, ic, x, f, ctx, st = centre_case(vscale=2.0)
    ctx.set_b_center(False)
    corner = G.oracle_state(wl, ic, x, f)
    eg = ctx.push_deposit()
    corner.push()
    eo = corner.deposit()
    compare_particles(ctx, corner)
    check_moments(ctx, corner, eg, eo)


def test_center_b_rejected_on_amr():
    """centre B is built for uniform meshes: an AMR context refuses it"""
    from tests.test_gpu_amr import amr_case, gpu_for
    mesh, wl, ic, x, f = amr_case(nb0=(2, 2, 2), ppc=2)
    ctx = gpu_for(mesh, wl, ic, x, f)
    with pytest.raises(A.AmpsGpuError):
        ctx.set_b_center(True)
    ctx.set_b_center(False)


def test_center_b_open_axes_and_graphs():
    """open x and z (fast particles leave and are deleted) with centre B, the
    step as a CUDA graph: the surviving set, states and moments match the
    centre-B oracle over two steps"""
    lib = O.load()
    lib.orc_set_open_axes(1 | 4)
    try:
        wl, ic, x, f, ctx, st = centre_case(vscale=40.0)
        ctx.set_open_axes(True, False, True)
        ctx.set_graphs(True)
        for step in range(2):
            eg = ctx.push_deposit()
            st.push()
            eo = st.deposit()
            alive = st.block >= 0
            assert ctx.num_particles() == int(alive.sum())
            g = G.by_id(ctx.export_particles())
            np.testing.assert_array_equal(g["id"], np.flatnonzero(alive))
            L = np.array(wl.mesh.shape) * wl.mesh.dx
            d = np.abs(g["x"] - st.x[alive])
            d = np.minimum(d, np.abs(d - L))
            assert d.max() <= 4e-6 * (step + 1)
            assert np.abs(g["v"] - st.v[alive]).max() <= 2e-5 * np.abs(st.v).max()
            check_moments(ctx, st, eg, eo)
        assert (st.block < 0).sum() > 100
    finally:
        lib.orc_set_open_axes(0)
