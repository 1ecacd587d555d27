"""GPU parity of the ECSIM hot path against the FP64 oracle, through the C ABI.

Tolerances (FP32 push/deposit against FP64):
  positions  |dx| <= 4e-6 cell            (FP32 block-local offsets: ulp(8) = 4.8e-7)
  velocities |dv| <= 2e-5 * max|v|
  J, M       max|d| / max|ref| <= 1e-5    (the 1e-5 field/moment target)
  energies   relative 1e-6
  block / cell ids bit-exact except particles whose FP64 position lies within
  2e-6 cell of a cell face (these are counted and reported)
Field solve (FP64 both sides, GMRES to 1e-11): relative 1e-8.
"""
import numpy as np
import pytest

import amps_gb300 as A
from tests import gpu_cases as G
from tests import oracle_lib as O

pytestmark = pytest.mark.gpu


def compare_particles(ctx, st, pos_tol=4e-6, face_eps=2e-6):
    g = G.by_id(ctx.export_particles())
    assert len(g["id"]) == len(st.spec)
    np.testing.assert_array_equal(g["id"], np.arange(len(st.spec)))
    np.testing.assert_array_equal(g["spec"], st.spec)
    dxp = np.abs(g["x"] - st.x)
    L = np.array(st.wl.mesh.shape) * st.wl.mesh.dx  # domain length per axis
    dxp = np.minimum(dxp, np.abs(dxp - L))   # periodic images
    assert dxp.max() <= pos_tol, dxp.max()
    vmax = np.abs(st.v).max()
    assert np.abs(g["v"] - st.v).max() <= 2e-5 * vmax
    mism = (g["block"] != st.block) | (g["cell"] != st.cell)
    near = G.face_distance(st.x) < face_eps
    assert not (mism & ~near).any(), np.flatnonzero(mism & ~near)[:10]
    return int(mism.sum()), int(near.sum())


@pytest.mark.parametrize("vscale", [1.0, 40.0])
def test_push_matches_oracle(vscale):
    wl, ic, x, f = G.make_case(vscale=vscale)
    ctx = G.gpu_ctx(wl, ic, x, f)
    st = G.oracle_state(wl, ic, x, f)
    # import locates particles with the reference rules
    g0 = G.by_id(ctx.export_particles())
    np.testing.assert_array_equal(g0["block"], st.block)
    np.testing.assert_array_equal(g0["cell"], st.cell)
    np.testing.assert_array_equal(g0["x"], st.x)
    nout = ctx.MoveParticles()
    assert nout == 0
    assert st.push() == 0
    mism, near = compare_particles(ctx, st)
    print("push vscale=%g: %d id mismatches, %d particles within 2e-6 of a face" % (vscale, mism, near))
    if vscale > 1:
        g1 = G.by_id(ctx.export_particles())
        # block crossings, including the periodic wrap, were exercised
        assert (g1["block"] != g0["block"]).sum() > 1000


def test_deposit_matches_oracle():
    wl, ic, x, f = G.make_case()
    ctx = G.gpu_ctx(wl, ic, x, f)
    st = G.oracle_state(wl, ic, x, f)
    eg = ctx.UpdateJMassMatrix()
    eo = st.deposit()
    J, M = ctx.export_moments()
    assert G.rel_err(J, st.J) <= 1e-5, G.rel_err(J, st.J)
    assert G.rel_err(M, st.M) <= 1e-5, G.rel_err(M, st.M)
    # diagonal 3x3 self-blocks separately (largest terms)
    assert G.rel_err(M[:, :9], st.M[:, :9]) <= 1e-5
    assert eg == pytest.approx(eo, rel=1e-6)


def test_deposit_with_weight_correction():
    wl, ic, x, f = G.make_case(nb=(1, 1, 2), ppc=4)
    rng = np.random.default_rng(3)
    wc = rng.uniform(0.5, 2.0, len(ic["spec"])).astype(np.float32).astype(np.float64)
    ctx = G.gpu_ctx(wl, ic, x, f, wcorr=wc)
    st = G.oracle_state(wl, ic, x, f, wcorr=wc)
    eg = ctx.UpdateJMassMatrix()
    eo = st.deposit()
    J, M = ctx.export_moments()
    assert G.rel_err(J, st.J) <= 1e-5
    assert G.rel_err(M, st.M) <= 1e-5
    assert eg == pytest.approx(eo, rel=1e-6)


def oracle_field_solve(st, tol, precond):
    lib = O.load()
    b = st.rhs()
    xs = np.zeros_like(b)
    res = np.zeros(1)
    it = lib.orc_gmres(O.C.byref(st.m), O.p(st.M), O.p(b), O.p(xs), tol, 500, 30, precond, O.p(res))
    assert it > 0
    Eh = st.E_n + xs
    Bn = np.zeros_like(st.Bcen)
    lib.orc_update_b(O.C.byref(st.m), O.p(Eh), O.p(st.Bcen), O.p(Bn))
    Bc = np.zeros_like(Bn)
    lib.orc_center_to_corner(O.C.byref(st.m), O.p(Bn), O.p(Bc))
    En = st.E_n.copy()
    wave = lib.orc_update_e(O.C.byref(st.m), O.p(Eh), O.p(En), O.p(Bn))
    return {"E_half": Eh, "B_center": Bn, "B_corner_cur": Bc, "E_n": En, "wave": wave, "it": it}


@pytest.mark.parametrize("precond", [0, 1])
def test_field_solve_matches_oracle(precond):
    wl, ic, x, f = G.make_case(nb=(2, 2, 1), ppc=8)
    st = G.oracle_state(wl, ic, x, f)
    st.deposit()
    ctx = G.gpu_ctx(wl, ic, x, f)
    ctx.import_moments(st.J, st.M)
    s = ctx.TimeStep(tol=1e-11, maxit=400, precond=precond)
    assert s.converged == 1 and s.rel_residual <= 1e-10
    ref = oracle_field_solve(st, 1e-11, precond)
    out = ctx.export_fields()
    for k in ("E_half", "B_center", "B_corner_cur", "E_n"):
        assert G.rel_err(out[k], ref[k]) <= 1e-8, (k, G.rel_err(out[k], ref[k]))
    np.testing.assert_allclose(out["B_corner_prev"], f["B_corner_cur"], rtol=0, atol=0)
    assert s.wave_energy == pytest.approx(ref["wave"], rel=1e-10)
    print("GMRES precond=%d: gpu %d iterations, oracle %d" % (precond, s.iterations, ref["it"]))


def test_full_steps_match_oracle_and_conserve_energy():
    wl, ic, x, f = G.make_case(nb=(2, 2, 2), ppc=8, e_amp=0.0, b_amp=0.0)
    ctx = G.gpu_ctx(wl, ic, x, f)
    st = G.oracle_state(wl, ic, x, f)
    e0 = st.deposit()
    wave0 = np.sum(st.Bcen ** 2 + st.E_n ** 2) / (8 * np.pi)
    tot0 = e0 + wave0
    for _ in range(3):
        s = ctx.PicTimeStep(tol=1e-10, maxit=400, precond=1)
        it, diag = st.step(tol=1e-10, maxit=400, precond=1)
        assert s.solve.converged == 1
        assert s.particle_energy == pytest.approx(diag[0], rel=1e-6)
        assert s.solve.wave_energy == pytest.approx(diag[1], rel=1e-5)
        drift = abs(s.particle_energy + s.solve.wave_energy - tot0) / tot0
        assert drift < 1e-6, drift
    out = ctx.export_fields()
    J, M = ctx.export_moments()
    # field perturbations are tiny relative to B0: compare perturbation parts
    for k, ref in (("E_n", st.E_n), ("E_half", st.E_half)):
        assert G.rel_err(out[k], ref) <= 1e-4, (k, G.rel_err(out[k], ref))
    assert G.rel_err(out["B_center"] - np.array(wl.b0), st.Bcen - np.array(wl.b0)) <= 1e-4
    assert G.rel_err(J, st.J) <= 1e-5 and G.rel_err(M, st.M) <= 1e-5
    compare_particles(ctx, st, pos_tol=2e-5)


def test_empty_particle_set():
    wl, ic, x, f = G.make_case(nb=(1, 1, 1), ppc=1)
    ctx = A.EcsimContext(wl, capacity=16, track_ids=True)
    ctx.import_fields(**f)
    ctx.import_particles(np.zeros((0, 3)), np.zeros((0, 3)), np.zeros(0, np.uint8))
    assert ctx.num_particles() == 0
    e = ctx.push_deposit()
    J, M = ctx.export_moments()
    assert e == 0.0 and not J.any() and not M.any()
    s = ctx.PicTimeStep(tol=1e-8, maxit=50, precond=0)
    assert s.solve.converged == 1


def test_capacity_and_argument_errors():
    wl, ic, x, f = G.make_case(nb=(1, 1, 1), ppc=2)
    ctx = A.EcsimContext(wl, capacity=10)
    with pytest.raises(A.AmpsGpuError) as e:
        ctx.import_particles(x, ic["v"].astype(np.float64), ic["spec"])
    assert e.value.status == 6
    with pytest.raises(A.AmpsGpuError) as e:
        ctx.TimeStep(tol=-1.0)
    assert e.value.status == 1
    bad = A.electron_proton_plasma("bad", 0, 1, 1, 1, 1)
    with pytest.raises(A.AmpsGpuError) as e:
        A.EcsimContext(bad)
    assert e.value.status == 1


def test_gmres_not_converged_reports_status():
    wl, ic, x, f = G.make_case(nb=(1, 1, 1), ppc=4)
    ctx = G.gpu_ctx(wl, ic, x, f)
    ctx.UpdateJMassMatrix()
    with pytest.raises(A.AmpsGpuError) as e:
        ctx.TimeStep(tol=1e-14, maxit=1, precond=0)
    assert e.value.status == 3


def test_face_positions_import_and_wrap():
    wl = A.electron_proton_plasma("faces", 2, 1, 1, 1, 1)
    L = 16.0
    x = np.array([[0.0, 0.5, 0.5], [8.0, 0.5, 0.5], [16.0 - 1e-12, 3.0, 7.999999999],
                  [-1e-9, 0.25, 0.25], [16.0, 1.0, 1.0], [7.9999999999, 4.0, 4.0]])
    v = np.zeros_like(x)
    spec = np.zeros(len(x), np.uint8)
    ctx = A.EcsimContext(wl, capacity=16)
    ctx.import_fields(**A.initial_fields(wl))
    ctx.import_particles(x, v, spec)
    st = O.OracleState(wl, x, v, spec, A.initial_fields(wl))
    g = G.by_id(ctx.export_particles())
    np.testing.assert_array_equal(g["block"], st.block)
    np.testing.assert_array_equal(g["cell"], st.cell)
    assert np.all(g["x"] >= 0) and np.all(g["x"][:, 0] < L)


@pytest.mark.parametrize("vscale", [1.0, 8.0, 40.0])
def test_fused_push_deposit_matches_oracle(vscale):
    """One fused push + deposit step; vscale 40 moves most particles and
    overflows the per-cell slack, exercising the rebuild path."""
    wl, ic, x, f = G.make_case(vscale=vscale)
    ctx = G.gpu_ctx(wl, ic, x, f)
    st = G.oracle_state(wl, ic, x, f)
    eg = ctx.push_deposit()
    st.push()
    eo = st.deposit()
    compare_particles(ctx, st)
    J, M = ctx.export_moments()
    assert G.rel_err(J, st.J) <= 1e-5, G.rel_err(J, st.J)
    assert G.rel_err(M, st.M) <= 1e-5, G.rel_err(M, st.M)
    assert eg == pytest.approx(eo, rel=1e-6)


@pytest.mark.parametrize("chunk", [16, 32])
def test_arrivals_chunk_matches_oracle(chunk):
    """the arrivals kernel staging 16 or 32 arrivals at a time (the autotuner's
    two variants) gives the oracle's particles, J and M"""
    wl, ic, x, f = G.make_case(vscale=8.0)
    ctx = G.gpu_ctx(wl, ic, x, f)
    ctx.set_arrivals_chunk(chunk)
    assert ctx.particle_tuning()["arrivals_chunk"] == chunk
    st = G.oracle_state(wl, ic, x, f)
    eg = ctx.push_deposit()
    st.push()
    eo = st.deposit()
    compare_particles(ctx, st)
    J, M = ctx.export_moments()
    assert G.rel_err(J, st.J) <= 1e-5 and G.rel_err(M, st.M) <= 1e-5
    assert eg == pytest.approx(eo, rel=1e-6)


def test_fused_and_separate_paths_agree():
    wl, ic, x, f = G.make_case(vscale=4.0)
    a = G.gpu_ctx(wl, ic, x, f)
    b = G.gpu_ctx(wl, ic, x, f)
    ea = a.push_deposit()
    b.MoveParticles()
    eb = b.UpdateJMassMatrix()
    Ja, Ma = a.export_moments()
    Jb, Mb = b.export_moments()
    assert G.rel_err(Ja, Jb) <= 2e-6 and G.rel_err(Ma, Mb) <= 2e-6
    assert ea == pytest.approx(eb, rel=1e-6)
    pa, pb = G.by_id(a.export_particles()), G.by_id(b.export_particles())
    for k in ("x", "v", "block", "cell"):
        np.testing.assert_array_equal(pa[k], pb[k])


def test_many_steps_layout_invariants():
    wl, ic, x, f = G.make_case(nb=(2, 2, 2), ppc=8, vscale=3.0)
    ctx = G.gpu_ctx(wl, ic, x, f)
    n = len(ic["spec"])
    for _ in range(25):
        ctx.push_deposit(want_energy=False)
    g = ctx.export_particles()
    assert len(g["id"]) == n
    np.testing.assert_array_equal(np.sort(g["id"]), np.arange(n))
    # each particle lies inside the cell it is filed under
    org = A.block_origins(wl.mesh, g["block"])
    ci = np.stack([g["cell"] % 8, (g["cell"] // 8) % 8, g["cell"] // 64], 1)
    lo = org + ci * wl.mesh.dx
    assert np.all(g["x"] >= lo - 1e-12) and np.all(g["x"] < lo + wl.mesh.dx + 1e-12)
    # fused moments equal a fresh full deposit of the same layout
    J1, M1 = ctx.export_moments()
    ctx.UpdateJMassMatrix()
    J2, M2 = ctx.export_moments()
    assert G.rel_err(J1, J2) <= 2e-6 and G.rel_err(M1, M2) <= 2e-6


def check_layout_and_moments(ctx, wl, n):
    """every id once, each particle inside the cell it is filed under, fused
    moments equal to a fresh deposit of the layout"""
    g = ctx.export_particles()
    np.testing.assert_array_equal(np.sort(g["id"]), np.arange(n))
    org = A.block_origins(wl.mesh, g["block"])
    ci = np.stack([g["cell"] % 8, (g["cell"] // 8) % 8, g["cell"] // 64], 1)
    lo = org + ci * wl.mesh.dx
    assert np.all(g["x"] >= lo - 1e-12) and np.all(g["x"] < lo + wl.mesh.dx + 1e-12)
    J1, M1 = ctx.export_moments()
    ctx.UpdateJMassMatrix()
    J2, M2 = ctx.export_moments()
    assert G.rel_err(J1, J2) <= 2e-6 and G.rel_err(M1, M2) <= 2e-6


def row_case(name, cells, seed=5):
    """protons placed cell by cell: cells = [(ix, count, vx)] in the row
    (iy, iz) = (4, 4), offsets in [0.3, 0.7) of a cell, unperturbed fields"""
    wl = A.electron_proton_plasma(name, 2, 2, 2, 1, 3)
    rng = np.random.default_rng(seed)
    dx = wl.mesh.dx
    xs, vs = [], []
    for ix, m, vx in cells:
        off = rng.uniform(0.3, 0.7, (m, 3))
        xs.append((np.array([ix, 4, 4]) + off) * dx)
        vs.append(np.tile([vx, 0.0, 0.0], (m, 1)))
    x = np.concatenate(xs)
    v = np.concatenate(vs).astype(np.float32)
    ic = {"v": v, "spec": np.ones(len(x), np.uint8)}
    return wl, ic, x, A.initial_fields(wl)


def steps_match_oracle(ctx, st, steps):
    for _ in range(steps):
        ctx.push_deposit(want_energy=False)
        st.push()
        st.deposit()
        compare_particles(ctx, st)
        J, M = ctx.export_moments()
        assert G.rel_err(J, st.J) <= 1e-5 and G.rel_err(M, st.M) <= 1e-5


def test_overflow_fills_vacated_slots():
    """A periodic row of 16 cells, each with 30 protons at rest and 100 moving
    exactly one cell per step along x (the proton gyration is 0.002 rad per
    step).  Every cell receives 100 arrivals, more than its count/4 + 32 slack,
    while its own 100 leave: every step overflows, and every overflowed
    particle goes to a vacated slot and is deposited there (no relayout).
    Positions, J and M match the oracle after every step; the layout stays
    valid."""
    wl, ic, x, f = row_case("row", [(i, 30, 0.0) for i in range(16)] +
                            [(i, 100, 10.0) for i in range(16)])
    assert wl.mesh.dx / wl.dt == 10.0
    ctx = G.gpu_ctx(wl, ic, x, f)
    st = G.oracle_state(wl, ic, x, f)
    ctx.set_kernel_timing(True)
    steps_match_oracle(ctx, st, 4)
    kt = ctx.kernel_times()
    ctx.set_kernel_timing(False)
    assert kt.get("overflow_place", (0.0, 0))[1] == 4, kt
    assert kt.get("relayout", (0.0, 0))[1] == 0, kt
    check_layout_and_moments(ctx, wl, len(x))


def test_overflow_into_full_cells_rebuilds():
    """A conveyor: 64 protons at rest in cell (10, 4, 4) and 100 in each of the
    six cells behind it along x, moving exactly one cell per step (unperturbed
    fields; the proton gyration is 0.002 rad per step).  Every step the
    conveyor's front moves 100 particles into a cell with no vacated slots and
    fewer free slots (count/4 + 32), so the overflow cannot be placed and the
    layout is rebuilt from itself (particle buffers swapped): four relayouts in
    four steps.  Positions, J and M match the oracle after every step."""
    wl, ic, x, f = row_case("conveyor", [(10, 64, 0.0)] + [(10 - k, 100, 10.0) for k in range(1, 7)])
    dx = wl.mesh.dx
    n = len(x)
    ctx = G.gpu_ctx(wl, ic, x, f)
    st = G.oracle_state(wl, ic, x, f)
    ctx.set_kernel_timing(True)
    steps_match_oracle(ctx, st, 4)
    kt = ctx.kernel_times()
    ctx.set_kernel_timing(False)
    assert kt.get("relayout", (0.0, 0))[1] == 4, kt
    g = ctx.export_particles()
    ix = np.floor(g["x"][:, 0] / dx).astype(int)
    # the six moving columns now in cells 8..13, the resting 64 in cell 10
    expect = np.zeros(16, int)
    expect[8:14] = 100
    expect[10] += 64
    np.testing.assert_array_equal(np.bincount(ix, minlength=16), expect)
    check_layout_and_moments(ctx, wl, n)
