"""GPU ECSIM path on block-structured AMR meshes against the FP64 AMR oracle.

* import: block/cell of every particle located on the device equals the
  oracle's FP64 findTreeNode/FindCellIndex (bit-exact);
* deposition: per-cell J and mass-matrix partials (FP32 accumulation) within
  1e-5 of the FP64 oracle, particle energy within 1e-6;
* push + re-binning across coarse/fine interfaces: positions and velocities
  within 1e-5, block/cell assignments identical except for particles within
  1e-5 cell of a face;
* field solve (GMRES on the cell-assembled operator with hanging-corner
  constraints): E, B and the wave energy agree with the oracle's solve from
  the same moments to 1e-7;
* full steps: the GPU step matches the oracle step and conserves total energy;
* on a single-level AMR mesh the AMR context reproduces the uniform context.
"""
import numpy as np
import pytest

import amps_gb300 as A
from amps_gb300 import amr
from tests import oracle_amr as OA
from tests.gpu_cases import rel_err

pytestmark = pytest.mark.gpu


def amr_case(nb0=(4, 4, 4), lmax=1, ppc=8, seed=11, e_amp=2e-3, b_amp=0.05, vscale=1.0):
    mesh = amr.central_refined_mesh(nb0, lmax=lmax, frac=0.5)
    wl = A.electron_proton_plasma("amr", 1, 1, 1, ppc, 2)
    ic = amr.amr_initial_condition(mesh, wl.species, ppc, seed=seed)
    if vscale != 1.0:
        ic["v"] = (ic["v"] * np.float32(vscale)).astype(np.float32)
    x = mesh.block_origins()[ic["block"]] + ic["u"].astype(np.float64) * mesh.block_dx()[ic["block"]][:, None]
    rng = np.random.default_rng(seed)
    nc, ncell = mesh.ncorners, mesh.ncells
    f = {
        "E_n": e_amp * rng.standard_normal((nc, 3)),
        "E_half": e_amp * rng.standard_normal((nc, 3)),
        "B_center": np.array(wl.b0) + b_amp * rng.standard_normal((ncell, 3)),
        "B_corner_prev": np.array(wl.b0) + b_amp * rng.standard_normal((nc, 3)),
        "B_corner_cur": np.array(wl.b0) + b_amp * rng.standard_normal((nc, 3)),
    }
    return mesh, wl, ic, x, f


def oracle_for(mesh, wl, ic, x, f):
    ao = OA.AmrOracle(mesh, wl.species, wl.dt, wl.theta, x, ic["v"].astype(np.float64), ic["spec"])
    ao.E_n[:] = f["E_n"]
    ao.E_half[:] = f["E_half"]
    ao.Bcen[:] = f["B_center"]
    ao.Bprev[:] = f["B_corner_prev"]
    ao.Bcur[:] = f["B_corner_cur"]
    return ao


def gpu_for(mesh, wl, ic, x, f):
    ctx = A.EcsimContext(wl, capacity=len(ic["spec"]) + 1024, track_ids=True, amr_mesh=mesh)
    ctx.import_particles(x, ic["v"].astype(np.float64), ic["spec"])
    ctx.import_fields(**f)
    return ctx


def by_id(exp):
    order = np.argsort(exp["id"])
    return {k: v[order] for k, v in exp.items()}


def face_dist(mesh, x, block):
    u = (x - mesh.block_origins()[block]) / mesh.block_dx()[block][:, None]
    return np.min(np.abs(u - np.rint(u)), axis=1)


@pytest.fixture(scope="module")
def case():
    return amr_case()


def test_amr_import_locates_like_oracle(case):
    mesh, wl, ic, x, f = case
    ao = oracle_for(mesh, wl, ic, x, f)
    with gpu_for(mesh, wl, ic, x, f) as ctx:
        assert ctx.ncorners == mesh.ncorners and ctx.ncells == mesh.ncells
        e = by_id(ctx.export_particles())
    np.testing.assert_array_equal(e["block"], ao.block)
    np.testing.assert_array_equal(e["cell"], ao.cell)
    assert rel_err(e["x"], x) < 1e-7


def test_amr_deposit_matches_oracle(case):
    mesh, wl, ic, x, f = case
    ao = oracle_for(mesh, wl, ic, x, f)
    e_ref = ao.deposit()
    with gpu_for(mesh, wl, ic, x, f) as ctx:
        e_gpu = ctx.UpdateJMassMatrix()
        J, M = ctx.export_cell_moments()
    assert e_gpu == pytest.approx(e_ref, rel=1e-6)
    assert rel_err(J.ravel(), ao.cellJ) < 1e-5
    assert rel_err(M.ravel(), ao.cellM) < 1e-5
    # fine cells carry their own partials
    fine = np.repeat(mesh.level == 1, 512)
    assert rel_err(M[fine].ravel(), ao.cellM.reshape(-1, 324)[fine].ravel()) < 1e-5


@pytest.mark.parametrize("vscale", [1.0, 8.0])
def test_amr_push_crosses_levels_like_oracle(vscale):
    mesh, wl, ic, x, f = amr_case(seed=23, vscale=vscale)
    ao = oracle_for(mesh, wl, ic, x, f)
    with gpu_for(mesh, wl, ic, x, f) as ctx:
        ctx.MoveParticles()
        e = by_id(ctx.export_particles())
    blk0 = ao.block.copy()
    ao.push()
    assert len(e["x"]) == len(x)
    L = np.array(mesh.nfine, float) * mesh.dxf
    d = e["x"] - ao.x
    d -= L * np.rint(d / L)
    assert np.max(np.abs(d)) / mesh.dx0 < 1e-5
    assert rel_err(e["v"], ao.v) < 1e-5
    mism = (e["block"] != ao.block) | (e["cell"] != ao.cell)
    assert np.all(face_dist(mesh, ao.x[mism], ao.block[mism]) < 1e-5), mism.sum()
    assert mism.sum() <= max(2, len(x) // 10000)
    crossed = mesh.level[ao.block] != mesh.level[blk0]
    assert crossed.sum() > 0  # some particles changed level


@pytest.mark.parametrize("precond", [0, 1])
def test_amr_field_solve_matches_oracle(case, precond):
    mesh, wl, ic, x, f = case
    ao = oracle_for(mesh, wl, ic, x, f)
    with gpu_for(mesh, wl, ic, x, f) as ctx:
        ctx.UpdateJMassMatrix()
        J, M = ctx.export_cell_moments()
        st = ctx.TimeStep(tol=1e-11, maxit=600, precond=precond)
        g = ctx.export_fields()
    assert st.converged
    ao.cellJ[:] = J.ravel()
    ao.cellM[:] = M.ravel()
    it, wave = ao.field_solve(tol=1e-11, maxit=600)
    assert it > 0
    for k, ref in (("E_n", ao.E_n), ("E_half", ao.E_half), ("B_center", ao.Bcen),
                   ("B_corner_prev", ao.Bprev), ("B_corner_cur", ao.Bcur)):
        assert rel_err(g[k], ref) < 1e-7, k
    assert st.wave_energy == pytest.approx(wave, rel=1e-9)


def test_amr_steps_match_oracle_and_conserve_energy():
    mesh, wl, ic, x, f = amr_case(seed=5, e_amp=0.0, b_amp=0.0)
    f["B_corner_prev"][:] = wl.b0
    f["B_corner_cur"][:] = wl.b0
    ao = oracle_for(mesh, wl, ic, x, f)
    e0 = ao.deposit()
    tot0 = e0 + ao.wave_energy()
    with gpu_for(mesh, wl, ic, x, f) as ctx:
        for _ in range(3):
            s = ctx.PicTimeStep(tol=1e-12, maxit=600, precond=1)
            it, diag = ao.step(tol=1e-12, maxit=600)
            assert s.solve.converged and it > 0
            assert s.particle_energy == pytest.approx(diag[0], rel=1e-6)
            assert s.solve.wave_energy == pytest.approx(diag[1], rel=1e-4)
            drift = abs(s.particle_energy + s.solve.wave_energy - tot0) / tot0
            assert drift < 1e-6, drift
        assert ctx.num_particles() == len(x)


def test_amr_context_on_uniform_mesh_matches_uniform_context():
    nb = (2, 2, 2)
    wl = A.electron_proton_plasma("u", *nb, 8, 2)
    wl.seed = 9
    ic = A.make_initial_condition(wl, nthreads=2)
    mesh = amr.uniform_mesh(nb)
    rng = np.random.default_rng(9)
    n = mesh.ncorners
    # uniform context numbering: I + NX (J + NY K); AMR: mesh corners, cells by block
    xyz = mesh.corner_xyz.reshape(-1, 3)
    NX, NY, NZ = wl.mesh.shape
    gidx = xyz[:, 0] + NX * (xyz[:, 1] + NY * xyz[:, 2])
    b = np.repeat(np.arange(mesh.nblocks), 512)
    l = np.tile(np.arange(512), mesh.nblocks)
    bx, by, bz = b % nb[0], (b // nb[0]) % nb[1], b // (nb[0] * nb[1])
    cidx = (bx * 8 + (l & 7)) + NX * ((by * 8 + ((l >> 3) & 7)) + NY * (bz * 8 + (l >> 6)))
    fu = {"E_n": 2e-3 * rng.standard_normal((n, 3)), "E_half": 2e-3 * rng.standard_normal((n, 3)),
          "B_center": np.array(wl.b0) + 0.05 * rng.standard_normal((n, 3)),
          "B_corner_prev": np.array(wl.b0) + 0.05 * rng.standard_normal((n, 3)),
          "B_corner_cur": np.array(wl.b0) + 0.05 * rng.standard_normal((n, 3))}
    fa = {k: (v[cidx] if k == "B_center" else v[gidx]) for k, v in fu.items()}
    cap = len(ic["spec"]) + 1024
    with A.EcsimContext(wl, capacity=cap) as cu, \
            A.EcsimContext(wl, capacity=cap, amr_mesh=mesh) as ca:
        for c, fld in ((cu, fu), (ca, fa)):
            c.import_particles_local(ic["u"], ic["v"], ic["spec"], ic["block"])
            c.import_fields(**fld)
        su = cu.PicTimeStep(tol=1e-12, maxit=400, precond=1)
        sa = ca.PicTimeStep(tol=1e-12, maxit=400, precond=1)
        eu, ea = by_id(cu.export_particles()), by_id(ca.export_particles())
        gu, ga = cu.export_fields(), ca.export_fields()
    np.testing.assert_array_equal(eu["block"], ea["block"])
    np.testing.assert_array_equal(eu["cell"], ea["cell"])
    assert rel_err(ea["v"], eu["v"]) < 1e-6
    assert np.max(np.abs(ea["x"] - eu["x"])) < 1e-5
    # the uniform context sums the 8 cell partials of a corner in FP32 before
    # widening, the AMR context widens each partial: moments differ at FP32
    # rounding (~1e-7), the fields by less
    assert rel_err(ga["E_n"], gu["E_n"][gidx]) < 1e-6
    assert rel_err(ga["B_center"], gu["B_center"][cidx]) < 1e-6
    assert sa.solve.wave_energy == pytest.approx(su.solve.wave_energy, rel=1e-9)
    assert sa.particle_energy == pytest.approx(su.particle_energy, rel=1e-6)


TABLE_OFF = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]


def corner_sums(mesh, cellJ, cellM):
    """ProcessCell's flush (pic_field_solver_ecsim.cpp:2362-2426) of per-cell
    blocks (cellJ [cell][8 corners x 3], cellM [cell][36 pairs c2 <= c1][9])
    into the mesh's unique corners, in numpy"""
    nb = mesh.nblocks
    ncell = nb * 512
    l = np.arange(512)
    ci, cj, ck = l % 8, (l // 8) % 8, l // 64
    tab = mesh.corner_tab.reshape(nb, 729)
    cor = np.stack([tab[:, (ci + o[0]) + 9 * ((cj + o[1]) + 9 * (ck + o[2]))].reshape(ncell)
                    for o in TABLE_OFF], 1)                     # [cell][table corner]
    inv_v = np.repeat(1.0 / mesh.block_dx() ** 3, 512)
    J = np.zeros((mesh.ncorners, 3))
    M = np.zeros((mesh.ncorners, 243))
    cJ = cellJ.reshape(ncell, 8, 3)
    cM = cellM.reshape(ncell, 36, 9)
    dig = lambda d: 0 if d == 0 else (1 if d < 0 else 2)
    slot = lambda a, b: sum(dig(TABLE_OFF[b][x] - TABLE_OFF[a][x]) * 3 ** x for x in range(3))
    for c in range(8):
        np.add.at(J, cor[:, c], cJ[:, c] * inv_v[:, None])
    pr = 0
    for c1 in range(8):
        for c2 in range(c1 + 1):
            s1 = slot(c1, c2)
            np.add.at(M, (cor[:, c1][:, None], 9 * s1 + np.arange(9)[None, :]), cM[:, pr])
            if c1 != c2:
                s2 = slot(c2, c1)
                np.add.at(M, (cor[:, c2][:, None], 9 * s2 + np.arange(9)[None, :]), cM[:, pr])
            pr += 1
    return J, M


def test_amr_corner_moments_match_oracle():
    """export_moments on an AMR context: the corner layout of the per-cell
    blocks, against the same flush of the FP64 oracle's blocks"""
    mesh, wl, ic, x, f = amr_case(ppc=8, seed=31)
    with gpu_for(mesh, wl, ic, x, f) as ctx:
        ctx.UpdateJMassMatrix()
        J, M = ctx.export_moments()
        gJ, gM = ctx.export_cell_moments()
    ao = oracle_for(mesh, wl, ic, x, f)
    ao.deposit()
    rJ, rM = corner_sums(mesh, ao.cellJ, ao.cellM)
    assert J.shape == (mesh.ncorners, 3) and M.shape == (mesh.ncorners, 243)
    assert rel_err(J, rJ) <= 1e-5, rel_err(J, rJ)
    assert rel_err(M, rM) <= 1e-5, rel_err(M, rM)
    # the device's own per-cell blocks, flushed the same way, agree to rounding
    sJ, sM = corner_sums(mesh, gJ, gM)
    assert rel_err(J, sJ) <= 1e-12 and rel_err(M, sM) <= 1e-12
