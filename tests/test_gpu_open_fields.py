"""Field boundary conditions on meshes with open (non-periodic) axes against
the FP64 oracle: the free corners on the open domain faces are constraint rows
of the field solve (Dirichlet dE = 0, Neumann dE = mean of the inward
face-normal donors), the cells on those faces take UpdateB's boundary branch
(Dirichlet keeps B^n, Neumann copies the mean of the inward neighbours), and
particles leaving through those faces are deleted.  Single-level and
two-level meshes, both boundary types, field solves and full ECSIM steps."""
import numpy as np
import pytest

import amps_gb300 as A
from amps_gb300 import amr
from tests import oracle_lib as O
from tests.gpu_cases import rel_err
from tests.test_gpu_amr import gpu_for, oracle_for

pytestmark = pytest.mark.gpu


def open_case(nb0, lmax, open_axes, field_bc, ppc=8, seed=81, e_amp=2e-3, b_amp=0.05, vscale=1.0):
    base = amr.central_refined_mesh(nb0, lmax=lmax, frac=0.5) if lmax else None
    leaves = base.leaves if base is not None else [
        (0, i * 8, j * 8, k * 8) for k in range(nb0[2]) for j in range(nb0[1]) for i in range(nb0[0])]
    mesh = amr.AmrMesh(nb0, lmax, leaves, open_axes=open_axes, field_bc=field_bc)
    wl = A.electron_proton_plasma("open", 1, 1, 1, ppc, 2)
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


@pytest.fixture
def open_oracle():
    lib = O.load()
    yield lib
    lib.orc_set_open_axes(0)


def boundary_cells(mesh):
    """(ncells,) number of open domain faces each cell touches"""
    st = (1 << (mesh.lmax - mesh.level))[:, None]
    l = np.arange(512)
    idx = np.stack([l & 7, (l >> 3) & 7, l >> 6], axis=1)
    n = np.zeros((mesh.nblocks, 512), np.int32)
    for d in range(3):
        if not mesh.open_axes[d]:
            continue
        lo = mesh.origin[:, d][:, None] + idx[None, :, d] * st
        n += (lo == 0) | (lo + st == mesh.nfine[d])
    return n.ravel()


# field boundary types: one for every open face, or one per face (-x, +x, -y,
# +y, -z, +z: cDomainBC's per-face policy)
CASES = [((3, 2, 2), 0, (True, False, False), 0),
         ((3, 2, 2), 0, (True, False, True), 1),
         ((4, 4, 4), 1, (True, True, False), 1),
         ((4, 4, 4), 1, (False, False, True), 0),
         ((3, 2, 2), 0, (True, False, True), (0, 1, 0, 0, 1, 0)),
         ((4, 4, 4), 1, (True, True, False), (1, 0, 0, 1, 0, 0))]


@pytest.mark.parametrize("nb0,lmax,open_axes,bc", CASES)
def test_open_field_solve_matches_oracle(nb0, lmax, open_axes, bc):
    mesh, wl, ic, x, f = open_case(nb0, lmax, open_axes, bc)
    assert mesh.bnd_flag.sum() > 0
    ao = oracle_for(mesh, wl, ic, x, f)
    with gpu_for(mesh, wl, ic, x, f) as ctx:
        ctx.UpdateJMassMatrix()
        J, M = ctx.export_cell_moments()
        st = ctx.TimeStep(tol=1e-11, maxit=600, precond=1)
        g = ctx.export_fields()
    assert st.converged
    ao.cellJ[:] = J.ravel()
    ao.cellM[:] = M.ravel()
    E0 = f["E_n"].copy()
    it, wave = ao.field_solve(tol=1e-11, maxit=800)
    assert it > 0
    for k, ref in (("E_n", ao.E_n), ("E_half", ao.E_half), ("B_center", ao.Bcen),
                   ("B_corner_prev", ao.Bprev), ("B_corner_cur", ao.Bcur)):
        assert rel_err(g[k], ref) < 1e-7, k
    assert st.wave_energy == pytest.approx(wave, rel=1e-9)
    # the boundary rows hold
    b = np.flatnonzero(mesh.bnd_flag)
    dE = g["E_half"] - E0
    if bc == 0:
        assert np.abs(dE[b]).max() <= 1e-12 * np.abs(dE).max()
        cells = boundary_cells(mesh) > 0
        np.testing.assert_array_equal(g["B_center"][cells], f["B_center"][cells])
    else:
        mean = np.zeros_like(dE[b])
        for r, c in enumerate(b):
            s, e = mesh.bnd_start[c], mesh.bnd_start[c + 1]
            mean[r] = (mesh.bnd_weight[s:e, None] * dE[mesh.bnd_col[s:e]]).sum(axis=0)
        assert np.abs(dE[b] - mean).max() <= 1e-9 * np.abs(dE).max()


@pytest.mark.parametrize("nb0,lmax,open_axes,bc", [CASES[1], CASES[2], CASES[5]])
def test_open_steps_match_oracle(open_oracle, nb0, lmax, open_axes, bc):
    """two full ECSIM steps with fast particles: the set deleted at the open
    faces, the surviving particles and the fields follow the oracle"""
    mesh, wl, ic, x, f = open_case(nb0, lmax, open_axes, bc, seed=83, vscale=40.0)
    open_oracle.orc_set_open_axes(sum(1 << d for d in range(3) if open_axes[d]))
    ao = oracle_for(mesh, wl, ic, x, f)
    ao.deposit()
    with gpu_for(mesh, wl, ic, x, f) as ctx:
        n0 = ctx.num_particles()
        for _ in range(2):
            s = ctx.PicTimeStep(tol=1e-12, maxit=600, precond=1)
            it, diag = ao.step(tol=1e-12, maxit=800)
            assert s.solve.converged and it > 0
        alive = ao.block >= 0
        assert (~alive).sum() > 50
        assert ctx.num_particles() == n0 - (~alive).sum()
        g = ctx.export_fields()
        cJ, cM = ctx.export_cell_moments()
    for k, ref in (("E_n", ao.E_n), ("B_center", ao.Bcen)):
        assert rel_err(g[k], ref) < 1e-5, k
    assert rel_err(cJ.reshape(-1), ao.cellJ) < 1e-5
    assert rel_err(cM.reshape(-1), ao.cellM) < 1e-5


def test_open_mesh_fixes_particle_open_axes():
    mesh, wl, ic, x, f = open_case((3, 2, 2), 0, (True, False, False), 0)
    with gpu_for(mesh, wl, ic, x, f) as ctx:
        ctx.set_open_axes(True, False, False)
        with pytest.raises(A.AmpsGpuError):
            ctx.set_open_axes(False, False, False)


def test_amr_injection_matches_oracle(open_oracle):
    """OpenFlow injection on a two-level mesh with open x: the same finest-patch
    streams on the device and in the oracle give the same injected particles
    (count, positions after the partial push, velocities)"""
    from tests.test_gpu_injection import match
    import ctypes as C
    from tests.oracle_amr import p as pa
    mesh, wl, ic, x, f = open_case((4, 4, 4), 1, (True, False, False), 1, seed=85)
    open_oracle.orc_set_open_axes(1)
    e, i = wl.species
    srcs = [(0, 0, 400.0 * e.weight, e.vth, (0.02, 0.0, 0.0)),
            (1, 1, 400.0 * i.weight, i.vth, (-0.004, 0.001, 0.0))]
    ao = oracle_for(mesh, wl, ic, x, f)
    with gpu_for(mesh, wl, ic, x, f) as ctx:
        ctx.set_injection_seed(91)
        for face, spec, dens, vth, drift in srcs:
            ctx.add_injection(face, spec, dens, vth, drift)
        n0 = ctx.num_particles()
        ctx.push_deposit()
        ao.push()
        xs, vs = [], []
        for s, (face, spec, dens, vth, drift) in enumerate(srcs):
            cap = 400000
            xo, vo = np.zeros((cap, 3)), np.zeros((cap, 3))
            blk, cel = np.zeros(cap, np.int32), np.zeros(cap, np.int32)
            k = ao.L.orc_amr_inject(C.byref(ao.g), face, spec, dens, pa(np.array(drift, np.float64)), vth, 91, 0,
                                    s, pa(ao.E_half), pa(ao.Bprev), cap, pa(xo), pa(vo), pa(blk, C.c_int32),
                                    pa(cel, C.c_int32))
            assert 50 < k <= cap
            xs.append(xo[:k]); vs.append(vo[:k])
        xi, vi = np.concatenate(xs), np.concatenate(vs)
        ninj = ctx.injected_particles()
        assert ninj == len(xi)
        alive = ao.block >= 0
        assert ctx.num_particles() == n0 - (~alive).sum() + ninj
        g = ctx.export_particles()
        order = np.argsort(g["id"])
        g = {k: v[order] for k, v in g.items()}
        new = g["id"] >= n0
        m = match(g["x"][new], xi)
        assert np.abs(g["x"][new] - xi[m]).max() <= 1e-5 * mesh.dx0
        assert np.abs(g["v"][new] - vi[m]).max() <= 2e-5 * np.abs(vi).max()
