"""AMR mesh builder and the cell-assembled ECSIM operator (CPU only).

* builder invariants: coverage, hanging-corner constraints (weights sum to 1,
  parents free), 2:1 balance rejected when violated;
* on a single-level mesh the cell-assembled operator and RHS of the AMR oracle
  equal the uniform oracle's (itself pinned to the reference stencil taps)
  times the cell volume -- so the AMR extension reduces to the reference;
* on a two-level mesh with hanging corners the ECSIM step conserves total
  energy (theta = 0.5), the property the reference's discretisation is built on.
"""
import numpy as np
import pytest

import amps_gb300 as A
from amps_gb300 import amr
from tests import oracle_amr as OA
from tests import oracle_lib as O


def test_uniform_mesh_has_no_hanging_corners():
    m = amr.uniform_mesh((2, 1, 2))
    assert m.nblocks == 4 and m.ncorners == m.ncells and m.nhanging == 0
    assert (m.fine_map >= 0).all()


def test_central_refined_mesh_tables():
    m = amr.central_refined_mesh((4, 4, 4), lmax=1, frac=0.5)
    assert m.nblocks == 56 + 64
    assert m.nhanging > 0
    vol = np.sum((8 * m.block_dx()) ** 3)
    assert vol == pytest.approx(32.0 ** 3)
    hs = m.hang_start
    for c in np.flatnonzero(hs[1:] > hs[:-1]):
        w = m.hang_weight[hs[c]:hs[c + 1]]
        par = m.hang_parent[hs[c]:hs[c + 1]]
        assert w.sum() == pytest.approx(1.0)
        assert np.all(hs[par + 1] == hs[par])          # parents are free corners
        # the hanging corner is the weighted mean of its parents' positions
        xyz = m.corner_xyz.reshape(-1, 3).astype(float)
        mid = (w[:, None] * xyz[par]).sum(0)
        d = np.abs(mid - xyz[c])
        d = np.minimum(d, np.array(m.nfine) - d)
        assert d.max() < 1e-9
    # config 2 mesh: 448 coarse + 512 fine blocks
    m2 = amr.central_refined_mesh((8, 8, 8), lmax=1, frac=0.5)
    assert m2.nblocks == 960 and np.sum(m2.level == 1) == 512


def test_unbalanced_mesh_rejected():
    # a level-2 block next to a level-0 block violates 2:1 balance
    leaves = [(2, 0, 0, 0)]
    leaves += [(2, x, y, z) for z in (0, 8) for y in (0, 8) for x in (0, 8) if (x, y, z) != (0, 0, 0)]
    leaves += [(1, x, y, z) for z in (0, 16) for y in (0, 16) for x in (0, 16) if (x, y, z) != (0, 0, 0)]
    leaves += [(0, 32, 0, 0)]  # level-0 neighbour of the level-1 block is fine, of level-2 is not
    with pytest.raises(A.AmpsGpuError):
        amr.AmrMesh((2, 1, 1), 2, np.array(leaves, np.int32)).close()


def uniform_pair(nb, ppc=4, seed=5):
    wl = A.electron_proton_plasma("t", *nb, ppc, 2)
    wl.seed = seed
    ic = A.make_initial_condition(wl, nthreads=2)
    x = A.physical_positions(wl.mesh, ic["u"], ic["block"])
    v = ic["v"].astype(np.float64)
    rng = np.random.default_rng(seed)
    f = A.initial_fields(wl)
    for k in ("B_corner_cur", "B_corner_prev", "B_center"):
        f[k] = f[k] + 0.05 * rng.standard_normal(f[k].shape)
    st = O.OracleState(wl, x, v, ic["spec"], f)
    st.deposit()
    m = amr.uniform_mesh(nb)
    ao = OA.AmrOracle(m, wl.species, wl.dt, wl.theta, x, v, ic["spec"])
    xyz = m.corner_xyz.reshape(-1, 3)
    NX, NY, _ = wl.mesh.shape
    gidx = xyz[:, 0] + NX * (xyz[:, 1] + NY * xyz[:, 2])   # AMR corner -> uniform corner
    ao.Bcur[:] = f["B_corner_cur"][gidx]
    # cells: both use block*512 + local numbering
    ao.Bcen[:] = f["B_center"][cell_map(wl)]
    ao.deposit()
    return wl, st, ao, gidx, rng


def cell_map(wl):
    """uniform global cell index of every AMR cell (block*512 + local)"""
    nb = wl.mesh.nblocks
    b = np.repeat(np.arange(nb), 512)
    l = np.tile(np.arange(512), nb)
    bx = b % wl.mesh.nbx; by = (b // wl.mesh.nbx) % wl.mesh.nby; bz = b // (wl.mesh.nbx * wl.mesh.nby)
    I = bx * 8 + (l & 7); J = by * 8 + ((l >> 3) & 7); K = bz * 8 + (l >> 6)
    NX, NY, _ = wl.mesh.shape
    return I + NX * (J + NY * K)


def test_amr_operator_equals_uniform_reference_operator():
    wl, st, ao, gidx, rng = uniform_pair((1, 2, 1))
    x_u = rng.standard_normal((wl.mesh.ncells, 3))
    y_u = st.matvec(x_u)
    y_a = ao.apply(x_u[gidx])
    V = wl.mesh.dx ** 3
    np.testing.assert_allclose(y_a, V * y_u[gidx], rtol=1e-11, atol=1e-13)


def test_amr_rhs_equals_uniform_reference_rhs():
    wl, st, ao, gidx, rng = uniform_pair((2, 1, 1))
    st.E_n[:] = 1e-2 * rng.standard_normal(st.E_n.shape)
    ao.E_n[:] = st.E_n[gidx]
    st.Bcen[:] = ao.Bcen[np.argsort(cell_map(wl))]
    r_u = st.rhs()
    r_a = np.zeros_like(ao.E_n)
    OA.lib().orc_amr_rhs(OA.C.byref(ao.g), OA.p(ao.E_n), OA.p(ao.Bcen), OA.p(ao.cellJ),
                         OA.p(ao.cellM), OA.p(r_a))
    np.testing.assert_allclose(r_a, wl.mesh.dx ** 3 * r_u[gidx], rtol=1e-10, atol=1e-14)


def test_amr_energy_conserved_two_levels():
    m = amr.central_refined_mesh((4, 4, 4), lmax=1, frac=0.5)
    wl = A.electron_proton_plasma("amr", 1, 1, 1, 8, 3)
    ic = amr.amr_initial_condition(m, wl.species, 8, seed=3)
    x = m.block_origins()[ic["block"]] + ic["u"].astype(np.float64) * m.block_dx()[ic["block"]][:, None]
    ao = OA.AmrOracle(m, wl.species, wl.dt, wl.theta, x, ic["v"].astype(np.float64), ic["spec"])
    np.testing.assert_array_equal(ao.block, ic["block"])
    ao.Bcen[:] = np.array(wl.b0)
    ao.c2n()
    e0 = ao.deposit()
    tot0 = e0 + ao.wave_energy()
    for _ in range(3):
        it, diag = ao.step(tol=1e-12, maxit=600)
        assert it > 0
        drift = abs(diag[0] + diag[1] - tot0) / tot0
        assert drift < 1e-8, drift


@pytest.mark.parametrize("recipe", ["box2", "sphere3"])
def test_every_free_corner_is_one_cells_low_corner(recipe):
    """The learned preconditioner writes each free (non-hanging) corner from the
    block whose cell has it as low corner: on nested meshes that cell exists
    and is unique for every free corner."""
    if recipe == "box2":
        m = amr.central_refined_mesh((4, 4, 4), lmax=1, frac=0.5)
    else:
        m = amr.sphere_refined_mesh((4, 4, 4), lmax=2, radius=0.2)
    tab = m.corner_tab.reshape(m.nblocks, 9, 9, 9)      # [b][k][j][i]
    low = tab[:, :8, :8, :8].reshape(-1)
    hanging = m.hang_start[1:] > m.hang_start[:-1]
    count = np.bincount(low[~hanging[low]], minlength=m.ncorners)
    free = ~hanging
    assert np.all(count[free] == 1), (np.sum(count[free] == 0), np.sum(count[free] > 1))


def test_open_axis_mesh_boundary_rows():
    """open axes: corners 0..nfine on those axes, the free corners on their
    domain faces are boundary rows (Dirichlet: no donors; Neumann: one inward
    donor per touching face, weights summing to 1)"""
    from amps_gb300 import amr as AM
    leaves = [(0, i * 8, j * 8, k * 8) for k in range(2) for j in range(2) for i in range(3)]
    per = AM.AmrMesh((3, 2, 2), 0, leaves)
    assert per.ncorners == 24 * 16 * 16 and per.bnd_flag.sum() == 0
    for bc in (0, 1):
        m = AM.AmrMesh((3, 2, 2), 0, leaves, open_axes=(True, False, True), field_bc=bc)
        assert m.ncorners == 25 * 16 * 17
        xyz = m.corner_xyz.reshape(-1, 3)
        on = (xyz[:, 0] == 0) | (xyz[:, 0] == 24) | (xyz[:, 2] == 0) | (xyz[:, 2] == 16)
        np.testing.assert_array_equal(m.bnd_flag.astype(bool), on)
        nent = np.diff(m.bnd_start)
        if bc == 0:
            assert nent.sum() == 0
            continue
        for c in np.flatnonzero(on):
            s, e = m.bnd_start[c], m.bnd_start[c + 1]
            faces = int(xyz[c, 0] in (0, 24)) + int(xyz[c, 2] in (0, 16))
            assert e - s == faces and abs(m.bnd_weight[s:e].sum() - 1.0) < 1e-15
            for q in m.bnd_col[s:e]:
                assert np.abs(xyz[q] - xyz[c]).sum() == 1   # one lattice step inward
    # two levels: hanging donors expand to their parents, the rows stay normalised
    base = AM.central_refined_mesh((4, 4, 4), lmax=1, frac=0.5)
    m2 = AM.AmrMesh((4, 4, 4), 1, base.leaves, open_axes=(True, True, False), field_bc=1)
    assert m2.nhanging == base.nhanging
    rows = np.flatnonzero(m2.bnd_flag)
    sums = np.add.reduceat(m2.bnd_weight, m2.bnd_start[rows]) if len(rows) else []
    assert np.allclose(sums, 1.0)


def test_per_face_boundary_rows():
    """one field boundary type per face (-x D, +x N, -z N, +z D on open x and z):
    a corner on a Neumann face has donors (one per open face it touches, also
    the Dirichlet ones), a corner only on Dirichlet faces has none"""
    from amps_gb300 import amr as AM
    leaves = [(0, i * 8, j * 8, k * 8) for k in range(2) for j in range(2) for i in range(3)]
    m = AM.AmrMesh((3, 2, 2), 0, leaves, open_axes=(True, False, True), field_bc=(0, 1, 0, 0, 1, 0))
    assert m.neumann_mask == (1 << 1) | (1 << 4)
    xyz = m.corner_xyz.reshape(-1, 3)
    xm, xp, zm, zp = xyz[:, 0] == 0, xyz[:, 0] == 24, xyz[:, 2] == 0, xyz[:, 2] == 16
    np.testing.assert_array_equal(m.bnd_flag.astype(bool), xm | xp | zm | zp)
    nent = np.diff(m.bnd_start)
    neumann = xp | zm
    faces = (xm | xp).astype(int) + (zm | zp).astype(int)
    np.testing.assert_array_equal(nent[neumann], faces[neumann])
    assert (nent[~neumann] == 0).all()
    # the all-Dirichlet and all-Neumann masks of the single-type call
    assert AM.AmrMesh((3, 2, 2), 0, leaves, open_axes=(True, False, True), field_bc=0).neumann_mask == 0
    assert AM.AmrMesh((3, 2, 2), 0, leaves, open_axes=(True, False, True),
                      field_bc=1).neumann_mask == 0b110011


def test_oracle_per_face_update_b():
    """UpdateB's boundary branch with per-face types: cells on a Neumann face
    average their inward neighbours (over every open face they touch), cells
    only on Dirichlet faces keep B^n"""
    import ctypes as C
    from amps_gb300 import amr as AM
    from tests import oracle_amr as OA
    from tests.oracle_amr import AmrOracle
    import amps_gb300 as A
    leaves = [(0, i * 8, j * 8, k * 8) for k in range(2) for j in range(2) for i in range(2)]
    wl = A.electron_proton_plasma("o", 1, 1, 1, 2, 2)
    m = AM.AmrMesh((2, 2, 2), 0, leaves, open_axes=(True, True, False), field_bc=(1, 0, 0, 1, 0, 0))
    ao = AmrOracle(m, wl.species, wl.dt, wl.theta, np.zeros((0, 3)), np.zeros((0, 3)),
                   np.zeros(0, np.uint8))
    rng = np.random.default_rng(2)
    ao.E_half[:] = 1e-2 * rng.standard_normal(ao.E_half.shape)
    ao.Bcen[:] = rng.standard_normal(ao.Bcen.shape)
    Bn = ao.Bcen.copy()
    B1 = np.zeros_like(Bn)
    ao.L.orc_amr_update_b(C.byref(ao.g), OA.p(ao.E_half), OA.p(Bn), OA.p(B1))
    org = m.origin
    cells = np.arange(m.nblocks * 512)
    b, l = cells // 512, cells % 512
    ijk = np.stack([l % 8, (l // 8) % 8, l // 64], 1) + org[b]
    side = np.zeros((len(cells), 3), int)
    for d in range(2):
        side[ijk[:, d] == 0, d] = -1
        side[ijk[:, d] == 15, d] = 1
    neu = (side[:, 0] == -1) | (side[:, 1] == 1)
    dir_only = (side != 0).any(1) & ~neu
    np.testing.assert_array_equal(B1[dir_only], Bn[dir_only])
    for c in np.flatnonzero(neu)[:40]:
        donors = []
        for d in range(2):
            if side[c, d]:
                j = ijk[c].copy()
                j[d] -= side[c, d]
                donors.append(np.flatnonzero((ijk == j).all(1))[0])
        np.testing.assert_allclose(B1[c], B1[donors].mean(0), rtol=0, atol=1e-14)


def test_oracle_open_boundary_rows_and_update_b():
    """the oracle's operator rows and UpdateB boundary branch on an open mesh"""
    from amps_gb300 import amr as AM
    from tests.oracle_amr import AmrOracle
    import amps_gb300 as A
    leaves = [(0, i * 8, j * 8, k * 8) for k in range(2) for j in range(2) for i in range(2)]
    wl = A.electron_proton_plasma("o", 1, 1, 1, 2, 2)
    for bc in (0, 1):
        m = AM.AmrMesh((2, 2, 2), 0, leaves, open_axes=(False, True, False), field_bc=bc)
        x = np.zeros((0, 3))
        ao = AmrOracle(m, wl.species, wl.dt, wl.theta, x, np.zeros((0, 3)), np.zeros(0, np.uint8))
        rng = np.random.default_rng(bc)
        v = rng.standard_normal((m.ncorners, 3))
        y = ao.apply(v)
        for c in np.flatnonzero(m.bnd_flag)[:50]:
            s, e = m.bnd_start[c], m.bnd_start[c + 1]
            want = v[c] - (m.bnd_weight[s:e, None] * v[m.bnd_col[s:e]]).sum(axis=0)
            np.testing.assert_allclose(y[c], want, rtol=0, atol=1e-15)
        ao.Bcen[:] = rng.standard_normal(ao.Bcen.shape)
        ao.E_half[:] = 1e-3 * rng.standard_normal(ao.E_half.shape)
        import ctypes as C
        from tests.oracle_amr import p
        bnew = np.zeros_like(ao.Bcen)
        ao.L.orc_amr_update_b(C.byref(ao.g), p(ao.E_half), p(ao.Bcen), p(bnew))
        # cells with j = 0 in the blocks at y = 0 (first layer)
        l = np.arange(m.ncells) % 512
        blk = np.arange(m.ncells) // 512
        jy = (l >> 3) & 7
        at0 = (m.origin[blk, 1] == 0) & (jy == 0)
        if bc == 0:
            np.testing.assert_array_equal(bnew[at0], ao.Bcen[at0])
        else:
            inward = np.flatnonzero(at0) + 8                   # j + 1, same block
            np.testing.assert_allclose(bnew[at0], bnew[inward], rtol=0, atol=0)


def test_amr_relboris_equals_uniform_relboris():
    """the AMR restatement of Mover::Relativistic::Boris on a single-level mesh
    takes the uniform-mesh restatement's sub-steps, positions and velocities"""
    wl, st, ao, gidx, rng = uniform_pair((2, 1, 1), ppc=2, seed=9)
    st.E_n[:] = 2e-2 * rng.standard_normal(st.E_n.shape)
    ao.E_n[:] = st.E_n[gidx]
    v = st.v * 6.0
    sp = np.linalg.norm(v, axis=1)
    v = np.where(sp[:, None] >= 0.95, v * (0.95 / sp)[:, None], v)
    st.v[:] = v
    ao.v[:] = v
    n_u = st.relboris(30.0, 1.0)
    n_a = ao.relboris(30.0, 1.0)
    assert n_a == n_u and n_a > len(v)
    L = np.array(wl.mesh.shape, float) * wl.mesh.dx
    d = ao.x - st.x
    d -= L * np.rint(d / L)
    assert np.abs(d).max() < 1e-9 * wl.mesh.dx
    np.testing.assert_allclose(ao.v, st.v, rtol=0, atol=1e-10)


def test_threaded_push_deposit_equals_serial():
    """the threaded oracle step of the CPU reference arm (push over particle
    ranges, deposit over block ranges) gives the serial restatement's
    particles and per-cell blocks exactly, the energy to its summation order"""
    mesh = amr.central_refined_mesh((4, 4, 4), lmax=1, frac=0.5)
    wl = A.electron_proton_plasma("mt", 1, 1, 1, 4, 2)
    ic = amr.amr_initial_condition(mesh, wl.species, 4, seed=23)
    x = mesh.block_origins()[ic["block"]] + ic["u"].astype(np.float64) * mesh.block_dx()[ic["block"]][:, None]
    f = amr.amr_initial_fields(mesh, wl.b0)
    states = []
    for _ in range(3):
        ao = OA.AmrOracle(mesh, wl.species, wl.dt, wl.theta, x, ic["v"].astype(np.float64) * 5.0,
                          ic["spec"])
        ao.E_half[:] = 1e-2 * np.cos(np.arange(ao.E_half.size)).reshape(ao.E_half.shape)
        ao.Bprev[:] = f["B_corner_prev"]
        ao.Bcur[:] = f["B_corner_cur"]
        states.append(ao)
    a, b, c = states
    a.push()
    ea = a.deposit()
    eb = b.push_deposit_mt(5)
    np.testing.assert_array_equal(a.x, b.x)
    np.testing.assert_array_equal(a.v, b.v)
    np.testing.assert_array_equal(a.block, b.block)
    np.testing.assert_array_equal(a.cellJ, b.cellJ)
    np.testing.assert_array_equal(a.cellM, b.cellM)
    assert eb == pytest.approx(ea, rel=1e-13)
    assert (a.block != mesh.nblocks).all() and len(np.unique(a.block)) > 10
    # a block selection (the reference arm's bounded sample): the selected
    # blocks' partials as above, the others untouched
    sel = (np.arange(mesh.nblocks) % 3 == 0).astype(np.uint8)
    c.cellJ[:] = 7.0
    c.cellM[:] = 7.0
    c.push_deposit_mt(4, sel)
    np.testing.assert_array_equal(c.x, a.x)
    cj, cm = c.cellJ.reshape(mesh.nblocks, -1), c.cellM.reshape(mesh.nblocks, -1)
    aj, am = a.cellJ.reshape(mesh.nblocks, -1), a.cellM.reshape(mesh.nblocks, -1)
    on = sel.astype(bool)
    np.testing.assert_array_equal(cj[on], aj[on])
    np.testing.assert_array_equal(cm[on], am[on])
    assert (cj[~on] == 7.0).all() and (cm[~on] == 7.0).all()
