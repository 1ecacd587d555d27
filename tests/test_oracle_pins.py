"""The FP64 oracle against the reference's own code and known answers (CPU only).

* operator taps vs the reference stencil algebra (golden stencil_taps.json)
* corner-pair slot table vs ProcessCell's IndexMatrix (golden index_matrix.json)
* gridless relativistic Boris vs the reference-compiled BorisStep (golden
  gridless_boris.json)
* ECSIM invariants the reference relies on: theta = 0.5 conserves total energy,
  the mass matrix is symmetric in the corner pair, GMRES meets its stop rule
"""
import json
import os

import numpy as np
import pytest

from tests import oracle_lib as O

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def slot(di, dj, dk):
    dig = lambda o: 0 if o == 0 else (1 if o < 0 else 2)
    return dig(di) + 3 * dig(dj) + 9 * dig(dk)


def table(name, *args):
    lib = O.load()
    out = np.zeros(27)
    getattr(lib, name)(*args, O.p(out))
    return out


def taps_to_table(taps):
    t = np.zeros(27)
    for i, j, k, a in taps:
        t[slot(i, j, k)] += a
    return t


def test_stencil_taps_match_reference_stencil_library():
    g = json.load(open(os.path.join(GOLD, "stencil_taps.json")))
    for ax, key in enumerate(("lap_x", "lap_y", "lap_z")):
        np.testing.assert_array_equal(table("orc_laplacian_table", ax), taps_to_table(g[key]))
        np.testing.assert_array_equal(table("orc_graddiv_table", ax, ax), taps_to_table(g[key]))
    for (p, q), key in {(0, 1): "gd_xy", (0, 2): "gd_xz", (1, 2): "gd_yz"}.items():
        ref = taps_to_table(g[key])
        np.testing.assert_array_equal(table("orc_graddiv_table", p, q), ref)
        np.testing.assert_array_equal(table("orc_graddiv_table", q, p), ref)


def test_stencils_are_consistent_second_derivatives():
    # applied to x^2 the Laplacian taps give 2, to x*y the mixed taps give 1
    for ax in range(3):
        lap = table("orc_laplacian_table", ax)
        s = 0.0
        for dk in (-1, 0, 1):
            for dj in (-1, 0, 1):
                for di in (-1, 0, 1):
                    s += lap[slot(di, dj, dk)] * (di, dj, dk)[ax] ** 2
        assert s == pytest.approx(2.0)
    gd = table("orc_graddiv_table", 0, 1)
    s = sum(gd[slot(di, dj, dk)] * di * dj for di in (-1, 0, 1) for dj in (-1, 0, 1)
            for dk in (-1, 0, 1))
    assert s == pytest.approx(1.0)


def test_corner_pair_slots_match_index_matrix():
    g = json.load(open(os.path.join(GOLD, "index_matrix.json")))["IndexMatrix"]
    off = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    for c1 in range(8):
        for c2 in range(8):
            d = [off[c2][a] - off[c1][a] for a in range(3)]
            assert slot(*d) == g[c1][c2]


def test_corner_weights_table_order():
    lib = O.load()
    xl = np.array([0.25, 0.5, 0.75])
    w = np.zeros(8)
    lib.orc_corner_weights(O.p(xl), O.p(w))
    off = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    for t, o in enumerate(off):
        e = np.prod([xl[a] if o[a] else 1 - xl[a] for a in range(3)])
        assert w[t] == pytest.approx(e, rel=1e-15)
    assert w.sum() == pytest.approx(1.0, rel=1e-15)


def test_gridless_boris_matches_reference_build():
    g = json.load(open(os.path.join(GOLD, "gridless_boris.json")))
    x, pm, st, steps, tot = O.trace(np.array(g["x0"]), np.array(g["p0"]), g["q"], g["m0"],
                                    g["b_eq"], g["r_e"], np.array(g["b_ext"]), g["r_in"],
                                    g["r_out"], g["max_steps"], g["dphi"], g["dt_max"])
    np.testing.assert_array_equal(st, np.array(g["status"]))
    np.testing.assert_array_equal(steps, np.array(g["steps"]))
    # same operations up to the dipole factorisation; rounding differences grow
    # over up to 3000 steps to a few 1e-9 relative
    gx, gp = np.array(g["x"]), np.array(g["p"])
    assert (np.linalg.norm(x - gx, axis=1) / np.linalg.norm(gx, axis=1)).max() < 1e-7
    assert (np.linalg.norm(pm - gp, axis=1) / np.linalg.norm(gp, axis=1)).max() < 1e-7


def small_state(nb=(1, 1, 1), ppc=4, seed=100, b0=(0.0, 0.0, 0.5), e_amp=0.0):
    import amps_gb300 as A
    wl = A.electron_proton_plasma("t", *nb, ppc, 3)
    wl.seed = seed
    ic = A.make_initial_condition(wl, nthreads=2)
    x = A.physical_positions(wl.mesh, ic["u"], ic["block"])
    f = A.initial_fields(wl)
    if e_amp:
        rng = np.random.default_rng(seed)
        for k in ("E_n", "E_half"):
            f[k] = e_amp * rng.standard_normal(f[k].shape)
    return wl, ic, x, f


def test_ecsim_energy_conserved_theta_half():
    wl, ic, x, f = small_state(nb=(1, 1, 1), ppc=8)
    st = O.OracleState(wl, x, ic["v"].astype(np.float64), ic["spec"], f)
    e0 = st.deposit()
    # wave energy of the initial state
    wave0 = np.sum(st.Bcen ** 2 + st.E_n ** 2) / (8 * np.pi) * wl.mesh.dx ** 3
    tot0 = e0 + wave0
    hist = []
    for _ in range(3):
        it, diag = st.step(tol=1e-12, maxit=400, precond=1)
        assert it > 0
        hist.append(diag[0] + diag[1])
    drift = np.abs(np.array(hist) - tot0) / tot0
    assert drift.max() < 1e-9, (tot0, hist)


def test_mass_matrix_pair_symmetry():
    # M_c[slot(d)] of corner c equals M_{c+d}[slot(-d)] (ProcessCell adds the same
    # 3x3 block to both corners of a pair)
    wl, ic, x, f = small_state(nb=(1, 1, 1), ppc=4)
    st = O.OracleState(wl, x, ic["v"].astype(np.float64), ic["spec"], f)
    st.deposit()
    M = st.M.reshape(8, 8, 8, 27, 9)  # [K][J][I][slot][ab]
    rng = np.random.default_rng(0)
    for _ in range(50):
        I, J, K = rng.integers(0, 8, 3)
        d = rng.integers(-1, 2, 3)
        a = M[K, J, I, slot(*d)]
        b = M[(K + d[2]) % 8, (J + d[1]) % 8, (I + d[0]) % 8, slot(*(-d))]
        np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-18)


def test_gmres_meets_stop_rule():
    wl, ic, x, f = small_state(nb=(1, 1, 1), ppc=4, e_amp=1e-3)
    st = O.OracleState(wl, x, ic["v"].astype(np.float64), ic["spec"], f)
    st.deposit()
    b = st.rhs().ravel().copy()
    for precond in (0, 1):
        xs = np.zeros_like(b)
        res = np.zeros(1)
        it = O.load().orc_gmres(O.C.byref(st.m), O.p(st.M), O.p(b), O.p(xs), 1e-10, 500, 30,
                                precond, O.p(res))
        assert it > 0
        r = b - st.matvec(xs.reshape(-1, 3)).ravel()
        assert np.linalg.norm(r) <= 1e-9 * np.linalg.norm(b)


# ---- ProcessCell and Lapenta2017 of the reference, compiled from its sources
# (golden ecsim_ref.json, oracle/pins/ecsim_pin.cpp): the oracle on the same
# particles, fields and plasma in a periodic 8^3-cell block (the reference runs
# in its default 5^3-cell block; the golden particles and their corners lie in
# cells 0..4, where the two blocks coincide).
CORNER_OFF = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]


def ref_golden():
    return json.load(open(os.path.join(GOLD, "ecsim_ref.json")))


def ref_mesh(g, species):
    m = O.Mesh()
    m.nbx = m.nby = m.nbz = 1
    for d in range(3):
        m.x0[d] = 0.0
        m.dx[d] = g["dx"]
    m.nspec = 1
    m.q[0], m.m[0], m.w[0] = g["charge"][species], g["mass"][species], g["weight"]
    m.dt, m.theta = g["dt"], 0.5
    return m


def ref_fields(g):
    """E^{n+theta} and B on the 8^3 block's corners from the golden corner values"""
    n1 = g["block_cells"] + 1
    E, B = np.zeros((512, 3)), np.zeros((512, 3))
    cf = np.array(g["corner_fields"])
    for t in range(len(cf)):
        i, j, k = t % n1, (t // n1) % n1, t // (n1 * n1)
        E[i + 8 * (j + 8 * k)] = cf[t, :3]
        B[i + 8 * (j + 8 * k)] = cf[t, 3:]
    return E, B


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / np.max(np.abs(b)))


def test_process_cell_matches_reference_build():
    g = ref_golden()
    lib = O.load()
    _, Bc = ref_fields(g)
    for rec in g["process_cell"]:
        m = ref_mesh(g, rec["species"])
        ps = rec["particles"]
        n = len(ps)
        x = np.ascontiguousarray([p["x"] for p in ps], np.float64)
        v = np.ascontiguousarray([p["v"] for p in ps], np.float64)
        wc = np.ascontiguousarray([p["wcorr"] for p in ps], np.float64)
        sp = np.zeros(n, np.uint8)
        blk, cel = np.zeros(n, np.int32), np.zeros(n, np.int32)
        lib.orc_locate(O.C.byref(m), n, O.p(x), O.p(blk, O.C.c_int32), O.p(cel, O.C.c_int32))
        ci, cj, ck = rec["cell"]
        assert np.all(cel == ci + 8 * (cj + 8 * ck))
        J, M = np.zeros((512, 3)), np.zeros((512, 243))
        e = lib.orc_deposit(O.C.byref(m), n, O.p(x), O.p(v), O.p(sp, O.C.c_uint8), O.p(wc),
                            O.p(blk, O.C.c_int32), O.p(cel, O.C.c_int32), O.p(Bc), O.p(J), O.p(M))
        cor = [(ci + o[0]) + 8 * ((cj + o[1]) + 8 * (ck + o[2])) for o in CORNER_OFF]
        gJ = np.array(rec["J"]).reshape(8, 3)
        gM = np.array(rec["M"]).reshape(8, 243)
        assert rel(J[cor], gJ) < 1e-13, rel(J[cor], gJ)
        assert rel(M[cor], gM) < 1e-13, rel(M[cor], gM)
        # nothing else was deposited
        others = np.setdiff1d(np.arange(512), cor)
        assert not J[others].any() and not M[others].any()
        assert e == pytest.approx(rec["energy"], rel=1e-13)
        cfl = np.zeros(1)
        lib.orc_cfl(O.C.byref(m), n, O.p(v), O.p(sp, O.C.c_uint8), O.p(blk, O.C.c_int32),
                    O.p(cel, O.C.c_int32), O.p(cfl))
        assert cfl[0] == pytest.approx(rec["cfl"], rel=1e-13)


def test_lapenta2017_matches_reference_build():
    g = ref_golden()
    lib = O.load()
    E, B = ref_fields(g)
    for species in (0, 1):
        recs = [r for r in g["lapenta"] if r["species"] == species]
        m = ref_mesh(g, species)
        n = len(recs)
        x = np.ascontiguousarray([r["in"]["x"] for r in recs], np.float64)
        v = np.ascontiguousarray([r["in"]["v"] for r in recs], np.float64)
        sp = np.zeros(n, np.uint8)
        blk, cel = np.zeros(n, np.int32), np.zeros(n, np.int32)
        lib.orc_locate(O.C.byref(m), n, O.p(x), O.p(blk, O.C.c_int32), O.p(cel, O.C.c_int32))
        out = lib.orc_push(O.C.byref(m), n, O.p(x), O.p(v), O.p(sp, O.C.c_uint8),
                           O.p(blk, O.C.c_int32), O.p(cel, O.C.c_int32), O.p(E), O.p(B))
        assert out == 0
        gx = np.array([r["x"] for r in recs])
        gv = np.array([r["v"] for r in recs])
        assert np.max(np.abs(x - gx)) < 1e-13 * g["dx"], np.max(np.abs(x - gx))
        assert rel(v, gv) < 1e-13, rel(v, gv)
        assert all(r["code"] == 3 for r in recs)   # _PARTICLE_MOTION_FINISHED_
        gc = np.array([r["cell"][0] + 8 * (r["cell"][1] + 8 * r["cell"][2]) for r in recs])
        np.testing.assert_array_equal(cel, gc)


def test_boris_matches_reference_build():
    g = ref_golden()
    lib = O.load()
    E, B = ref_fields(g)
    for species in (0, 1):
        recs = [r for r in g["boris"] if r["species"] == species]
        m = ref_mesh(g, species)
        n = len(recs)
        x = np.ascontiguousarray([r["in"]["x"] for r in recs], np.float64)
        v = np.ascontiguousarray([r["in"]["v"] for r in recs], np.float64)
        sp = np.zeros(n, np.uint8)
        blk, cel = np.zeros(n, np.int32), np.zeros(n, np.int32)
        lib.orc_locate(O.C.byref(m), n, O.p(x), O.p(blk, O.C.c_int32), O.p(cel, O.C.c_int32))
        ndel = lib.orc_boris(O.C.byref(m), n, O.p(x), O.p(v), O.p(sp, O.C.c_uint8),
                             O.p(blk, O.C.c_int32), O.p(cel, O.C.c_int32), O.p(E), O.p(B),
                             recs[0]["dt"])
        assert ndel == 0
        gx = np.array([r["x"] for r in recs])
        gv = np.array([r["v"] for r in recs])
        assert np.max(np.abs(x - gx)) < 1e-13 * g["dx"], np.max(np.abs(x - gx))
        assert rel(v, gv) < 1e-13, rel(v, gv)
        assert all(r["code"] == 3 for r in recs)   # _PARTICLE_MOTION_FINISHED_
        gc = np.array([r["cell"][0] + 8 * (r["cell"][1] + 8 * r["cell"][2]) for r in recs])
        np.testing.assert_array_equal(cel, gc)


# ---- the same routines configured with the magnetic field on the cell centres
# (the reference's default, golden ecsim_ref_cb.json, oracle/_ref/ecsim_pin_cb):
# ProcessCell and Lapenta2017 read B from the centres with CellCentered::
# Linear's stencil (pic_interpolation_routines.cpp:820-905)
def ref_golden_cb():
    return json.load(open(os.path.join(GOLD, "ecsim_ref_cb.json")))


def ref_center_b(g):
    """B on the 8^3 block's cells from the golden centre values of cells 0..4"""
    n = g["block_cells"]
    B = np.zeros((512, 3))
    cf = np.array(g["center_fields"])
    for t in range(len(cf)):
        i, j, k = t % n, (t // n) % n, t // (n * n)
        B[i + 8 * (j + 8 * k)] = cf[t]
    return B


def test_process_cell_center_b_matches_reference_build():
    g = ref_golden_cb()
    assert g["b_mode"] == "center"
    lib = O.load()
    Bc = ref_center_b(g)
    lib.orc_set_b_center(1)
    try:
        for rec in g["process_cell"]:
            m = ref_mesh(g, rec["species"])
            ps = rec["particles"]
            n = len(ps)
            x = np.ascontiguousarray([p["x"] for p in ps], np.float64)
            v = np.ascontiguousarray([p["v"] for p in ps], np.float64)
            wc = np.ascontiguousarray([p["wcorr"] for p in ps], np.float64)
            sp = np.zeros(n, np.uint8)
            blk, cel = np.zeros(n, np.int32), np.zeros(n, np.int32)
            lib.orc_locate(O.C.byref(m), n, O.p(x), O.p(blk, O.C.c_int32), O.p(cel, O.C.c_int32))
            ci, cj, ck = rec["cell"]
            J, M = np.zeros((512, 3)), np.zeros((512, 243))
            e = lib.orc_deposit(O.C.byref(m), n, O.p(x), O.p(v), O.p(sp, O.C.c_uint8), O.p(wc),
                                O.p(blk, O.C.c_int32), O.p(cel, O.C.c_int32), O.p(Bc), O.p(J), O.p(M))
            cor = [(ci + o[0]) + 8 * ((cj + o[1]) + 8 * (ck + o[2])) for o in CORNER_OFF]
            assert rel(J[cor], np.array(rec["J"]).reshape(8, 3)) < 1e-13
            assert rel(M[cor], np.array(rec["M"]).reshape(8, 243)) < 1e-13
            assert e == pytest.approx(rec["energy"], rel=1e-13)
    finally:
        lib.orc_set_b_center(0)


def test_lapenta2017_center_b_matches_reference_build():
    g = ref_golden_cb()
    lib = O.load()
    E, _ = ref_fields(g)
    Bc = ref_center_b(g)
    lib.orc_set_b_center(1)
    try:
        for species in (0, 1):
            recs = [r for r in g["lapenta"] if r["species"] == species]
            m = ref_mesh(g, species)
            n = len(recs)
            x = np.ascontiguousarray([r["in"]["x"] for r in recs], np.float64)
            v = np.ascontiguousarray([r["in"]["v"] for r in recs], np.float64)
            sp = np.zeros(n, np.uint8)
            blk, cel = np.zeros(n, np.int32), np.zeros(n, np.int32)
            lib.orc_locate(O.C.byref(m), n, O.p(x), O.p(blk, O.C.c_int32), O.p(cel, O.C.c_int32))
            assert lib.orc_push(O.C.byref(m), n, O.p(x), O.p(v), O.p(sp, O.C.c_uint8),
                                O.p(blk, O.C.c_int32), O.p(cel, O.C.c_int32), O.p(E), O.p(Bc)) == 0
            assert np.max(np.abs(x - np.array([r["x"] for r in recs]))) < 1e-13 * g["dx"]
            assert rel(v, np.array([r["v"] for r in recs])) < 1e-13
    finally:
        lib.orc_set_b_center(0)


def test_oracle_centre_b_stencil_exact_for_linear_fields():
    """CellCentered::Linear's trilinear stencil over cell centres reproduces a
    field linear in position wherever the stencil does not wrap (points at
    least 1.5 cells from the domain faces, across block boundaries too), and a
    constant field everywhere, the periodic wrap included (its weights sum to 1)"""
    import amps_gb300 as A
    wl = A.electron_proton_plasma("centre-b", 2, 2, 2, 1, 3)
    lib = O.load()
    m = O.mesh_of(wl)
    shp = wl.mesh.shape  # cells per axis
    dx, x0 = wl.mesh.dx, np.array(wl.mesh.x0, float)
    I, J, K = np.meshgrid(np.arange(shp[0]), np.arange(shp[1]), np.arange(shp[2]), indexing="ij")
    # cell-centre coordinates in the oracle's order I + NX (J + NY K)
    xc = np.stack([(I.ravel(order="F") + 0.5), (J.ravel(order="F") + 0.5),
                   (K.ravel(order="F") + 0.5)], axis=1) * dx + x0
    rng = np.random.default_rng(7)
    a = rng.standard_normal(3)
    G = rng.standard_normal((3, 3))
    Bc = np.ascontiguousarray(a + xc @ G.T)
    L = np.array(shp, float) * dx
    n = 4000
    x = x0 + 1.5 * dx + rng.random((n, 3)) * (L - 3.0 * dx)
    x = np.ascontiguousarray(x)
    block = np.zeros(n, np.int32)
    cell = np.zeros(n, np.int32)
    lib.orc_locate(O.C.byref(m), n, O.p(x), O.p(block, O.C.c_int32), O.p(cell, O.C.c_int32))
    B = np.zeros((n, 3))
    lib.orc_centre_b_at(O.C.byref(m), n, O.p(x), O.p(block, O.C.c_int32), O.p(Bc), O.p(B))
    np.testing.assert_allclose(B, a + x @ G.T, rtol=0, atol=1e-12 * np.abs(Bc).max())
    # a constant field, points anywhere (stencils that wrap the periodic faces)
    xa = np.ascontiguousarray(x0 + rng.random((n, 3)) * L)
    lib.orc_locate(O.C.byref(m), n, O.p(xa), O.p(block, O.C.c_int32), O.p(cell, O.C.c_int32))
    Bk = np.ascontiguousarray(np.broadcast_to(a, Bc.shape))
    lib.orc_centre_b_at(O.C.byref(m), n, O.p(xa), O.p(block, O.C.c_int32), O.p(Bk), O.p(B))
    np.testing.assert_allclose(B, np.broadcast_to(a, B.shape), rtol=0, atol=1e-14)
