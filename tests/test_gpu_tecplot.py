"""Tecplot output of the corner fields (amps_gpu_write_tecplot) in the layout
of the reference's mesh writer (src/meshAMR/meshAMRgeneric.h:7685-7710,
:8845): the file is parsed back and checked -- header, zone sizes, every
brick an axis-aligned cell of the mesh's cell size, node values equal to the
exported corner fields at the node's position (to the "%e" print precision,
6 significant digits)."""
import numpy as np
import pytest

import amps_gb300 as A
from amps_gb300 import amr
from tests import gpu_cases as G
from tests.test_gpu_amr import amr_case, gpu_for

pytestmark = pytest.mark.gpu


def parse(path):
    with open(path) as f:
        head = f.readline()
        zone = f.readline()
        assert zone.startswith("ZONE ")
        parts = dict(t.split("=") for t in zone[len("ZONE "):].replace(" ", "").strip().split(","))
        n, e = int(parts["N"]), int(parts["E"])
        nodes = np.array([[float(t) for t in f.readline().split()] for _ in range(n)])
        conn = np.array([[int(t) for t in f.readline().split()] for _ in range(e)]) - 1
    return head, parts, nodes, conn


def check_bricks(nodes, conn, dx_of_cell):
    p = nodes[:, :3][conn]                        # (E, 8, 3)
    d = p - p[:, :1]
    off = np.array([(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1),
                    (0, 1, 1)], float)
    np.testing.assert_allclose(d, off[None] * dx_of_cell[:, None, None], rtol=1e-5, atol=1e-9)


def test_tecplot_uniform(tmp_path):
    wl, ic, x, f = G.make_case(nb=(2, 1, 1), ppc=2)
    ctx = G.gpu_ctx(wl, ic, x, f)
    try:
        path = tmp_path / "fields.dat"
        ctx.write_tecplot(path)
        out = ctx.export_fields()
    finally:
        ctx.close()
    head, zone, nodes, conn = parse(path)
    assert head.startswith('VARIABLES="X", "Y", "Z","Ex (corner node)"')
    assert zone["DATAPACKING"] == "POINT" and zone["ZONETYPE"] == "FEBRICK"
    NX, NY, NZ = wl.mesh.shape
    assert len(nodes) == (NX + 1) * (NY + 1) * (NZ + 1) and len(conn) == NX * NY * NZ
    check_bricks(nodes, conn, np.full(len(conn), wl.mesh.dx))
    # values: the corner a node wraps to (global index I + NX (J + NY K))
    ijk = np.rint(nodes[:, :3] / wl.mesh.dx).astype(int)
    g = (ijk[:, 0] % NX) + NX * ((ijk[:, 1] % NY) + NY * (ijk[:, 2] % NZ))
    for k, col in (("E_n", 3), ("B_corner_cur", 6), ("E_half", 9)):
        np.testing.assert_allclose(nodes[:, col:col + 3], out[k][g], rtol=1e-5,
                                   atol=1e-5 * np.abs(out[k]).max())


def test_tecplot_amr(tmp_path):
    mesh, wl, ic, x, f = amr_case(ppc=2, seed=13)
    with gpu_for(mesh, wl, ic, x, f) as ctx:
        ctx.UpdateJMassMatrix()
        ctx.PicTimeStep(tol=1e-8, maxit=200, precond=1)
        path = tmp_path / "amr.dat"
        ctx.write_tecplot(path)
        out = ctx.export_fields()
    head, zone, nodes, conn = parse(path)
    assert len(conn) == mesh.ncells
    # one node per distinct corner position, at least the unique corners
    assert len(np.unique(np.round(nodes[:, :3], 6), axis=0)) == len(nodes) >= mesh.ncorners
    dxc = np.repeat(mesh.block_dx(), 512)
    check_bricks(nodes, conn, dxc)
    # every node's values are those of the unique corner at its (wrapped) position
    L = np.array(mesh.nfine) * mesh.dxf
    key = {}
    for c, xyz in enumerate(mesh.corner_xyz.reshape(-1, 3)):
        key[tuple(xyz)] = c
    for t in range(0, len(nodes), max(1, len(nodes) // 500)):
        xyz = np.rint((np.mod(nodes[t, :3], L)) / mesh.dxf).astype(int) % np.array(mesh.nfine)
        c = key[tuple(xyz)]
        np.testing.assert_allclose(nodes[t, 3:6], out["E_n"][c], rtol=1e-5,
                                   atol=1e-5 * np.abs(out["E_n"]).max())
