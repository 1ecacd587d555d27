"""Open particle boundaries (the mover's delete-on-exit processing) against
the FP64 oracle: particles whose move leaves the domain through a face of an
open axis are deleted, the others move and wrap as before; the surviving set,
their states and the moments they deposit match the oracle, on a uniform and
on a two-level AMR mesh, with the step as a CUDA graph and without."""
import numpy as np
import pytest

from tests import gpu_cases as G
from tests import oracle_lib as O
from tests.test_gpu_amr import amr_case, gpu_for, oracle_for

pytestmark = pytest.mark.gpu


@pytest.fixture
def open_oracle():
    lib = O.load()
    yield lib
    lib.orc_set_open_axes(0)


@pytest.mark.parametrize("graphs", [False, True])
def test_uniform_open_axes_delete_leaving_particles(open_oracle, graphs):
    wl, ic, x, f = G.make_case(nb=(2, 2, 2), ppc=8, seed=41, vscale=40.0)
    open_oracle.orc_set_open_axes(1 | 4)          # x and z open, y periodic
    with G.gpu_ctx(wl, ic, x, f) as ctx:
        ctx.set_open_axes(True, False, True)
        ctx.set_graphs(graphs)
        n0 = ctx.num_particles()
        ctx.push_deposit()
        st = G.oracle_state(wl, ic, x, f)
        st.push()
        st.deposit()
        alive = st.block >= 0
        assert (~alive).sum() > 100                # the case does exercise the faces
        assert ctx.deleted_particles() == (~alive).sum()
        assert ctx.num_particles() == n0 - (~alive).sum()
        g = G.by_id(ctx.export_particles())
        np.testing.assert_array_equal(g["id"], np.flatnonzero(alive))
        L = np.array(wl.mesh.shape) * wl.mesh.dx
        d = np.abs(g["x"] - st.x[alive])
        d = np.minimum(d, np.abs(d - L))
        assert d.max() <= 4e-6
        assert np.abs(g["v"] - st.v[alive]).max() <= 2e-5 * np.abs(st.v).max()
        J, M = ctx.export_moments()
        assert G.rel_err(J, st.J) <= 1e-5 and G.rel_err(M, st.M) <= 1e-5
        # a second step from the reduced set
        ctx.push_deposit()
        st.push()
        assert ctx.num_particles() == int((st.block >= 0).sum())


def test_amr_open_axis_deletes_leaving_particles(open_oracle):
    mesh, wl, ic, x, f = amr_case(ppc=8, seed=42, vscale=40.0)
    open_oracle.orc_set_open_axes(2)               # y open
    with gpu_for(mesh, wl, ic, x, f) as ctx:
        ctx.set_open_axes(False, True, False)
        n0 = ctx.num_particles()
        ctx.push_deposit()
        ao = oracle_for(mesh, wl, ic, x, f)
        ao.push()
        ao.deposit()
        alive = ao.block >= 0
        assert (~alive).sum() > 100
        assert ctx.num_particles() == n0 - (~alive).sum()
        g = G.by_id(ctx.export_particles())
        np.testing.assert_array_equal(g["id"], np.flatnonzero(alive))
        cJ, cM = ctx.export_cell_moments()
        assert G.rel_err(cJ.reshape(-1), ao.cellJ) <= 1e-5
        assert G.rel_err(cM.reshape(-1), ao.cellM) <= 1e-5
