"""Plain (non-relativistic) Boris mover, Mover::Boris
(src/pic/pic_mover_boris.cpp:126-553), on the GPU against the FP64 oracle
(orc_boris / orc_amr_boris, pinned to the reference's compiled Boris by
tests/test_oracle_pins.py): one step of dt with E^n and the corner B "cur"
slot at the start position, then re-binning.

Tolerances: velocities 2e-6 relative (FP32 storage of the FP64 result),
positions 2e-6 cell per unit of dt*|v|/dx, block/cell ids exact except next to
cell faces; on meshes with open axes the deleted set equals the oracle's."""
import numpy as np
import pytest

import amps_gb300 as A
from tests import oracle_lib as O
from tests.gpu_cases import by_id, face_distance, make_case, rel_err
from tests.test_gpu_amr import amr_case, face_dist, gpu_for, oracle_for
from tests.test_gpu_open_fields import open_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dt,vscale", [(1.0, 1.0), (20.0, 6.0)])
def test_boris_matches_oracle(dt, vscale):
    wl, ic, x, f = make_case(nb=(2, 2, 2), ppc=4, seed=71, vscale=vscale, e_amp=0.02, b_amp=0.3)
    with A.EcsimContext(wl, capacity=len(x) + 1024, track_ids=True) as ctx:
        ctx.import_particles(x, ic["v"].astype(np.float64), ic["spec"])
        ctx.import_fields(**f)
        # the oracle starts from the device's FP32-stored state
        e0 = by_id(ctx.export_particles())
        ctx.MoveParticlesBoris(dt)
        e = by_id(ctx.export_particles())
        assert ctx.num_particles() == len(x)
    st = O.OracleState(wl, e0["x"], e0["v"], e0["spec"], f)
    assert st.boris(dt) == 0
    assert rel_err(e["v"], st.v) < 2e-6
    L = np.array(wl.mesh.shape, float) * wl.mesh.dx
    d = e["x"] - st.x
    d -= L * np.rint(d / L)
    assert np.max(np.abs(d)) < 2e-6 * wl.mesh.dx * max(1.0, dt * np.abs(st.v).max() / wl.mesh.dx)
    mism = (e["block"] != st.block) | (e["cell"] != st.cell)
    assert np.all(face_distance(st.x[mism]) < 1e-5), mism.sum()
    if vscale > 1:
        assert (e["block"] != e0["block"]).sum() > 100   # block crossings and periodic wraps


def test_amr_boris_matches_oracle():
    mesh, wl, ic, x, f = amr_case(ppc=4, seed=73, e_amp=0.02, b_amp=0.3)
    ic["v"] = ic["v"].astype(np.float64) * 6.0
    dt = 20.0
    with gpu_for(mesh, wl, ic, x, f) as ctx:
        e0 = by_id(ctx.export_particles())
        ctx.MoveParticlesBoris(dt)
        e = by_id(ctx.export_particles())
        assert ctx.num_particles() == len(x)
    ao = oracle_for(mesh, wl, {"v": e0["v"], "spec": e0["spec"]}, e0["x"], f)
    np.testing.assert_array_equal(ao.block, e0["block"])
    assert ao.boris(dt) == 0
    assert rel_err(e["v"], ao.v) < 2e-6
    L = np.array(mesh.nfine, float) * mesh.dx0 / (1 << mesh.lmax)
    d = e["x"] - ao.x
    d -= L * np.rint(d / L)
    assert np.max(np.abs(d)) < 2e-6 * mesh.dx0 * max(1.0, dt * np.abs(ao.v).max() / mesh.dx0)
    mism = (e["block"] != ao.block) | (e["cell"] != ao.cell)
    assert mism.sum() < max(5, len(x) // 10000)
    assert np.all(face_dist(mesh, ao.x[mism], ao.block[mism]) < 1e-4), mism.sum()
    lv = mesh.level
    assert np.any(lv[e["block"]] != lv[e0["block"]])   # particles crossed levels


@pytest.fixture
def open_oracle():
    lib = O.load()
    yield lib
    lib.orc_set_open_axes(0)


@pytest.mark.parametrize("nb0,lmax,open_axes", [((3, 2, 2), 0, (True, False, True)),
                                                 ((4, 4, 4), 1, (True, True, False))])
def test_boris_open_faces_delete_like_oracle(open_oracle, nb0, lmax, open_axes):
    mesh, wl, ic, x, f = open_case(nb0, lmax, open_axes, 1, seed=89, vscale=6.0)
    open_oracle.orc_set_open_axes(sum(1 << d for d in range(3) if open_axes[d]))
    dt = 30.0
    with gpu_for(mesh, wl, ic, x, f) as ctx:
        e0 = by_id(ctx.export_particles())
        ctx.MoveParticlesBoris(dt)
        e = by_id(ctx.export_particles())
        n_left = ctx.num_particles()
    ao = oracle_for(mesh, wl, {"v": e0["v"], "spec": e0["spec"]}, e0["x"], f)
    ndel = ao.boris(dt)
    alive = ao.block >= 0
    assert ndel == (~alive).sum() and ndel > 50 and alive.sum() > 50
    assert n_left == alive.sum()
    np.testing.assert_array_equal(e["id"], e0["id"][alive])
    assert rel_err(e["v"], ao.v[alive]) < 2e-6
    L = np.array(mesh.nfine, float) * mesh.dx0 / (1 << mesh.lmax)
    d = e["x"] - ao.x[alive]
    d -= L * np.rint(d / L)
    assert np.max(np.abs(d)) < 2e-6 * mesh.dx0 * max(1.0, dt * np.abs(ao.v).max() / mesh.dx0)
