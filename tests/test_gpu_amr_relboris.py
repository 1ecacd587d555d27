"""Mesh relativistic Boris mover (Mover::Relativistic::Boris) on a two-level
periodic AMR mesh against the FP64 AMR oracle: every sub-step re-locates the
particle in the block tree and interpolates E^n and the corner B from its leaf
block (hanging corners through their constraint).  Sub-step counts agree,
positions and velocities within FP32 storage error, block/cell ids exact
except next to cell faces; a mesh with open axes is refused."""
import numpy as np
import pytest

import amps_gb300 as A
from tests.gpu_cases import make_case, rel_err
from tests.test_gpu_amr import amr_case, by_id, face_dist, gpu_for, oracle_for
from tests.test_gpu_open_fields import open_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dt_total,vscale", [(20.0, 4.0), (60.0, 8.0)])
def test_amr_relboris_matches_oracle(dt_total, vscale):
    mesh, wl, ic, x, f = amr_case(ppc=4, seed=67, e_amp=0.02, b_amp=0.3)
    v = ic["v"].astype(np.float64) * vscale
    sp = np.linalg.norm(v, axis=1)
    ic["v"] = np.where(sp[:, None] >= 0.95, v * (0.95 / sp)[:, None], v)   # keep |v| < c = 1
    with gpu_for(mesh, wl, ic, x, f) as ctx:
        # the oracle starts from the device's FP32-stored state
        e0 = by_id(ctx.export_particles())
        nsub = ctx.MoveParticlesRelativistic(dt_total, 1.0)
        e = by_id(ctx.export_particles())
        assert ctx.num_particles() == len(x)
    ao = oracle_for(mesh, wl, {"v": e0["v"], "spec": e0["spec"]}, e0["x"], f)
    np.testing.assert_array_equal(ao.block, e0["block"])
    nsub_ref = ao.relboris(dt_total, 1.0)
    assert nsub > len(x) and abs(nsub - nsub_ref) <= max(2, nsub_ref // 10000)
    assert rel_err(e["v"], ao.v) < 2e-6
    L = np.array(mesh.nfine, float) * mesh.dx0 / (1 << mesh.lmax)
    d = e["x"] - ao.x
    d -= L * np.rint(d / L)
    assert np.max(np.abs(d)) < 2e-6 * mesh.dx0 * max(1.0, dt_total / 10.0)
    mism = (e["block"] != ao.block) | (e["cell"] != ao.cell)
    assert mism.sum() < max(5, len(x) // 10000)
    assert np.all(face_dist(mesh, ao.x[mism], ao.block[mism]) < 1e-4), mism.sum()
    # particles crossed levels
    lv = mesh.level
    assert np.any(lv[e["block"]] != lv[e0["block"]])


@pytest.fixture
def open_oracle():
    from tests import oracle_lib as O
    lib = O.load()
    yield lib
    lib.orc_set_open_axes(0)


@pytest.mark.parametrize("nb0,lmax,open_axes", [((3, 2, 2), 0, (True, False, True)),
                                                 ((4, 4, 4), 1, (True, True, False))])
def test_relboris_open_faces_delete_like_oracle(open_oracle, nb0, lmax, open_axes):
    """fast particles on a mesh with open axes: the set deleted at the open
    faces is the oracle's, the survivors follow it"""
    mesh, wl, ic, x, f = open_case(nb0, lmax, open_axes, 1, seed=87, vscale=6.0)
    v = ic["v"].astype(np.float64)
    sp = np.linalg.norm(v, axis=1)
    ic["v"] = np.where(sp[:, None] >= 0.95, v * (0.95 / sp)[:, None], v)
    open_oracle.orc_set_open_axes(sum(1 << d for d in range(3) if open_axes[d]))
    with gpu_for(mesh, wl, ic, x, f) as ctx:
        e0 = by_id(ctx.export_particles())
        ctx.MoveParticlesRelativistic(8.0, 1.0)
        e = by_id(ctx.export_particles())
        n_left = ctx.num_particles()
    ao = oracle_for(mesh, wl, {"v": e0["v"], "spec": e0["spec"]}, e0["x"], f)
    ao.relboris(8.0, 1.0)
    alive = ao.block >= 0
    assert (~alive).sum() > 50 and alive.sum() > 50
    assert n_left == alive.sum()
    np.testing.assert_array_equal(e["id"], e0["id"][alive])
    assert rel_err(e["v"], ao.v[alive]) < 2e-6
    L = np.array(mesh.nfine, float) * mesh.dx0 / (1 << mesh.lmax)
    d = e["x"] - ao.x[alive]
    d -= L * np.rint(d / L)
    assert np.max(np.abs(d)) < 2e-6 * mesh.dx0
