"""Mesh relativistic Boris mover (Mover::Relativistic::Boris) on the GPU
against the FP64 oracle: sub-step counts equal, positions and velocities within
FP32 storage error, block/cell ids exact except next to cell faces."""
import numpy as np
import pytest

import amps_gb300 as A
from tests import oracle_lib as O
from tests.gpu_cases import by_id, face_distance, make_case, rel_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dt_total,vscale", [(20.0, 4.0), (60.0, 8.0)])
def test_relboris_matches_oracle(dt_total, vscale):
    # relativistic speeds: scale the thermal velocities up (c = 1); B of ~0.5
    wl, ic, x, f = make_case(nb=(2, 2, 2), ppc=4, seed=61, vscale=vscale, e_amp=0.02, b_amp=0.3)
    v = ic["v"].astype(np.float64)
    sp = np.linalg.norm(v, axis=1)
    v = np.where(sp[:, None] >= 0.95, v * (0.95 / sp)[:, None], v)   # keep |v| < c
    with A.EcsimContext(wl, capacity=len(x) + 1024, track_ids=True) as ctx:
        ctx.import_particles(x, v, ic["spec"])
        ctx.import_fields(**f)
        # the oracle starts from the device's FP32-stored state
        e0 = by_id(ctx.export_particles())
        nsub = ctx.MoveParticlesRelativistic(dt_total, 1.0)
        e = by_id(ctx.export_particles())
    st = O.OracleState(wl, e0["x"], e0["v"], e0["spec"], f)
    nsub_ref = st.relboris(dt_total, 1.0)
    assert nsub > len(x) and abs(nsub - nsub_ref) <= max(2, nsub_ref // 10000)
    # the device stores the result in FP32 (offsets and velocities)
    assert rel_err(e["v"], st.v) < 2e-6
    L = np.array(wl.mesh.shape, float) * wl.mesh.dx
    d = e["x"] - st.x
    d -= L * np.rint(d / L)
    assert np.max(np.abs(d)) < 2e-6 * wl.mesh.dx * max(1.0, dt_total / 10.0)
    mism = (e["block"] != st.block) | (e["cell"] != st.cell)
    assert np.all(face_distance(st.x[mism]) < 1e-4), mism.sum()
