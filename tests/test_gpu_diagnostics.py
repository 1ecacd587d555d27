"""UpdateJMassMatrix's diagnostics on the GPU against the FP64 oracle: the
total particle kinetic energy (ProcessCell :2238, summed in FP64 by the
reference; float pairs on the GPU) and the per-species maximum CFL number
(:2236, :2356-2359, :3972-3987; amps_gpu_particle_cfl).

Both are compared on identical particles (the oracle reads the GPU's exported,
FP32-representable state), so the only difference is arithmetic: relative
1e-12 for both."""
import numpy as np
import pytest

import amps_gb300 as A
from tests import gpu_cases as G
from tests import oracle_lib as O
from tests.test_gpu_amr import amr_case, gpu_for, oracle_for

pytestmark = pytest.mark.gpu


def cfl_restated(v, spec, cell_key, diag, dt, nspec):
    """numpy restatement of the per-species maximum of ProcessCell's cflCell"""
    out = np.zeros(nspec)
    speed = np.sqrt(np.sum(v * v, axis=1)) * dt
    for s in range(nspec):
        m = spec == s
        keys, inv = np.unique(cell_key[m], return_inverse=True)
        sums = np.bincount(inv, weights=speed[m])
        cnt = np.bincount(inv)
        out[s] = np.max(sums / (cnt * diag[keys]))
    return out


@pytest.mark.parametrize("wcorr", [False, True])
def test_energy_and_cfl_match_oracle_uniform(wcorr):
    wl, ic, x, f = G.make_case(nb=(2, 2, 2), ppc=8, vscale=3.0)
    wc = None
    if wcorr:
        wc = np.random.default_rng(5).uniform(0.5, 2.0, len(x)).astype(np.float32).astype(np.float64)
    ctx = G.gpu_ctx(wl, ic, x, f, wcorr=wc)
    try:
        eg = ctx.UpdateJMassMatrix()
        cg = ctx.particle_cfl()
        st = G.oracle_state(wl, ic, x, f, wcorr=wc)
        eo = st.deposit()
        assert eg == pytest.approx(eo, rel=1e-12), (eg, eo)
        np.testing.assert_allclose(cg, st.cfl(), rtol=1e-12)
        # after a fused push + deposit: the oracle on the pushed particles
        eg2 = ctx.push_deposit()
        cg2 = ctx.particle_cfl()
        g = ctx.export_particles()
        wc2 = None
        if wcorr:
            wc2 = wc[g["id"]]
        st2 = O.OracleState(wl, g["x"], g["v"], g["spec"], f, wc2)
        assert eg2 == pytest.approx(st2.deposit(), rel=1e-12)
        np.testing.assert_allclose(cg2, st2.cfl(), rtol=1e-12)
    finally:
        ctx.close()


def test_energy_and_cfl_match_oracle_amr():
    mesh, wl, ic, x, f = amr_case(ppc=8, seed=29, vscale=2.0)
    with gpu_for(mesh, wl, ic, x, f) as ctx:
        eg = ctx.UpdateJMassMatrix()
        cg = ctx.particle_cfl()
        g = ctx.export_particles()
    ao = oracle_for(mesh, wl, {"v": g["v"], "spec": g["spec"]}, g["x"], f)
    assert eg == pytest.approx(ao.deposit(), rel=1e-12)
    diag = np.sqrt(3.0) * mesh.block_dx()
    key = g["block"].astype(np.int64)
    ref = cfl_restated(g["v"], g["spec"], key * 512 + g["cell"], np.repeat(diag, 512), wl.dt,
                       len(wl.species))
    np.testing.assert_allclose(cg, ref, rtol=1e-12)
