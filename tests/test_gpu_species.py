"""Species moments on corners (the reference's
_PIC_FIELD_SOLVER_SAMPLE_SPECIES_ON_CORNER_ sampling in ProcessCell) against
the FP64 oracle: rho, rho u, rho u u per species and corner, on a uniform mesh
with per-particle weight corrections and on a two-level AMR mesh, at the
deposition of the imported state and after a full ECSIM step; the total mass
of every species is conserved by the corner sums."""
import numpy as np
import pytest

from tests import gpu_cases as G
from tests import oracle_lib as O
from tests.gpu_cases import rel_err
from tests.test_gpu_amr import amr_case, gpu_for, oracle_for

pytestmark = pytest.mark.gpu


def check(gpu, orc, tol):
    assert gpu.shape == orc.shape
    for s in range(gpu.shape[1]):
        for q in range(10):
            assert rel_err(gpu[:, s, q], orc[:, s, q]) < tol, (s, q, rel_err(gpu[:, s, q], orc[:, s, q]))


def test_uniform_species_moments_match_oracle():
    wl, ic, x, f = G.make_case(nb=(2, 2, 2), ppc=8, seed=12)
    rng = np.random.default_rng(12)
    wc = rng.uniform(0.5, 1.5, len(ic["spec"]))
    with G.gpu_ctx(wl, ic, x, f, wcorr=wc) as ctx:
        ctx.set_species_moments(True)
        ctx.UpdateJMassMatrix()
        g0 = ctx.export_species_moments()
        st = G.oracle_state(wl, ic, x, f, wcorr=wc)
        check(g0, st.species_moments(), 1e-6)
        # total mass per species: sum over corners of rho times the cell volume
        V = float(wl.mesh.dx) ** 3
        for s, sp in enumerate(wl.species):
            m_tot = np.sum(sp.mass * sp.weight * wc[ic["spec"] == s])
            assert abs(np.sum(g0[:, s, 0]) * V - m_tot) < 1e-6 * m_tot
        # after a full step: the oracle from the device's exported particles
        ctx.PicTimeStep(tol=1e-8, maxit=200, precond=1)
        g1 = ctx.export_species_moments()
        e = G.by_id(ctx.export_particles())
        o1 = O.OracleState(wl, e["x"], e["v"], e["spec"], ctx.export_fields(), wcorr=wc)
        check(g1, o1.species_moments(), 1e-5)


def test_amr_species_moments_match_oracle():
    mesh, wl, ic, x, f = amr_case(ppc=8, seed=13)
    with gpu_for(mesh, wl, ic, x, f) as ctx:
        ctx.set_species_moments(True)
        ctx.UpdateJMassMatrix()
        g0 = ctx.export_species_moments()
    ao = oracle_for(mesh, wl, ic, x, f)
    check(g0, ao.species_moments(), 1e-6)
