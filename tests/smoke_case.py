"""One small ECSIM time step on cuda:0 through the C ABI, checked against the
FP64 oracle (used by __graft_entry__.smoke())."""
import numpy as np

from tests import gpu_cases as G


def run_smoke():
    wl, ic, x, f = G.make_case(nb=(1, 1, 2), ppc=4, seed=100)
    ctx = G.gpu_ctx(wl, ic, x, f)
    st = G.oracle_state(wl, ic, x, f)
    ctx.UpdateJMassMatrix()
    st.deposit()
    s = ctx.PicTimeStep(tol=1e-10, maxit=200, precond=1)
    it, diag = st.step(tol=1e-10, maxit=200, precond=1)
    assert s.solve.converged == 1, "GMRES did not converge"
    J, M = ctx.export_moments()
    ej, em = G.rel_err(J, st.J), G.rel_err(M, st.M)
    assert ej <= 1e-5 and em <= 1e-5, (ej, em)
    assert abs(s.particle_energy - diag[0]) <= 1e-6 * abs(diag[0])
    g = G.by_id(ctx.export_particles())
    assert np.abs(g["x"] - st.x).max() < 1e-4
    ctx.close()
    print("smoke ok: J err %.2e, M err %.2e, GMRES %d iterations" % (ej, em, s.solve.iterations))
