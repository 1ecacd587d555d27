"""The outer GMRES residual and the RHS are evaluated in FP32 pairs (FP64
accuracy at FP32 throughput): if that evaluation lost accuracy, residuals
below ~1e-8 would be out of reach.  Uniform and AMR solves must converge to
1e-11 and agree with the oracle's FP64 solve from the same state."""
import ctypes as C

import numpy as np
import pytest

from tests import gpu_cases as G
from tests.gpu_cases import rel_err
from tests.oracle_lib import p
from tests.test_gpu_amr import amr_case, gpu_for, oracle_for

pytestmark = pytest.mark.gpu


def test_uniform_solve_reaches_1e11():
    wl, ic, x, f = G.make_case(nb=(2, 2, 2), ppc=8, seed=31)
    with G.gpu_ctx(wl, ic, x, f) as ctx:
        ctx.UpdateJMassMatrix()
        for fp64 in (False, True):
            ctx.import_fields(**f)
            ctx.set_inner_fp64(fp64)
            st = ctx.TimeStep(tol=1e-11, maxit=400, precond=1)
            assert st.converged and st.rel_residual <= 1e-11, (fp64, st.rel_residual)
        g = ctx.export_fields()
        J, M = ctx.export_moments()
    o = G.oracle_state(wl, ic, x, f)
    o.J[:], o.M[:] = J, M
    b = o.rhs()
    dE = np.zeros_like(b)
    res = np.zeros(1)
    o.lib.orc_gmres(C.byref(o.m), p(o.M), p(b), p(dE), 1e-12, 2000, 30, 1, p(res))
    assert rel_err(g["E_half"], o.E_n + dE) < 1e-9


def test_amr_solve_reaches_1e11():
    mesh, wl, ic, x, f = amr_case(ppc=8, seed=32)
    with gpu_for(mesh, wl, ic, x, f) as ctx:
        ctx.UpdateJMassMatrix()
        st = ctx.TimeStep(tol=1e-11, maxit=600, precond=1)
        assert st.converged and st.rel_residual <= 1e-11, st.rel_residual
        g = ctx.export_fields()
        cJ, cM = ctx.export_cell_moments()
    ao = oracle_for(mesh, wl, ic, x, f)
    ao.cellJ[:], ao.cellM[:] = cJ.reshape(-1), cM.reshape(-1)
    ao.field_solve(tol=1e-12, maxit=3000)
    assert rel_err(g["E_half"], ao.E_half) < 1e-9
