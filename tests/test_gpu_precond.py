"""Learned GMRES preconditioner on the GPU.

* the training kernels' loss and weight gradients equal the FP64 oracle's
  (tests/../oracle/precond_oracle.py, itself checked by finite differences);
* the inference paths (FP32 training forward; BF16 tensor cores) equal the
  oracle's forward within their precision;
* harvesting pairs from Jacobi solves and training on them lowers the loss,
  and the trained network as right preconditioner reaches the same tolerance
  and the same solution as Jacobi GMRES in fewer iterations;
* the FP32 inner operator with FP64 refinement converges to the same solution
  as the FP64 operator.
"""
import numpy as np
import pytest

import amps_gb300 as A
from amps_gb300 import precond as PC
from oracle import precond_oracle as PO
from tests.gpu_cases import rel_err

pytestmark = pytest.mark.gpu


def small_ctx(nb=(2, 2, 2), ppc=8):
    wl = A.electron_proton_plasma("pc", *nb, ppc, 3)
    ctx = A.EcsimContext(wl, capacity=wl.nparticles, track_ids=False)
    return wl, ctx


def random_samples(rng, S):
    return (rng.standard_normal((S, 1000, 3)).astype(np.float32),
            rng.standard_normal((S, 512, 3)).astype(np.float32))


def test_loss_and_gradients_match_oracle():
    rng = np.random.default_rng(3)
    wl, ctx = small_ctx()
    with ctx:
        w = A.init_precond_weights(seed=4, out_scale=0.5)
        ctx.precond_load(*w)
        x, e = random_samples(rng, 5)
        loss, g = ctx.precond_loss_grad(x, e)
    lref, gref = PO.loss_grad(x, e, *w)
    assert loss == pytest.approx(lref, rel=1e-5)
    for a, b in zip(g, gref):
        assert rel_err(a, b) < 1e-4


def test_forward_fp32_matches_oracle():
    rng = np.random.default_rng(5)
    wl, ctx = small_ctx()
    with ctx:
        w = A.init_precond_weights(seed=6, out_scale=1.0)
        ctx.precond_load(*w)
        x, _ = random_samples(rng, 7)
        y = ctx.precond_forward(x, tensor_cores=False)
    _, _, _, yref = PO.forward(x, *w)
    assert rel_err(y, PO.owned(yref)) < 1e-5


def test_forward_tensor_cores_matches_oracle():
    # BF16 inputs, weights and activations with FP32 accumulation: ~1% of |y|
    rng = np.random.default_rng(8)
    wl, ctx = small_ctx()
    with ctx:
        w = A.init_precond_weights(seed=9, out_scale=1.0)
        ctx.precond_load(*w)
        x, _ = random_samples(rng, 9)
        y_tc = ctx.precond_forward(x, tensor_cores=True)
        y32 = ctx.precond_forward(x, tensor_cores=False)
    yref = PO.owned(PO.forward(x, *w)[3])
    assert np.all(np.isfinite(y_tc))
    assert np.linalg.norm(y_tc - yref) / np.linalg.norm(yref) < 1e-2
    assert rel_err(y_tc, yref) < 3e-2
    assert rel_err(y32, yref) < 1e-5


def test_inner_fp32_solution_matches_fp64():
    wl, ctx = small_ctx()
    out = {}
    with ctx:
        PC.random_state(ctx, wl, 11, e_amp=1e-3, b_amp=0.02)
        f0 = ctx.export_fields()
        for fp64 in (True, False):
            ctx.import_fields(**f0)
            ctx.set_inner_fp64(fp64)
            st = ctx.TimeStep(tol=1e-10, maxit=400, precond=1)
            assert st.converged and st.rel_residual <= 1e-10
            out[fp64] = ctx.export_fields()
    for k in ("E_n", "E_half", "B_center"):
        assert rel_err(out[False][k], out[True][k]) < 1e-8, k


def test_trained_preconditioner_beats_jacobi():
    wl, ctx = small_ctx(ppc=16)
    with ctx:
        ctx.precond_load(*A.init_precond_weights(seed=0))
        info = PC.harvest_training_pairs(ctx, wl, 3000, e_amp=1e-3, b_amp=0.02)
        assert info["samples"] == 3000
        x, e = ctx.precond_samples(0, 4)
        assert np.all(np.isfinite(x)) and np.all(np.isfinite(e))
        loss = ctx.precond_train(epochs=30, batch=32, lr=2e-3, seed=2)
        assert loss[-1] < 0.5 * loss[0], loss
        # held-out pairs from a Jacobi solve on a new state: the network's
        # correction beats Jacobi alone (N = 0) by a wide margin
        ctx.precond_harvest(600)
        PC.random_state(ctx, wl, 77, e_amp=1e-3, b_amp=0.02)
        ctx.TimeStep(tol=1e-8, maxit=400, precond=1)
        n = ctx.precond_num_samples()
        assert n > 0
        xh, eh = ctx.precond_samples(0, n)
        l_net, _ = ctx.precond_loss_grad(xh, eh)
        l_jac = float(np.mean((PO.owned(xh.reshape(n, 10, 10, 10, 3).astype(np.float64)) - eh) ** 2))
        assert l_net < 0.1 * l_jac, (l_net, l_jac)
        ctx.precond_harvest(0)
        # held-out state: same tolerance, same solution, no more iterations than Jacobi
        PC.random_state(ctx, wl, 99, e_amp=1e-3, b_amp=0.02)
        f0 = ctx.export_fields()
        res = {}
        for pc, tc in ((1, False), (2, False), (2, True)):
            if pc == 2:
                ctx.precond_use_tensor_cores(tc)
            ctx.import_fields(**f0)
            st = ctx.TimeStep(tol=1e-8, maxit=400, precond=pc)
            assert st.converged and st.rel_residual <= 1e-8
            res[(pc, tc)] = (st.iterations, ctx.export_fields())
    jac = res[(1, False)][0]
    assert res[(2, False)][0] <= jac and res[(2, True)][0] <= jac, {k: v[0] for k, v in res.items()}
    for key in ((2, False), (2, True)):
        for k in ("E_n", "B_center"):
            assert rel_err(res[key][1][k], res[(1, False)][1][k]) < 1e-6, (key, k)
