"""Launch configuration: CUDA-graph particle steps and the autotuner change
how kernels are launched, never what they compute."""
import numpy as np
import pytest

import amps_gb300 as A
from tests.gpu_cases import by_id, make_case, rel_err
from tests.test_gpu_amr import amr_case, gpu_for

pytestmark = pytest.mark.gpu


def run_steps(graphs, nsteps=4):
    wl, ic, x, f = make_case(nb=(2, 2, 2), ppc=8, seed=41, vscale=4.0)
    with A.EcsimContext(wl, capacity=len(x) + 4096, track_ids=True) as ctx:
        ctx.set_graphs(graphs)
        ctx.import_particles(x, ic["v"].astype(np.float64), ic["spec"])
        ctx.import_fields(**f)
        energies = []
        for _ in range(nsteps):
            s = ctx.PicTimeStep(tol=1e-10, maxit=200, precond=1)
            energies.append((s.particle_energy, s.solve.wave_energy))
        e = by_id(ctx.export_particles())
        J, M = ctx.export_moments()
        return energies, e, J, M


def test_graph_steps_equal_stream_steps():
    # arrivals reserve destination slots with atomics, so particle order inside
    # a cell (and the rounding of per-cell sums) may differ from run to run
    en0, e0, J0, M0 = run_steps(False)
    en1, e1, J1, M1 = run_steps(True)
    assert np.mean((e0["block"] == e1["block"]) & (e0["cell"] == e1["cell"])) > 0.9999
    assert rel_err(e1["v"], e0["v"]) < 1e-5
    assert rel_err(J1, J0) < 1e-5
    assert rel_err(M1, M0) < 1e-5
    for a, b in zip(en0, en1):
        assert a[0] == pytest.approx(b[0], rel=1e-6)
        assert a[1] == pytest.approx(b[1], rel=1e-6)


def test_autotune_keeps_solution():
    wl, ic, x, f = make_case(nb=(2, 2, 2), ppc=8, seed=43)
    out = {}
    with A.EcsimContext(wl, capacity=len(x) + 1024) as ctx:
        ctx.import_particles(x, ic["v"].astype(np.float64), ic["spec"])
        ctx.import_fields(**f)
        ctx.UpdateJMassMatrix()
        f0 = ctx.export_fields()
        st = ctx.TimeStep(tol=1e-10, maxit=200, precond=1)
        out[0] = ctx.export_fields()
        rep = ctx.autotune()
        assert rep["threads_per_cta"] in (64, 128, 256)
        assert rep["reduction_ctas"] in (76, 152, 304)
        assert all(t > 0 for t in rep["operator_ms_tb64_128_256"] + rep["sweep_ms_cta76_152_304"])
        ctx.import_fields(**f0)
        st2 = ctx.TimeStep(tol=1e-10, maxit=200, precond=1)
        out[1] = ctx.export_fields()
    assert st.converged and st2.converged
    for k in ("E_n", "B_center"):
        assert rel_err(out[1][k], out[0][k]) < 1e-9


@pytest.mark.parametrize("amr", [False, True])
@pytest.mark.parametrize("precond", [0, 1])
def test_graph_field_solve_equals_stream_solve(amr, precond):
    """With graphs on, a solve's first GMRES cycle runs as one CUDA graph once
    an earlier solve told how many Arnoldi steps to queue: the same kernels in
    the same order as the stream solve.  In one context (one mass matrix),
    solves of the same system with graphs off and then on take the same
    iteration counts and give the same fields: bit for bit on the uniform mesh,
    to 1e-9 of the largest entry on the AMR mesh (its operator sums with FP32
    atomics, whose order varies from run to run)."""
    if amr:
        mesh, wl, ic, x, f = amr_case(seed=29)
        ctx = gpu_for(mesh, wl, ic, x, f)
    else:
        wl, ic, x, f = make_case(nb=(2, 2, 2), ppc=8, seed=47)
        ctx = A.EcsimContext(wl, capacity=len(x) + 1024)
        ctx.import_particles(x, ic["v"].astype(np.float64), ic["spec"])
        ctx.import_fields(**f)
    out = {}
    with ctx:
        ctx.UpdateJMassMatrix()
        f0 = ctx.export_fields()
        for graphs in (False, True):
            ctx.set_graphs(graphs)
            its = []
            for _ in range(3):
                ctx.import_fields(**f0)
                st = ctx.TimeStep(tol=1e-10, maxit=200, precond=precond)
                assert st.converged
                its.append(st.iterations)
            out[graphs] = (its, ctx.export_fields())
    assert out[True][0] == out[False][0]
    for k, v in out[False][1].items():
        if amr:
            assert rel_err(out[True][1][k], v) <= 1e-9, k
        else:
            np.testing.assert_array_equal(out[True][1][k], v, err_msg=k)


def test_autotune_compares_arrivals_chunks():
    """autotune arms a comparison of the two arrivals variants over the next 6
    particle steps (graphs on: those steps run as stream launches), then keeps
    the faster; the steps still do their work (layout and moments valid)"""
    wl, ic, x, f = make_case(nb=(2, 2, 2), ppc=8, seed=53, vscale=4.0)
    with A.EcsimContext(wl, capacity=len(x) + 4096, track_ids=True) as ctx:
        ctx.set_graphs(True)
        ctx.import_particles(x, ic["v"].astype(np.float64), ic["spec"])
        ctx.import_fields(**f)
        ctx.UpdateJMassMatrix()
        ctx.autotune()
        assert ctx.particle_tuning()["pending_steps"] == 6
        for _ in range(6):
            ctx.push_deposit(want_energy=False)
        t = ctx.particle_tuning()
        assert t["pending_steps"] == 0 and t["arrivals_chunk"] in (16, 32)
        assert all(m > 0 for m in t["arrivals_ms_16_32"]), t
        ms = t["arrivals_ms_16_32"]
        assert t["arrivals_chunk"] == (32 if ms[1] < ms[0] else 16)
        ctx.push_deposit(want_energy=False)          # a graph step with the choice
        e = by_id(ctx.export_particles())
        np.testing.assert_array_equal(e["id"], np.arange(len(x)))
        J1, M1 = ctx.export_moments()
        ctx.UpdateJMassMatrix()
        J2, M2 = ctx.export_moments()
        assert rel_err(J1, J2) <= 2e-6 and rel_err(M1, M2) <= 2e-6
