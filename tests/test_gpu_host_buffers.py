"""Host-buffer paths of the C ABI: page-locked host arrays are read and
written by the layout kernels directly across the host link, pageable ones go
through a device staging copy; both must give identical bytes.
"""
import numpy as np
import pytest

import amps_gb300 as A
from tests.test_gpu_amr import amr_case, gpu_for

pytestmark = pytest.mark.gpu


def pinned_like(pin, arrs):
    out = {}
    for k, a in arrs.items():
        out[k] = pin.empty(a.shape)
        out[k][:] = a
    return out


def test_uniform_fields_and_moments_pinned_equal_pageable():
    wl = A.electron_proton_plasma("u", 2, 2, 2, 8, 2)
    ic = A.make_initial_condition(wl)
    pin = A.PinnedArrays()
    with A.EcsimContext(wl, capacity=wl.nparticles + 1024) as ctx:
        ctx.import_particles_local(ic["u"], ic["v"], ic["spec"], ic["block"])
        rng = np.random.default_rng(3)
        f = A.initial_fields(wl)
        f = {k: v + 1e-3 * rng.standard_normal(v.shape) for k, v in f.items()}
        ctx.import_fields(**pinned_like(pin, f))
        g_np = ctx.export_fields()
        g_pin = ctx.export_fields(out=pinned_like(pin, {k: np.zeros_like(v) for k, v in g_np.items()}))
        for k in f:
            assert np.array_equal(g_np[k], f[k]), k
            assert np.array_equal(g_pin[k], f[k]), k
        ctx.UpdateJMassMatrix()
        J, M = ctx.export_moments()
        pJ, pM = pin.empty(J.shape), pin.empty(M.shape)
        ctx.export_moments(out=(pJ, pM))
        assert np.array_equal(J, pJ) and np.array_equal(M, pM)
    pin.free()


def test_amr_cell_moments_pinned_equal_pageable():
    mesh, wl, ic, x, f = amr_case(ppc=8)
    pin = A.PinnedArrays()
    with gpu_for(mesh, wl, ic, x, f) as ctx:
        ctx.UpdateJMassMatrix()
        J, M = ctx.export_cell_moments()
        pJ, pM = pin.empty(J.shape), pin.empty(M.shape)
        ctx.export_cell_moments(out=(pJ, pM))
        assert np.array_equal(J, pJ) and np.array_equal(M, pM)
        # J alone into a page-locked array, M into a pageable one
        qJ, qM = pin.empty(J.shape), np.empty(M.shape)
        ctx.export_cell_moments(out=(qJ, qM))
        assert np.array_equal(J, qJ) and np.array_equal(M, qM)
    pin.free()


def test_amr_corner_moments_pinned_equal_pageable():
    """the corner-layout export written across the host link into page-locked
    arrays equals the one copied through a device buffer, also mixed"""
    mesh, wl, ic, x, f = amr_case(ppc=8)
    pin = A.PinnedArrays()
    with gpu_for(mesh, wl, ic, x, f) as ctx:
        ctx.UpdateJMassMatrix()
        J, M = ctx.export_moments()
        pJ, pM = pin.empty(J.shape), pin.empty(M.shape)
        ctx.export_moments(out=(pJ, pM))
        assert np.array_equal(J, pJ) and np.array_equal(M, pM)
        qJ, qM = np.empty(J.shape), pin.empty(M.shape)
        ctx.export_moments(out=(qJ, qM))
        assert np.array_equal(J, qJ) and np.array_equal(M, qM)
        J1, _ = ctx.export_moments(with_m=False)
        assert np.array_equal(J, J1)
    pin.free()
