"""The no-allocation deposition entry point against the context path.

amps_gpu_update_j_mass_matrix_noalloc serves callers that cannot let a library
call cudaMalloc or cudaFree (their device memory belongs to their framework's
pool allocator, or they must not stall other streams in mid-step, which
cudaFree does).  This test plays such a caller: it allocates the input and output buffers itself, calls the
entry point twice in a row through the C ABI and checks both results against
amps_gpu_update_j_mass_matrix on the same particles and fields, within the
deposit tolerance used elsewhere (relative 1e-5 for J and M, 1e-6 for the
energy).  The file name sorts last so a run that stops at the first failure
has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import amps_gb300 as A
from amps_gb300 import _capi
from tests import gpu_cases as G

pytestmark = pytest.mark.gpu


class DeviceBuffers:
    """Test-owned device memory through the CUDA runtime."""

    def __init__(self):
        self.rt = C.CDLL("libcudart.so")
        self.ptrs = []

    def put(self, arr):
        arr = np.ascontiguousarray(arr)
        p = C.c_void_p()
        assert self.rt.cudaMalloc(C.byref(p), C.c_size_t(max(arr.nbytes, 1))) == 0
        self.ptrs.append(p)
        if arr.nbytes:
            assert self.rt.cudaMemcpy(p, arr.ctypes.data_as(C.c_void_p), C.c_size_t(arr.nbytes),
                                      1) == 0
        return p

    def empty(self, nbytes):
        return self.put(np.zeros(nbytes, np.uint8))

    def get(self, p, dtype, count):
        out = np.empty(count, dtype)
        assert self.rt.cudaDeviceSynchronize() == 0
        assert self.rt.cudaMemcpy(out.ctypes.data_as(C.c_void_p), p,
                                  C.c_size_t(out.nbytes), 2) == 0
        return out

    def free(self):
        for p in self.ptrs:
            self.rt.cudaFree(p)
        self.ptrs = []


def test_noalloc_deposit_matches_context_deposit_twice():
    wl, ic, x, f = G.make_case(nb=(2, 2, 2), ppc=8, vscale=2.0)
    ctx = G.gpu_ctx(wl, ic, x, f)
    e_ref = ctx.UpdateJMassMatrix()
    J_ref, M_ref = ctx.export_moments()
    exp = ctx.export_particles()          # cell order
    ncell = wl.mesh.ncells
    key = exp["block"].astype(np.int64) * 512 + exp["cell"]
    assert np.all(np.diff(key) >= 0)
    start = np.zeros(ncell + 1, np.int32)
    start[1:] = np.cumsum(np.bincount(key, minlength=ncell))
    u = ((exp["x"] - A.block_origins(wl.mesh, exp["block"])) / wl.mesh.dx).astype(np.float32)
    v = exp["v"].astype(np.float32)
    n = len(key)
    mem = DeviceBuffers()
    try:
        d_start = mem.put(start)
        d_u = mem.put(np.ascontiguousarray(u.T))
        d_v = mem.put(np.ascontiguousarray(v.T))
        d_sp = mem.put(exp["spec"].astype(np.uint8))
        d_B = mem.put(np.ascontiguousarray(f["B_corner_cur"], np.float64))
        d_J = mem.empty(ncell * 3 * 8)
        d_M = mem.empty(ncell * 243 * 8)
        d_e = mem.empty(8)
        lib = _capi.load()
        for _ in range(2):
            st = lib.amps_gpu_update_j_mass_matrix_noalloc(
                C.byref(ctx.cfg), n, d_start, d_u, d_v, d_sp, d_B, d_J, d_M, d_e, None)
            assert st == 0
            J = mem.get(d_J, np.float64, ncell * 3).reshape(ncell, 3)
            M = mem.get(d_M, np.float64, ncell * 243).reshape(ncell, 243)
            e = mem.get(d_e, np.float64, 1)[0]
            assert G.rel_err(J, J_ref) <= 1e-5, G.rel_err(J, J_ref)
            assert G.rel_err(M, M_ref) <= 1e-5, G.rel_err(M, M_ref)
            assert e == pytest.approx(e_ref, rel=1e-6)
        # a mesh larger than the static scratch is refused
        big = A.electron_proton_plasma("big", 4, 4, 2, 1, 1)
        bctx_cfg = _capi.Config()
        C.memmove(C.byref(bctx_cfg), C.byref(ctx.cfg), C.sizeof(_capi.Config))
        bctx_cfg.nbx, bctx_cfg.nby, bctx_cfg.nbz = big.mesh.nbx, big.mesh.nby, big.mesh.nbz
        assert lib.amps_gpu_update_j_mass_matrix_noalloc(
            C.byref(bctx_cfg), 0, d_start, d_u, d_v, d_sp, d_B, d_J, d_M, d_e, None) == 1
    finally:
        mem.free()
        ctx.close()
