"""Block-structured AMR meshes (host side, over the C ABI's amps_amr_* builder).

A mesh is a list of leaf blocks of 8^3 cells; a leaf at level L has cell size
dx0 / 2^L and an origin on the finest lattice.  AmrMesh holds the tables the
builder derives: block -> unique corner maps, hanging-corner constraints and
the finest-block -> leaf map (the reference's findTreeNode,
src/meshAMR/meshAMRgeneric.h:2793-2885).
"""
import ctypes as C

import numpy as np

from . import _capi
from ._capi import AmpsGpuError, ptr


class BlockDesc(C.Structure):
    _fields_ = [("level", C.c_int), ("ix", C.c_int), ("iy", C.c_int), ("iz", C.c_int)]


def nested_leaves(nb0, lmax, mode, frac):
    """Leaves of a nested refinement (mode 0: central box of relative half-width
    frac/2, mode 1: central sphere of relative radius frac; halved per level)."""
    lib = _capi.load_host()
    n = lib.amps_amr_nested_leaves(nb0[0], nb0[1], nb0[2], lmax, mode, frac, None, 0)
    if n < 0:
        raise AmpsGpuError(-n, "amps_amr_nested_leaves")
    arr = (BlockDesc * n)()
    lib.amps_amr_nested_leaves(nb0[0], nb0[1], nb0[2], lmax, mode, frac, C.cast(arr, C.c_void_p), n)
    return np.array([(b.level, b.ix, b.iy, b.iz) for b in arr], np.int32).reshape(-1, 4)


class AmrMesh:
    """open_axes: per axis, non-periodic (the domain faces carry the field
    boundary condition field_bc -- 0 Dirichlet, 1 Neumann, one value for every
    face or six, one per face in the order -x, +x, -y, +y, -z, +z -- and delete
    particles)"""

    def __init__(self, nb0, lmax, leaves, dx0=1.0, x0=(0.0, 0.0, 0.0), open_axes=(False, False, False),
                 field_bc=0):
        self.lib = _capi.load_host()
        self.nb0 = tuple(int(v) for v in nb0)
        self.lmax = int(lmax)
        self.dx0 = float(dx0)
        self.x0 = tuple(float(v) for v in x0)
        leaves = np.ascontiguousarray(leaves, np.int32).reshape(-1, 4)
        self.leaves = leaves
        descs = (BlockDesc * len(leaves))(*[BlockDesc(*map(int, r)) for r in leaves])
        h = C.c_void_p()
        x0a = np.array(self.x0, np.float64)
        self.open_axes = tuple(bool(v) for v in open_axes)
        faces = [int(field_bc)] * 6 if np.isscalar(field_bc) else [int(v) for v in field_bc]
        assert len(faces) == 6
        self.field_bc = field_bc
        self.face_bc = tuple(faces)
        self.neumann_mask = sum(1 << f for f in range(6) if self.open_axes[f // 2] and faces[f] == 1)
        op = (C.c_int * 3)(*[1 if v else 0 for v in self.open_axes])
        fb = (C.c_int * 6)(*faces)
        st = self.lib.amps_amr_build_open_faces(self.nb0[0], self.nb0[1], self.nb0[2], self.lmax,
                                                ptr(x0a, C.c_double), self.dx0,
                                                C.cast(descs, C.c_void_p), len(leaves), op, fb,
                                                C.byref(h))
        if st != 0:
            raise AmpsGpuError(st, "amps_amr_build")
        self.h = h
        nb, nc, nh, npar = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        nf = (C.c_int * 3)()
        self.lib.amps_amr_info(h, C.byref(nb), C.byref(nc), C.byref(nh), C.byref(npar), nf)
        self.nblocks, self.ncorners, self.nhanging = nb.value, nc.value, nh.value
        self.nfine = tuple(nf)
        self.corner_tab = np.zeros(self.nblocks * 729, np.int32)
        self.corner_xyz = np.zeros(self.ncorners * 3, np.int32)
        self.hang_start = np.zeros(self.ncorners + 1, np.int32)
        self.hang_parent = np.zeros(max(npar.value, 1), np.int32)
        self.hang_weight = np.zeros(max(npar.value, 1), np.float64)
        nfb = (self.nfine[0] // 8) * (self.nfine[1] // 8) * (self.nfine[2] // 8)
        self.fine_map = np.zeros(nfb, np.int32)
        self.lib.amps_amr_tables(h, ptr(self.corner_tab, C.c_int32), ptr(self.corner_xyz, C.c_int32),
                                 ptr(self.hang_start, C.c_int32), ptr(self.hang_parent, C.c_int32),
                                 ptr(self.hang_weight, C.c_double), ptr(self.fine_map, C.c_int32))
        self.level = np.ascontiguousarray(leaves[:, 0])
        self.origin = np.ascontiguousarray(leaves[:, 1:4])
        ne = C.c_int()
        self.lib.amps_amr_boundary_tables(h, C.byref(ne), None, None, None, None)
        self.bnd_flag = np.zeros(self.ncorners, np.int32)
        self.bnd_start = np.zeros(self.ncorners + 1, np.int32)
        self.bnd_col = np.zeros(max(ne.value, 1), np.int32)
        self.bnd_weight = np.zeros(max(ne.value, 1), np.float64)
        self.lib.amps_amr_boundary_tables(h, C.byref(ne), ptr(self.bnd_flag, C.c_int32),
                                          ptr(self.bnd_start, C.c_int32), ptr(self.bnd_col, C.c_int32),
                                          ptr(self.bnd_weight, C.c_double))

    @property
    def ncells(self):
        return self.nblocks * 512

    @property
    def dxf(self):
        return self.dx0 / (1 << self.lmax)

    def block_dx(self):
        return self.dx0 / (2.0 ** self.level)

    def block_origins(self):
        return np.array(self.x0) + self.origin * self.dxf

    def close(self):
        if getattr(self, "h", None):
            self.lib.amps_amr_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def uniform_mesh(nb0, dx0=1.0):
    """Single-level mesh of nb0 blocks per axis."""
    leaves = [(0, 8 * i, 8 * j, 8 * k) for k in range(nb0[2]) for j in range(nb0[1])
              for i in range(nb0[0])]
    return AmrMesh(nb0, 0, np.array(leaves, np.int32), dx0)


def central_refined_mesh(nb0, lmax=1, frac=0.5, dx0=1.0):
    """Base blocks with the central box (relative half-width frac/2) refined,
    the mesh of the AMR plasma workload."""
    return AmrMesh(nb0, lmax, nested_leaves(nb0, lmax, 0, frac), dx0)


def sphere_refined_mesh(nb0, lmax, radius=0.2, dx0=1.0):
    return AmrMesh(nb0, lmax, nested_leaves(nb0, lmax, 1, radius), dx0)


def amr_initial_condition(mesh, species, ppc_base, seed=100, nthreads=1, per_cell=False):
    """Uniform-density Maxwellian plasma on an AMR mesh, positions uniform within
    each cell, co-located species, reference LCG stream split per block.

    per_cell False: ppc_base particles per species per level-0 cell volume (a
    cell at level L holds ppc_base/8^L), all of weight 1.  per_cell True:
    ppc_base particles per species in every cell, a level-L particle carrying
    the weight correction 8^-L (the same density with equal statistics per
    cell).  Returns u (FP32 block-local cell units), v, spec, block, all
    FP32-representable, and wcorr (FP32, or None for per_cell False).  Blocks
    are generated on nthreads host threads (the result does not depend on it)."""
    ns = len(species)
    vth = np.array([s.vth for s in species], np.float64)
    lib = _capi.load_host()

    def block_ppc(b):
        return ppc_base if per_cell else max(1, ppc_base // (8 ** int(mesh.level[b])))

    counts = [lib.amps_ic_count(1, 1, 1, block_ppc(b), ns) for b in range(mesh.nblocks)]
    off = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    n = int(off[-1])
    u = np.empty((n, 3), np.float32)
    v = np.empty((n, 3), np.float32)
    sp = np.empty(n, np.uint8)
    bl = np.empty(n, np.int32)
    scratch = np.empty(n, np.int32)

    wc = np.empty(n, np.float32) if per_cell else None

    def one(b):
        ppc = block_ppc(b)
        a, e = int(off[b]), int(off[b + 1])
        st = lib.amps_ic_maxwellian(1, 1, 1, ppc, ns, ptr(vth, C.c_double),
                                    (seed * 7919 + 104729 * (b + 1)) & 0x7FFFFFFF or 1, 1,
                                    ptr(u[a:e], C.c_float), ptr(v[a:e], C.c_float),
                                    ptr(sp[a:e], C.c_uint8), ptr(scratch[a:e], C.c_int32))
        if st != 0:
            raise AmpsGpuError(st, "amps_ic_maxwellian")
        bl[a:e] = b
        if per_cell:
            wc[a:e] = 0.125 ** int(mesh.level[b])

    if nthreads > 1:
        from concurrent.futures import ThreadPoolExecutor
        with ThreadPoolExecutor(max_workers=nthreads) as ex:
            list(ex.map(one, range(mesh.nblocks)))
    else:
        for b in range(mesh.nblocks):
            one(b)
    return {"u": u, "v": v, "spec": sp, "block": bl, "wcorr": wc}


def amr_initial_fields(mesh, b0):
    """E = 0, B = b0 on every cell and corner (mesh numbering)."""
    nc, ncell = mesh.ncorners, mesh.ncells
    bc = np.tile(np.asarray(b0, np.float64), (nc, 1))
    return {"E_n": np.zeros((nc, 3)), "E_half": np.zeros((nc, 3)),
            "B_center": np.tile(np.asarray(b0, np.float64), (ncell, 1)),
            "B_corner_prev": bc, "B_corner_cur": bc.copy()}


class AmrWorkload:
    """Electron-proton plasma of the uniform workloads on an AMR mesh: the mesh
    recipe (level-0 blocks, levels, refined region) and ppc_base particles per
    species per level-0 cell volume (per_cell False) or in every cell with
    weight corrections 8^-L (per_cell True)."""

    def __init__(self, name, nb0, lmax, mode, frac, ppc_base, steps=10, per_cell=False):
        from .ecsim import electron_proton_plasma
        self.name = name
        self.nb0, self.lmax, self.mode, self.frac = tuple(nb0), lmax, mode, frac
        self.ppc = ppc_base
        self.per_cell = per_cell
        # species, dt, theta, b0 and tolerance: the uniform plasma (dx0 = 1)
        self.plasma = electron_proton_plasma(name, 1, 1, 1, ppc_base, steps)
        self.species, self.dt, self.theta = self.plasma.species, self.plasma.dt, self.plasma.theta
        self.b0, self.tol = self.plasma.b0, self.plasma.tol

    def mesh(self):
        return AmrMesh(self.nb0, self.lmax, nested_leaves(self.nb0, self.lmax, self.mode, self.frac))

    def initial_condition(self, mesh, seed=100, nthreads=1):
        return amr_initial_condition(mesh, self.species, self.ppc, seed=seed, nthreads=nthreads,
                                     per_cell=self.per_cell)


AMR_WORKLOADS = {
    # 64^3 base cells in 8^3 blocks, central 1/8 of the volume refined 2x,
    # 128 particles per species per base cell (67,108,864 particles)
    "amr_64c_128ppc": lambda: AmrWorkload("amr_64c_128ppc", (8, 8, 8), 1, 0, 0.5, 128),
    # the same recipe at 32^3 base cells and 16 ppc (small case: tests)
    "amr_32c_16ppc": lambda: AmrWorkload("amr_32c_16ppc", (4, 4, 4), 1, 0, 0.5, 16),
    # the 64^3 mesh at 32 ppc (16.8M particles, 0.8 GB of particle state: larger
    # than L2, small enough for full profiler captures)
    "amr_64c_32ppc": lambda: AmrWorkload("amr_64c_32ppc", (8, 8, 8), 1, 0, 0.5, 32),
    # three levels, 256^3 effective cells: level 2 inside a central sphere of
    # radius 0.3 box lengths, level 1 inside radius 0.6 (8912 blocks, 4.56M
    # cells); 64 particles per species in every cell, weight corrections 8^-L
    # (584,056,832 particles)
    "amr_256e_3lvl": lambda: AmrWorkload("amr_256e_3lvl", (8, 8, 8), 2, 1, 0.6, 64, per_cell=True),
    # level 2 inside radius 0.2, level 1 inside 0.4 (4432 blocks, 2.27M cells,
    # 290,455,168 particles)
    "amr_256e_3lvl_r02": lambda: AmrWorkload("amr_256e_3lvl_r02", (8, 8, 8), 2, 1, 0.4, 64,
                                             per_cell=True),
    # the radius-0.2 mesh at 64 particles per species per base-cell volume (8
    # per level-1 cell, 1 per level-2 cell; 33.5M particles)
    "amr_256e_3lvl_sparse": lambda: AmrWorkload("amr_256e_3lvl_sparse", (8, 8, 8), 2, 1, 0.4, 64),
}
