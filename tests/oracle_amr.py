"""ctypes binding of the FP64 AMR oracle (oracle/amps_oracle_amr.c).  Test
infrastructure: only tests/, smoke() and bench.py's CPU baseline use it."""
import ctypes as C

import numpy as np

from tests import oracle_lib as OL

D = C.POINTER(C.c_double)
I32 = C.POINTER(C.c_int32)
U8 = C.POINTER(C.c_uint8)


class Amr(C.Structure):
    _fields_ = [("nblocks", C.c_int), ("ncorners", C.c_int), ("lmax", C.c_int),
                ("nfine", C.c_int * 3), ("x0", C.c_double * 3), ("dx0", C.c_double),
                ("level", I32), ("origin", I32), ("corner_tab", I32), ("hang_start", I32),
                ("hang_parent", I32), ("hang_weight", D), ("fine_map", I32),
                ("nspec", C.c_int), ("q", C.c_double * 8), ("m", C.c_double * 8),
                ("w", C.c_double * 8), ("dt", C.c_double), ("theta", C.c_double),
                ("bnd_flag", I32), ("bnd_start", I32), ("bnd_col", I32), ("bnd_weight", D),
                ("open_mask", C.c_int), ("field_bc", C.c_int)]


_bound = False


def lib():
    global _bound
    L = OL.load()
    if not _bound:
        sig = {
            "orc_amr_locate": (None, [C.POINTER(Amr), C.c_long, D, I32, I32]),
            "orc_amr_push": (C.c_long, [C.POINTER(Amr), C.c_long, D, D, U8, I32, I32, D, D]),
            "orc_amr_relboris": (C.c_long, [C.POINTER(Amr), C.c_long, D, D, U8, I32, I32, D, D,
                                            C.c_double, C.c_double]),
            "orc_amr_boris": (C.c_long, [C.POINTER(Amr), C.c_long, D, D, U8, I32, I32, D, D,
                                         C.c_double]),
            "orc_amr_push_deposit_mt": (C.c_double, [C.POINTER(Amr), C.c_long, D, D, U8, D, I32,
                                                     I32, D, D, D, D, D, C.c_int, U8]),
            "orc_amr_deposit": (C.c_double, [C.POINTER(Amr), C.c_long, D, D, U8, D, I32, I32, D,
                                             D, D]),
            "orc_amr_apply": (None, [C.POINTER(Amr), D, D, D, C.c_int, C.c_int, C.c_int]),
            "orc_amr_species_moments": (None, [C.POINTER(Amr), C.c_long, D, D, U8, D, I32, D]),
            "orc_amr_rhs": (None, [C.POINTER(Amr), D, D, D, D, D]),
            "orc_amr_gmres": (C.c_int, [C.POINTER(Amr), D, D, D, C.c_double, C.c_int, C.c_int, D]),
            "orc_amr_update_b": (None, [C.POINTER(Amr), D, D, D]),
            "orc_amr_c2n": (None, [C.POINTER(Amr), D, D]),
            "orc_amr_update_e": (C.c_double, [C.POINTER(Amr), D, D, D]),
            "orc_amr_step": (C.c_int, [C.POINTER(Amr), C.c_long, D, D, U8, D, I32, I32, D, D, D,
                                       D, D, D, D, C.c_double, C.c_int, D]),
            "orc_amr_inject": (C.c_long, [C.POINTER(Amr), C.c_int, C.c_int, C.c_double, D, C.c_double,
                                          C.c_ulonglong, C.c_ulonglong, C.c_int, D, D, C.c_long, D, D,
                                          I32, I32]),
        }
        for k, (r, a) in sig.items():
            f = getattr(L, k)
            f.restype = r
            f.argtypes = a
        _bound = True
    return L


def p(a, t=C.c_double):
    return OL.p(a, t)


class AmrOracle:
    """FP64 oracle state on an AmrMesh (global corner numbering = the mesh's
    unique corner ids, cells = block*512 + local)."""

    def __init__(self, mesh, species, dt, theta, x, v, spec, wcorr=None):
        self.L = lib()
        self.mesh = mesh
        g = Amr()
        g.nblocks, g.ncorners, g.lmax = mesh.nblocks, mesh.ncorners, mesh.lmax
        for d in range(3):
            g.nfine[d] = mesh.nfine[d]
            g.x0[d] = mesh.x0[d]
        g.dx0 = mesh.dx0
        self._keep = [np.ascontiguousarray(mesh.level, np.int32),
                      np.ascontiguousarray(mesh.origin, np.int32).ravel()]
        g.level = p(self._keep[0], C.c_int32)
        g.origin = p(self._keep[1], C.c_int32)
        g.corner_tab = p(mesh.corner_tab, C.c_int32)
        g.hang_start = p(mesh.hang_start, C.c_int32)
        g.hang_parent = p(mesh.hang_parent, C.c_int32)
        g.hang_weight = p(mesh.hang_weight)
        g.fine_map = p(mesh.fine_map, C.c_int32)
        g.nspec = len(species)
        for i, s in enumerate(species):
            g.q[i], g.m[i], g.w[i] = s.charge, s.mass, s.weight
        g.dt, g.theta = dt, theta
        # open axes: boundary rows and UpdateB's boundary branch
        mask = sum(1 << d for d in range(3) if getattr(mesh, "open_axes", (False,) * 3)[d])
        g.open_mask = mask
        g.field_bc = getattr(mesh, "neumann_mask", 0)
        if mask:
            g.bnd_flag = p(mesh.bnd_flag, C.c_int32)
            g.bnd_start = p(mesh.bnd_start, C.c_int32)
            g.bnd_col = p(mesh.bnd_col, C.c_int32)
            g.bnd_weight = p(mesh.bnd_weight)
        self.g = g
        n = len(spec)
        self.x = np.ascontiguousarray(x, np.float64).copy()
        self.v = np.ascontiguousarray(v, np.float64).copy()
        self.spec = np.ascontiguousarray(spec, np.uint8).copy()
        self.wcorr = None if wcorr is None else np.ascontiguousarray(wcorr, np.float64)
        self.block = np.zeros(n, np.int32)
        self.cell = np.zeros(n, np.int32)
        self.L.orc_amr_locate(C.byref(g), n, p(self.x), p(self.block, C.c_int32),
                              p(self.cell, C.c_int32))
        nc, ncell = mesh.ncorners, mesh.ncells
        self.E_n = np.zeros((nc, 3))
        self.E_half = np.zeros((nc, 3))
        self.Bcen = np.zeros((ncell, 3))
        self.Bprev = np.zeros((nc, 3))
        self.Bcur = np.zeros((nc, 3))
        self.cellJ = np.zeros(ncell * 24)
        self.cellM = np.zeros(ncell * 324)

    def deposit(self):
        return self.L.orc_amr_deposit(C.byref(self.g), len(self.spec), p(self.x), p(self.v),
                                      p(self.spec, C.c_uint8), p(self.wcorr),
                                      p(self.block, C.c_int32), p(self.cell, C.c_int32),
                                      p(self.Bcur), p(self.cellJ), p(self.cellM))

    def push_deposit_mt(self, nthreads, sel=None):
        """push then deposit on nthreads host threads (same per-cell results as
        push() followed by deposit()); sel (uint8 per block, optional): deposit
        only the blocks with sel != 0, leave the others' partials untouched.
        Returns the kinetic energy."""
        if sel is not None:
            sel = np.ascontiguousarray(sel, np.uint8)
            assert sel.shape == (self.mesh.nblocks,)
        return self.L.orc_amr_push_deposit_mt(
            C.byref(self.g), len(self.spec), p(self.x), p(self.v), p(self.spec, C.c_uint8),
            p(self.wcorr), p(self.block, C.c_int32), p(self.cell, C.c_int32), p(self.E_half),
            p(self.Bprev), p(self.Bcur), p(self.cellJ), p(self.cellM), nthreads,
            p(sel, C.c_uint8))

    def species_moments(self):
        """(ncorners, nspec, 10) corner species moments of the current particles"""
        out = np.zeros((self.mesh.ncorners, self.g.nspec, 10))
        self.L.orc_amr_species_moments(C.byref(self.g), len(self.spec), p(self.x), p(self.v),
                                       p(self.spec, C.c_uint8), p(self.wcorr),
                                       p(self.block, C.c_int32), p(out))
        return out

    def push(self):
        return self.L.orc_amr_push(C.byref(self.g), len(self.spec), p(self.x), p(self.v),
                                   p(self.spec, C.c_uint8), p(self.block, C.c_int32),
                                   p(self.cell, C.c_int32), p(self.E_half), p(self.Bprev))

    def relboris(self, dt_total, c_light=1.0):
        """Mover::Relativistic::Boris with E^n and the corner B "cur" slot;
        returns the number of sub-steps"""
        return self.L.orc_amr_relboris(C.byref(self.g), len(self.spec), p(self.x), p(self.v),
                                       p(self.spec, C.c_uint8), p(self.block, C.c_int32),
                                       p(self.cell, C.c_int32), p(self.E_n), p(self.Bcur),
                                       dt_total, c_light)

    def boris(self, dt):
        """Mover::Boris with E^n and the corner B "cur" slot; returns the
        number of particles deleted at open faces"""
        return self.L.orc_amr_boris(C.byref(self.g), len(self.spec), p(self.x), p(self.v),
                                    p(self.spec, C.c_uint8), p(self.block, C.c_int32),
                                    p(self.cell, C.c_int32), p(self.E_n), p(self.Bcur), dt)

    def apply(self, x, identity=1, curl=1, mass=1):
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros_like(x)
        self.L.orc_amr_apply(C.byref(self.g), p(self.cellM), p(x), p(y), identity, curl, mass)
        return y

    def c2n(self):
        self.L.orc_amr_c2n(C.byref(self.g), p(self.Bcen), p(self.Bcur))
        self.Bprev[:] = self.Bcur

    def step(self, tol=1e-10, maxit=400):
        diag = np.zeros(3)
        it = self.L.orc_amr_step(C.byref(self.g), len(self.spec), p(self.x), p(self.v),
                                 p(self.spec, C.c_uint8), p(self.wcorr), p(self.block, C.c_int32),
                                 p(self.cell, C.c_int32), p(self.E_n), p(self.E_half),
                                 p(self.Bcen), p(self.Bprev), p(self.Bcur), p(self.cellJ),
                                 p(self.cellM), tol, maxit, p(diag))
        return it, diag

    def field_solve(self, tol=1e-10, maxit=400):
        """ECSIM field solve from the current cellJ/cellM (rhs, GMRES, E^{n+theta},
        UpdateB, corner B prev <- cur, C2N, UpdateE).  Returns (iterations, wave energy)."""
        g = C.byref(self.g)
        rhs = np.zeros_like(self.E_n)
        self.L.orc_amr_rhs(g, p(self.E_n), p(self.Bcen), p(self.cellJ), p(self.cellM), p(rhs))
        dE = np.zeros_like(self.E_n)
        res = np.zeros(1)
        it = self.L.orc_amr_gmres(g, p(self.cellM), p(rhs), p(dE), tol, maxit, 30, p(res))
        self.E_half[:] = self.E_n + dE
        bnew = np.zeros_like(self.Bcen)
        self.L.orc_amr_update_b(g, p(self.E_half), p(self.Bcen), p(bnew))
        self.Bcen[:] = bnew
        self.Bprev[:] = self.Bcur
        self.L.orc_amr_c2n(g, p(self.Bcen), p(self.Bcur))
        wave = self.L.orc_amr_update_e(g, p(self.E_half), p(self.E_n), p(self.Bcen))
        return it, wave

    def wave_energy(self):
        """sum_cells V (sum_corners |E|^2/8 + |B|^2)/(8 pi) of the current state"""
        tmp = self.E_n.copy()
        # update_e with E_half = E_n leaves E_n unchanged (theta-weighted identity)
        return self.L.orc_amr_update_e(C.byref(self.g), p(self.E_n.copy()), p(tmp), p(self.Bcen))
