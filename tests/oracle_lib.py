"""ctypes binding of the FP64 oracle (oracle/liboracle.so).

Test infrastructure: only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline use it, always as the checker.
"""
import ctypes as C
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
LIB = os.path.join(ORACLE_DIR, "liboracle.so")


class Mesh(C.Structure):
    _fields_ = [("nbx", C.c_int), ("nby", C.c_int), ("nbz", C.c_int),
                ("x0", C.c_double * 3), ("dx", C.c_double * 3), ("nspec", C.c_int),
                ("q", C.c_double * 8), ("m", C.c_double * 8), ("w", C.c_double * 8),
                ("dt", C.c_double), ("theta", C.c_double)]


class RecordLayout(C.Structure):
    _fields_ = [("len", C.c_int), ("off_v", C.c_int), ("off_x", C.c_int), ("off_sp", C.c_int),
                ("off_w", C.c_int)]


D = C.POINTER(C.c_double)
I32 = C.POINTER(C.c_int32)
U8 = C.POINTER(C.c_uint8)
I64 = C.POINTER(C.c_int64)

_lib = None


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        subprocess.run(["make", "-s", "-C", ORACLE_DIR, "all"], check=True)
    lib = C.CDLL(LIB)
    sig = {
        "orc_laplacian_table": (None, [C.c_int, D]),
        "orc_graddiv_table": (None, [C.c_int, C.c_int, D]),
        "orc_corner_weights": (None, [D, D]),
        "orc_push": (C.c_long, [C.POINTER(Mesh), C.c_long, D, D, U8, I32, I32, D, D]),
        "orc_relboris": (C.c_long, [C.POINTER(Mesh), C.c_long, D, D, U8, I32, I32, D, D,
                                    C.c_double, C.c_double]),
        "orc_boris": (C.c_long, [C.POINTER(Mesh), C.c_long, D, D, U8, I32, I32, D, D, C.c_double]),
        "orc_deposit": (C.c_double, [C.POINTER(Mesh), C.c_long, D, D, U8, D, I32, I32, D, D, D]),
        "orc_locate": (None, [C.POINTER(Mesh), C.c_long, D, I32, I32]),
        "orc_cfl": (None, [C.POINTER(Mesh), C.c_long, D, U8, I32, I32, D]),
        "orc_species_moments": (None, [C.POINTER(Mesh), C.c_long, D, D, U8, D, I32, I32, D]),
        "orc_set_open_axes": (None, [C.c_int]),
        "orc_set_b_center": (None, [C.c_int]),
        "orc_centre_b_at": (None, [C.POINTER(Mesh), C.c_long, D, C.POINTER(C.c_int32), D, D]),
        "orc_inject": (C.c_long, [C.POINTER(Mesh), C.c_int, C.c_int, C.c_double, D, C.c_double,
                                  C.c_ulonglong, C.c_ulonglong, C.c_int, D, D, C.c_long, D, D, I32,
                                  I32]),
        "orc_center_to_corner": (None, [C.POINTER(Mesh), D, D]),
        "orc_rhs": (None, [C.POINTER(Mesh), D, D, D, D, D]),
        "orc_matvec": (None, [C.POINTER(Mesh), D, D, D]),
        "orc_jacobi_diag": (None, [C.POINTER(Mesh), D, D]),
        "orc_gmres": (C.c_int, [C.POINTER(Mesh), D, D, D, C.c_double, C.c_int, C.c_int, C.c_int, D]),
        "orc_update_b": (None, [C.POINTER(Mesh), D, D, D]),
        "orc_update_e": (C.c_double, [C.POINTER(Mesh), D, D, D]),
        "orc_ecsim_step": (C.c_int, [C.POINTER(Mesh), C.c_long, D, D, U8, D, I32, I32, D, D, D, D,
                                     D, D, D, C.c_double, C.c_int, C.c_int, D]),
        "orc_crc32_add": (C.c_uint64, [C.c_uint64, U8, C.c_long]),
        "orc_restart_pack": (C.c_longlong, [C.POINTER(RecordLayout), C.c_int, I32, U8, C.c_int, C.c_int,
                                            D, C.c_long, D, D, U8, D, I32, I32, U8, C.c_longlong]),
        "orc_particle_checksum": (C.c_uint64, [C.POINTER(RecordLayout), C.c_int, I32, C.c_long, D, D,
                                               U8, D, I32, I32]),
        "orc_net_charge": (None, [C.POINTER(Mesh), C.c_long, D, U8, D, I32, D]),
        "orc_div_e": (None, [C.POINTER(Mesh), D, D]),
        "orc_poisson_rhs": (None, [C.POINTER(Mesh), D, D, D, D]),
        "orc_poisson_cg": (C.c_int, [C.POINTER(Mesh), D, D, C.c_double, C.c_int, D]),
        "orc_corner_charge": (None, [C.POINTER(Mesh), C.c_long, D, U8, D, I32, I32, C.c_int, D]),
        "orc_dive_correct": (C.c_long, [C.POINTER(Mesh), C.c_long, D, U8, I32, I32, D, D]),
        "orc_div_e_correction": (None, [C.POINTER(Mesh), C.c_long, D, U8, D, I32, I32, D, D, D, D,
                                        D, C.c_int, C.c_double, C.c_int, D]),
        "orc_dipole_b": (None, [D, C.c_double, C.c_double, D, D]),
        "orc_trace": (C.c_long, [C.c_long, D, D, I32, I64, C.c_double, C.c_double, C.c_double,
                                 C.c_double, D, C.c_double, C.c_double, C.c_long, C.c_double,
                                 C.c_double, C.c_int]),
    }
    for k, (r, a) in sig.items():
        f = getattr(lib, k)
        f.restype = r
        f.argtypes = a
    _lib = lib
    return lib


def p(a, t=C.c_double):
    if a is None:
        return None
    assert a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(t))


def mesh_of(wl):
    m = Mesh()
    m.nbx, m.nby, m.nbz = wl.mesh.nbx, wl.mesh.nby, wl.mesh.nbz
    for d in range(3):
        m.x0[d] = wl.mesh.x0[d]
        m.dx[d] = wl.mesh.dx
    m.nspec = len(wl.species)
    for i, s in enumerate(wl.species):
        m.q[i], m.m[i], m.w[i] = s.charge, s.mass, s.weight
    m.dt, m.theta = wl.dt, wl.theta
    return m


class OracleState:
    """FP64 oracle state for one workload (global periodic corner layout)."""

    def __init__(self, wl, x, v, spec, fields, wcorr=None, b_center=False):
        """b_center: the particles see B interpolated from the cell centres
        (_PIC_FIELD_SOLVER_B_CENTER_BASED_): the push reads Bcen_prev (B^n),
        the deposit Bcen (B^{n+1} after a step; both the imported B_center at
        first)"""
        self.lib = load()
        self.b_center = bool(b_center)
        self.wl = wl
        self.m = mesh_of(wl)
        n = len(spec)
        self.x = np.ascontiguousarray(x, np.float64).copy()
        self.v = np.ascontiguousarray(v, np.float64).copy()
        self.spec = np.ascontiguousarray(spec, np.uint8).copy()
        self.wcorr = None if wcorr is None else np.ascontiguousarray(wcorr, np.float64)
        self.block = np.zeros(n, np.int32)
        self.cell = np.zeros(n, np.int32)
        self.lib.orc_locate(C.byref(self.m), n, p(self.x), p(self.block, C.c_int32),
                            p(self.cell, C.c_int32))
        nc = wl.mesh.ncells
        self.E_n = np.ascontiguousarray(fields["E_n"], np.float64).copy()
        self.E_half = np.ascontiguousarray(fields["E_half"], np.float64).copy()
        self.Bcen = np.ascontiguousarray(fields["B_center"], np.float64).copy()
        self.Bprev = np.ascontiguousarray(fields["B_corner_prev"], np.float64).copy()
        self.Bcur = np.ascontiguousarray(fields["B_corner_cur"], np.float64).copy()
        self.Bcen_prev = self.Bcen.copy()
        self.J = np.zeros((nc, 3))
        self.M = np.zeros((nc, 243))

    def species_moments(self):
        """(ncorners, nspec, 10) corner species moments of the current particles"""
        ns = self.m.nspec
        out = np.zeros((self.wl.mesh.ncells, ns, 10))
        self.lib.orc_species_moments(C.byref(self.m), len(self.spec), p(self.x), p(self.v),
                                     p(self.spec, C.c_uint8), p(self.wcorr),
                                     p(self.block, C.c_int32), p(self.cell, C.c_int32), p(out))
        return out

    def relboris(self, dt_total, c_light=1.0):
        """Mover::Relativistic::Boris on E^n and the corner B cur slot"""
        return self.lib.orc_relboris(C.byref(self.m), len(self.spec), p(self.x), p(self.v),
                                     p(self.spec, C.c_uint8), p(self.block, C.c_int32),
                                     p(self.cell, C.c_int32), p(self.E_n), p(self.Bcur),
                                     dt_total, c_light)

    def boris(self, dt):
        """Mover::Boris on E^n and the corner B cur slot; returns the number of
        particles deleted at open faces"""
        return self.lib.orc_boris(C.byref(self.m), len(self.spec), p(self.x), p(self.v),
                                  p(self.spec, C.c_uint8), p(self.block, C.c_int32),
                                  p(self.cell, C.c_int32), p(self.E_n), p(self.Bcur), dt)

    def _with_b_mode(self, call):
        self.lib.orc_set_b_center(1 if self.b_center else 0)
        try:
            return call()
        finally:
            self.lib.orc_set_b_center(0)

    def push(self):
        B = self.Bcen_prev if self.b_center else self.Bprev
        return self._with_b_mode(lambda: self.lib.orc_push(
            C.byref(self.m), len(self.spec), p(self.x), p(self.v), p(self.spec, C.c_uint8),
            p(self.block, C.c_int32), p(self.cell, C.c_int32), p(self.E_half), p(B)))

    def deposit(self):
        B = self.Bcen if self.b_center else self.Bcur
        return self._with_b_mode(lambda: self.lib.orc_deposit(
            C.byref(self.m), len(self.spec), p(self.x), p(self.v), p(self.spec, C.c_uint8),
            p(self.wcorr), p(self.block, C.c_int32), p(self.cell, C.c_int32), p(B), p(self.J),
            p(self.M)))

    def div_e_correction(self, tol=1e-8, maxit=500):
        """ECSIM::divECorrection on the oracle's particles and E^n (its corner
        E^{n+1} after a step): net charge, div E, the Poisson solve, the
        species-0 position correction and re-binning.  The densities persist
        between calls.  Returns the statistics of orc_div_e_correction."""
        nc = self.wl.mesh.ncells
        first = not hasattr(self, "rho_new")
        if first:
            self.rho_new = np.zeros(nc)
            self.rho_old = np.zeros(nc)
            self.div_e = np.zeros(nc)
            self.phi = np.zeros(nc)
        st = np.zeros(5)
        self.lib.orc_div_e_correction(C.byref(self.m), len(self.spec), p(self.x),
                                      p(self.spec, C.c_uint8), p(self.wcorr),
                                      p(self.block, C.c_int32), p(self.cell, C.c_int32),
                                      p(self.E_n), p(self.rho_new), p(self.rho_old), p(self.div_e),
                                      p(self.phi), 1 if first else 0, tol, maxit, p(st))
        return {"iterations": int(st[0]), "rel_residual": st[1], "gauss_before": st[2],
                "gauss_after": st[3], "moved": int(st[4])}

    def cfl(self):
        """per-species maximum over cells of ProcessCell's cflCell"""
        out = np.zeros(self.m.nspec)
        self.lib.orc_cfl(C.byref(self.m), len(self.spec), p(self.v), p(self.spec, C.c_uint8),
                         p(self.block, C.c_int32), p(self.cell, C.c_int32), p(out))
        return out

    def step(self, tol=1e-8, maxit=200, precond=0):
        diag = np.zeros(3)
        prev = self.Bcen.copy()
        it = self._with_b_mode(lambda: self.lib.orc_ecsim_step(
            C.byref(self.m), len(self.spec), p(self.x), p(self.v), p(self.spec, C.c_uint8),
            p(self.wcorr), p(self.block, C.c_int32), p(self.cell, C.c_int32), p(self.E_n),
            p(self.E_half), p(self.Bcen), p(self.Bprev), p(self.Bcur), p(self.J), p(self.M), tol,
            maxit, precond, p(diag)))
        self.Bcen_prev = prev
        return it, diag

    def rhs(self):
        out = np.zeros_like(self.E_n)
        self.lib.orc_rhs(C.byref(self.m), p(self.E_n), p(self.Bcen), p(self.J), p(self.M), p(out))
        return out

    def matvec(self, x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros_like(x)
        self.lib.orc_matvec(C.byref(self.m), p(self.M), p(x), p(y))
        return y


def trace(x, pm, q, m0, b_eq, r_e, b_ext, r_in, r_out, max_steps, dphi, dt_max):
    lib = load()
    n = len(x)
    x = np.ascontiguousarray(x, np.float64).copy()
    pm = np.ascontiguousarray(pm, np.float64).copy()
    st = np.zeros(n, np.int32)
    steps = np.zeros(n, np.int64)
    ext = np.ascontiguousarray(b_ext, np.float64)
    tot = lib.orc_trace(n, p(x), p(pm), p(st, C.c_int32), p(steps, C.c_int64), q, m0, b_eq, r_e,
                        p(ext), r_in, r_out, max_steps, dphi, dt_max, 0)
    return x, pm, st, steps, tot


def crc32_add(acc, data):
    """the reference's CRC32::add over bytes, from accumulator acc (64-bit)"""
    b = np.ascontiguousarray(np.frombuffer(bytes(data), np.uint8))
    return int(load().orc_crc32_add(acc, p(b, C.c_uint8), b.size))


def _layout(layout):
    return RecordLayout(layout.record_length, layout.off_velocity, layout.off_position,
                        layout.off_species, layout.off_weight)


def restart_pack(layout, nb, x, v, spec, block, cell, weight, wcorr=None, block_order=None,
                 node_ids=None):
    """particle section bytes; particles in an order that keeps each cell's list order"""
    lib = load()
    L = _layout(layout)
    x = np.ascontiguousarray(x, np.float64); v = np.ascontiguousarray(v, np.float64)
    spec = np.ascontiguousarray(spec, np.uint8)
    block = np.ascontiguousarray(block, np.int32); cell = np.ascontiguousarray(cell, np.int32)
    wc = None if wcorr is None else np.ascontiguousarray(wcorr, np.float64)
    bo = None if block_order is None else np.ascontiguousarray(block_order, np.int32)
    if node_ids is None:
        node_ids = np.arange(nb, dtype=np.int64).view(np.uint8).reshape(nb, 8)
    ids = np.ascontiguousarray(node_ids, np.uint8)
    w = np.ascontiguousarray(weight, np.float64)
    args = (C.byref(L), nb, p(bo, C.c_int32), p(ids, C.c_uint8), ids.shape[1], w.size, p(w),
            x.shape[0], p(x), p(v), p(spec, C.c_uint8), p(wc), p(block, C.c_int32), p(cell, C.c_int32))
    size = lib.orc_restart_pack(*args, None, 0)
    out = np.zeros(size, np.uint8)
    assert lib.orc_restart_pack(*args, p(out, C.c_uint8), size) == size
    return out


def particle_checksum(layout, nb, x, v, spec, block, cell, wcorr=None, block_order=None):
    lib = load()
    L = _layout(layout)
    x = np.ascontiguousarray(x, np.float64); v = np.ascontiguousarray(v, np.float64)
    spec = np.ascontiguousarray(spec, np.uint8)
    block = np.ascontiguousarray(block, np.int32); cell = np.ascontiguousarray(cell, np.int32)
    wc = None if wcorr is None else np.ascontiguousarray(wcorr, np.float64)
    bo = None if block_order is None else np.ascontiguousarray(block_order, np.int32)
    return int(lib.orc_particle_checksum(C.byref(L), nb, p(bo, C.c_int32), x.shape[0], p(x), p(v),
                                         p(spec, C.c_uint8), p(wc), p(block, C.c_int32),
                                         p(cell, C.c_int32)))
