"""Host-side mirror of the reference call surfaces over the C ABI.

``EcsimContext`` groups the calls an AMPS run makes on this path:

    ParticleBuffer   import / export of particle state  (src/pic/pic.h:2716-3846)
    MoveParticles    PIC::Mover::MoveParticles + Lapenta2017 (src/pic/pic_mover.cpp:580)
    UpdateJMassMatrix ECSIM::UpdateJMassMatrix         (pic_field_solver_ecsim.cpp:3244)
    TimeStep         ECSIM::TimeStep (field solve)      (pic_field_solver_ecsim.cpp:6179)
    PicTimeStep      PIC::TimeStep's ECSIM track        (src/pic/pic_time_step.cpp:403)

Errors follow the C ABI: every failing call raises ``AmpsGpuError`` carrying the
status (the reference aborts instead).
"""
import ctypes as C
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import _capi
from ._capi import AmpsGpuError, ptr


@dataclass
class Species:
    name: str
    charge: float   # normalised charge (picunits::si2no_q)
    mass: float     # normalised mass (picunits::si2no_m)
    weight: float   # macro-particle weight
    vth: float      # thermal speed for the Maxwellian initial condition


@dataclass
class PeriodicMesh:
    """Periodic box of nbx*nby*nbz blocks of 8^3 cells."""
    nbx: int
    nby: int
    nbz: int
    dx: float = 1.0
    x0: tuple = (0.0, 0.0, 0.0)

    @property
    def ncells(self):
        return 512 * self.nbx * self.nby * self.nbz

    @property
    def nblocks(self):
        return self.nbx * self.nby * self.nbz

    @property
    def shape(self):
        return (8 * self.nbx, 8 * self.nby, 8 * self.nbz)


@dataclass
class Workload:
    """One ECSIM plasma workload in the reference's normalised units
    (c = 1, lengths in d_e = c/omega_pe, times in 1/omega_pe)."""
    name: str
    mesh: PeriodicMesh
    species: List[Species]
    ppc: int          # particles per cell per species
    dt: float
    theta: float = 0.5
    b0: tuple = (0.0, 0.0, 0.0)
    steps: int = 10
    tol: float = 1e-8
    seed: int = 100

    @property
    def nparticles(self):
        return self.mesh.ncells * self.ppc * len(self.species)


def electron_proton_plasma(name, nbx, nby, nbz, ppc, steps, mass_ratio=25.0, vth_e=0.05,
                           wpe_over_wce=2.0, dt=0.1, dx=1.0):
    """Two-species plasma of the ECSIM workloads: electrons and protons with
    mass ratio 25 (the H_PLUS / 25thELECTRON pair of input/species.input),
    omega_pe = 1 (so dx = 1 is one electron inertial length), T_i = T_e,
    uniform B0 along z with omega_pe/omega_ce = wpe_over_wce."""
    # omega_pe^2 = 4 pi n q^2 / m with n = ppc * w / dx^3, q = -1, m = 1
    w = dx ** 3 / (4.0 * np.pi * ppc)
    vth_i = vth_e / np.sqrt(mass_ratio)
    sp = [Species("electron", -1.0, 1.0, w, vth_e),
          Species("proton", 1.0, mass_ratio, w, vth_i)]
    b0 = (0.0, 0.0, 1.0 / wpe_over_wce)  # omega_ce = |q| B / (m c) = B for electrons
    return Workload(name, PeriodicMesh(nbx, nby, nbz, dx), sp, ppc, dt, 0.5, b0, steps)


WORKLOADS = {
    # 32^3 cells as 4^3 blocks, 64 ppc/species, 10 steps (4,194,304 particles)
    "ecsim_32c_64ppc": lambda: electron_proton_plasma("ecsim_32c_64ppc", 4, 4, 4, 64, 10),
    # 64^3 cells as 8^3 blocks, 128 ppc/species (67,108,864 particles)
    "ecsim_64c_128ppc": lambda: electron_proton_plasma("ecsim_64c_128ppc", 8, 8, 8, 128, 100),
    # 40^3 cells, 64 ppc/species (8,192,000 particles, 205 MB of particle state:
    # larger than the 129 MB L2, small enough for full ncu captures)
    "ecsim_40c_64ppc": lambda: electron_proton_plasma("ecsim_40c_64ppc", 5, 5, 5, 64, 10),
    # small cases for tests
    "ecsim_16c_8ppc": lambda: electron_proton_plasma("ecsim_16c_8ppc", 2, 2, 2, 8, 3),
    "ecsim_8c_4ppc": lambda: electron_proton_plasma("ecsim_8c_4ppc", 1, 1, 1, 4, 2),
}


def make_initial_condition(wl: Workload, nthreads: int = 8):
    """Maxwellian particles (FP32-representable) from the reference LCG.
    Returns dict with u (n,3) float32 cell-unit offsets, v (n,3) float32,
    spec (n,) uint8, block (n,) int32 and x (n,3) float64 physical."""
    lib = _capi.load_host()
    m = wl.mesh
    ns = len(wl.species)
    n = lib.amps_ic_count(m.nbx, m.nby, m.nbz, wl.ppc, ns)
    u = np.empty((n, 3), np.float32)
    v = np.empty((n, 3), np.float32)
    spec = np.empty(n, np.uint8)
    block = np.empty(n, np.int32)
    vth = np.array([s.vth for s in wl.species], np.float64)
    st = lib.amps_ic_maxwellian(m.nbx, m.nby, m.nbz, wl.ppc, ns, ptr(vth, C.c_double),
                                wl.seed, nthreads, ptr(u, C.c_float), ptr(v, C.c_float),
                                ptr(spec, C.c_uint8), ptr(block, C.c_int32))
    if st != 0:
        raise AmpsGpuError(st, "amps_ic_maxwellian")
    return {"u": u, "v": v, "spec": spec, "block": block}


def block_origins(mesh: PeriodicMesh, block):
    bx = block % mesh.nbx
    by = (block // mesh.nbx) % mesh.nby
    bz = block // (mesh.nbx * mesh.nby)
    L = 8.0 * mesh.dx
    return np.stack([mesh.x0[0] + bx * L, mesh.x0[1] + by * L, mesh.x0[2] + bz * L], axis=1)


def physical_positions(mesh: PeriodicMesh, u, block):
    return block_origins(mesh, block) + u.astype(np.float64) * mesh.dx


def initial_fields(wl: Workload):
    """E = 0, uniform B0 on cells and corners (both corner slots)."""
    nc = wl.mesh.ncells
    z = np.zeros((nc, 3))
    B = np.tile(np.array(wl.b0, np.float64), (nc, 1))
    return {"E_n": z.copy(), "E_half": z.copy(), "B_center": B.copy(),
            "B_corner_prev": B.copy(), "B_corner_cur": B.copy()}


class EcsimContext:
    """One device context: a periodic block mesh (uniform, or the AMR mesh
    `amr_mesh` with wl's species and time step), its fields and particles."""

    def __init__(self, wl: Workload, capacity: Optional[int] = None, track_ids: bool = True,
                 device: int = 0, amr_mesh=None):
        self.lib = _capi.load()
        self.wl = wl
        self.amr_mesh = amr_mesh
        cfg = _capi.Config()
        m = wl.mesh
        cfg.nbx, cfg.nby, cfg.nbz = m.nbx, m.nby, m.nbz
        for d in range(3):
            cfg.x0[d] = m.x0[d]
            cfg.dx[d] = m.dx
        cfg.nspec = len(wl.species)
        for i, s in enumerate(wl.species):
            cfg.charge[i], cfg.mass[i], cfg.weight[i] = s.charge, s.mass, s.weight
        cfg.dt, cfg.theta = wl.dt, wl.theta
        cfg.particle_capacity = int(capacity if capacity is not None else wl.nparticles)
        cfg.track_ids = 1 if track_ids else 0
        cfg.device = device
        self.cfg = cfg
        h = C.c_void_p()
        if amr_mesh is None:
            st = self.lib.amps_gpu_create(C.byref(cfg), C.byref(h))
        else:
            st = self.lib.amps_gpu_create_amr(C.byref(cfg), amr_mesh.h, C.byref(h))
        if st != 0:
            raise AmpsGpuError(st, "amps_gpu_create")
        self.h = h
        nb, ncell, ncor = C.c_longlong(), C.c_longlong(), C.c_longlong()
        self.lib.amps_gpu_mesh_sizes(h, C.byref(nb), C.byref(ncell), C.byref(ncor))
        self.nblocks, self.ncells, self.ncorners = nb.value, ncell.value, ncor.value

    # ---- helpers ----
    def _check(self, st, what):
        if st != 0:
            msg = self.lib.amps_gpu_last_error(self.h)
            raise AmpsGpuError(st, "%s: %s" % (what, msg.decode() if msg else ""))

    def close(self):
        if getattr(self, "h", None):
            self.lib.amps_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def stream(self):
        s = C.c_void_p()
        self._check(self.lib.amps_gpu_get_stream(self.h, C.byref(s)), "get_stream")
        return s.value

    def synchronize(self):
        self._check(self.lib.amps_gpu_synchronize(self.h), "synchronize")

    # ---- ParticleBuffer ----
    def import_particles(self, x, v, spec, wcorr=None):
        x = np.ascontiguousarray(x, np.float64)
        v = np.ascontiguousarray(v, np.float64)
        spec = np.ascontiguousarray(spec, np.uint8)
        wc = None if wcorr is None else np.ascontiguousarray(wcorr, np.float64)
        self._check(self.lib.amps_gpu_import_particles(
            self.h, len(spec), ptr(x, C.c_double), ptr(v, C.c_double), ptr(spec, C.c_uint8),
            ptr(wc, C.c_double)), "import_particles")

    def import_particles_local(self, u, v, spec, block, wcorr=None):
        u = np.ascontiguousarray(u, np.float32)
        v = np.ascontiguousarray(v, np.float32)
        spec = np.ascontiguousarray(spec, np.uint8)
        block = np.ascontiguousarray(block, np.int32)
        wc = None if wcorr is None else np.ascontiguousarray(wcorr, np.float32)
        self._check(self.lib.amps_gpu_import_particles_local_weighted(
            self.h, len(spec), ptr(u, C.c_float), ptr(v, C.c_float), ptr(spec, C.c_uint8),
            ptr(block, C.c_int32), ptr(wc, C.c_float)), "import_particles_local")

    def num_particles(self):
        n = C.c_longlong()
        self._check(self.lib.amps_gpu_num_particles(self.h, C.byref(n)), "num_particles")
        return n.value

    def export_particles(self, ids=True):
        n = self.num_particles()
        x = np.empty((n, 3)); v = np.empty((n, 3))
        spec = np.empty(n, np.uint8); block = np.empty(n, np.int32); cell = np.empty(n, np.int32)
        idv = np.empty(n, np.uint32) if (ids and self.cfg.track_ids) else None
        nn = C.c_longlong()
        self._check(self.lib.amps_gpu_export_particles(
            self.h, ptr(x, C.c_double), ptr(v, C.c_double), ptr(spec, C.c_uint8),
            ptr(block, C.c_int32), ptr(cell, C.c_int32), ptr(idv, C.c_uint32), C.byref(nn)),
            "export_particles")
        out = {"x": x, "v": v, "spec": spec, "block": block, "cell": cell}
        if idv is not None:
            out["id"] = idv
        return out

    # ---- fields / moments ----
    def import_fields(self, E_n=None, E_half=None, B_center=None, B_corner_prev=None,
                      B_corner_cur=None):
        arrs = [None if a is None else np.ascontiguousarray(a, np.float64)
                for a in (E_n, E_half, B_center, B_corner_prev, B_corner_cur)]
        self._check(self.lib.amps_gpu_import_fields(self.h, *[ptr(a, C.c_double) for a in arrs]),
                    "import_fields")

    def set_b_center(self, on=True):
        """True: the particles see B interpolated from the cell centres
        (_PIC_FIELD_SOLVER_B_CENTER_BASED_, the reference's default build;
        CellCentered::Linear, pic_interpolation_routines.cpp:820-905): the push
        reads centre B^n, the deposit centre B^{n+1}; E stays at the corners.
        False (default): the corner B slots.  Uniform meshes only."""
        self._check(self.lib.amps_gpu_set_b_center(self.h, 1 if on else 0), "set_b_center")

    def export_fields(self, out=None):
        """corner E^n, E^{n+theta}, B prev/cur and centre B; out: dict of
        arrays to fill (e.g. page-locked ones)"""
        if out is None:
            out = {k: np.empty((self.ncorners, 3)) for k in
                   ("E_n", "E_half", "B_corner_prev", "B_corner_cur")}
            out["B_center"] = np.empty((self.ncells, 3))
        self._check(self.lib.amps_gpu_export_fields(
            self.h, *[ptr(out[k], C.c_double) for k in
                      ("E_n", "E_half", "B_center", "B_corner_prev", "B_corner_cur")]),
            "export_fields")
        return out

    def import_moments(self, J, M):
        J = np.ascontiguousarray(J, np.float64)
        M = np.ascontiguousarray(M, np.float64)
        self._check(self.lib.amps_gpu_import_moments(self.h, ptr(J, C.c_double),
                                                     ptr(M, C.c_double)), "import_moments")

    def export_moments(self, with_m=True, out=None):
        """corner J (ncorners, 3) and M (ncorners, 243); out=(J, M) reuses arrays.
        On AMR contexts the mesh's unique corners, each summing ProcessCell's
        flush over the cells that have it."""
        nc = self.ncorners
        if out is not None:
            J, M = out
        else:
            J = np.empty((nc, 3))
            M = np.empty((nc, 243)) if with_m else None
        self._check(self.lib.amps_gpu_export_moments(self.h, ptr(J, C.c_double),
                                                     ptr(M, C.c_double)), "export_moments")
        return J, M

    def set_open_axes(self, x=False, y=False, z=False):
        """Delete particles leaving the domain through the faces of these axes."""
        self._check(self.lib.amps_gpu_set_open_axes(self.h, int(bool(x)), int(bool(y)), int(bool(z))),
                    "set_open_axes")

    def add_injection(self, face, spec, density, vth, drift=(0.0, 0.0, 0.0)):
        """Maxwellian flux injection through an open face (0 -x .. 5 +z)."""
        d = np.ascontiguousarray(drift, np.float64)
        self._check(self.lib.amps_gpu_add_injection(self.h, int(face), int(spec), float(density),
                                                    ptr(d, C.c_double), float(vth)), "add_injection")

    def clear_injection(self):
        self._check(self.lib.amps_gpu_clear_injection(self.h), "clear_injection")

    def set_injection_seed(self, seed):
        self._check(self.lib.amps_gpu_set_injection_seed(self.h, int(seed)), "set_injection_seed")

    def injected_particles(self):
        n = C.c_longlong()
        self._check(self.lib.amps_gpu_injected_particles(self.h, C.byref(n)), "injected_particles")
        return n.value

    def deleted_particles(self):
        n = C.c_longlong()
        self._check(self.lib.amps_gpu_deleted_particles(self.h, C.byref(n)), "deleted_particles")
        return n.value

    def set_species_moments(self, on=True):
        """Sample rho, rho u, rho u u per species on the corners at every deposition."""
        self._check(self.lib.amps_gpu_set_species_moments(self.h, 1 if on else 0),
                    "set_species_moments")

    def export_species_moments(self, out=None):
        """(ncorners, nspec, 10): Rho, RhoUx, RhoUy, RhoUz, RhoUxUx, RhoUyUy,
        RhoUzUz, RhoUxUy, RhoUyUz, RhoUxUz per species and corner"""
        ns = self.cfg.nspec
        if out is None:
            out = np.empty((self.ncorners, ns, 10))
        self._check(self.lib.amps_gpu_export_species_moments(self.h, ptr(out, C.c_double)),
                    "export_species_moments")
        return out

    # ---- restart particle section (pic_restart.cpp) -------------------------
    def _restart_args(self, layout, block_order, node_ids):
        layout = layout if layout is not None else _capi.RecordLayout.basic(False)
        bo = None
        if block_order is not None:
            bo = np.ascontiguousarray(block_order, np.int32)
            if bo.shape != (self.nblocks,):
                raise ValueError("block_order must hold every block once")
        if node_ids is None:  # the block index as a 64-bit node id
            node_ids = np.arange(self.nblocks, dtype=np.int64).view(np.uint8).reshape(self.nblocks, 8)
        node_ids = np.ascontiguousarray(node_ids, np.uint8)
        if node_ids.ndim != 2 or node_ids.shape[0] != self.nblocks:
            raise ValueError("node_ids must be (nblocks, id_length) bytes")
        return layout, bo, node_ids

    def restart_particle_bytes(self, layout=None, id_length=8):
        layout = layout if layout is not None else _capi.RecordLayout.basic(False)
        n = C.c_longlong()
        self._check(self.lib.amps_gpu_restart_particle_bytes(self.h, C.byref(layout), id_length,
                                                             C.byref(n)), "restart_particle_bytes")
        return n.value

    def write_restart_particles(self, layout=None, block_order=None, node_ids=None, out=None):
        """The particle section of a restart file (SaveParticleData) as uint8 bytes;
        node_ids (nblocks, id_length) uint8 are the blocks' cAMRnodeID bytes; out:
        a uint8 array of at least restart_particle_bytes() (page-locked: the
        device writes the records into it directly)"""
        layout, bo, ids = self._restart_args(layout, block_order, node_ids)
        need = self.restart_particle_bytes(layout, ids.shape[1])
        if out is None:
            out = np.empty(need, np.uint8)
        elif out.dtype != np.uint8 or not out.flags.c_contiguous or out.size < need:
            raise ValueError("out must be a contiguous uint8 array of at least %d bytes" % need)
        n = C.c_longlong()
        self._check(self.lib.amps_gpu_write_restart_particles(
            self.h, C.byref(layout), ptr(bo, C.c_int32), ids.ctypes.data_as(C.c_void_p), ids.shape[1],
            out.ctypes.data_as(C.c_void_p), out.size, C.byref(n)), "write_restart_particles")
        return out[:n.value]

    def read_restart_particles(self, data, layout=None, node_ids=None):
        """Replace the particles by those of a particle section (ReadParticleData)."""
        layout, _, ids = self._restart_args(layout, None, node_ids)
        data = np.ascontiguousarray(np.frombuffer(data, np.uint8) if isinstance(data, (bytes, bytearray))
                                    else data, np.uint8)
        n = C.c_longlong()
        self._check(self.lib.amps_gpu_read_restart_particles(
            self.h, C.byref(layout), data.ctypes.data_as(C.c_void_p), data.size,
            ids.ctypes.data_as(C.c_void_p), ids.shape[1], C.byref(n)), "read_restart_particles")
        # the species weights come from the section (GlobalParticleWeight)
        w = data[51:51 + 8 * self.cfg.nspec].view(np.float64)
        for i in range(self.cfg.nspec):
            self.cfg.weight[i] = float(w[i])
        return n.value

    def particle_checksum(self, layout=None, block_order=None):
        """GetParticleDataCheckSum: the reference's CRC32 (64-bit accumulator) over
        the records with zeroed links, blocks in block_order, cells i, j, k"""
        layout, bo, _ = self._restart_args(layout, block_order, None)
        v = C.c_ulonglong()
        self._check(self.lib.amps_gpu_particle_checksum(self.h, C.byref(layout), ptr(bo, C.c_int32),
                                                        C.byref(v)), "particle_checksum")
        return v.value

    def export_cell_moments(self, with_m=True, out=None):
        """per-cell ProcessCell partials (cells in block order): cellJ (ncells, 24),
        cellM (ncells, 324) or None; out=(J, M) reuses arrays"""
        if out is not None:
            J, M = out
        else:
            J = np.empty((self.ncells, 24))
            M = np.empty((self.ncells, 324)) if with_m else None
        self._check(self.lib.amps_gpu_export_cell_moments(self.h, ptr(J, C.c_double),
                                                          ptr(M, C.c_double)),
                    "export_cell_moments")
        return J, M

    # ---- reference call surfaces ----
    def MoveParticles(self):
        nout = C.c_longlong()
        self._check(self.lib.amps_gpu_move_particles(self.h, C.byref(nout)), "MoveParticles")
        return nout.value

    def MoveParticlesRelativistic(self, dt_total, light_speed=1.0):
        """Mover::Relativistic::Boris on the mesh fields (E^n, corner B cur);
        returns the number of sub-steps taken."""
        n = C.c_longlong()
        self._check(self.lib.amps_gpu_move_particles_relativistic(self.h, dt_total, light_speed,
                                                                  C.byref(n)),
                    "Mover::Relativistic::Boris")
        return n.value

    def MoveParticlesBoris(self, dt_total):
        """Mover::Boris (non-relativistic test-particle push) on the mesh
        fields (E^n, corner B cur): one step of dt_total, then re-binning."""
        self._check(self.lib.amps_gpu_move_particles_boris(self.h, dt_total), "Mover::Boris")

    def write_tecplot(self, path):
        """Tecplot ASCII file of the corner fields (the reference's mesh-writer
        layout: FEBRICK zone, corner E, B and E^{n+theta})"""
        self._check(self.lib.amps_gpu_write_tecplot(self.h, str(path).encode()), "write_tecplot")

    def div_e_correction(self, tol=1e-8, maxit=500, redeposit=True):
        """ECSIM::divECorrection on periodic uniform meshes: net charge, div E,
        the Poisson solve, the species-0 position correction and re-binning;
        redeposit: UpdateJMassMatrix on the corrected particles.  Returns the
        statistics (CG iterations and residual, the Gauss-law residual before
        and after, particles corrected)."""
        st = _capi.DiveStats()
        self._check(self.lib.amps_gpu_div_e_correction(self.h, tol, maxit, 1 if redeposit else 0,
                                                       C.byref(st)), "div_e_correction")
        return {"iterations": st.iterations, "rel_residual": st.rel_residual,
                "gauss_before": st.gauss_before, "gauss_after": st.gauss_after,
                "moved": st.moved}

    def export_div_e(self):
        """per-cell rho_new, rho_old, div E and phi of the last correction"""
        nc = self.wl.mesh.ncells
        out = {k: np.zeros(nc) for k in ("rho_new", "rho_old", "div_e", "phi")}
        self._check(self.lib.amps_gpu_export_div_e(
            self.h, ptr(out["rho_new"], C.c_double), ptr(out["rho_old"], C.c_double),
            ptr(out["div_e"], C.c_double), ptr(out["phi"], C.c_double)), "export_div_e")
        return out

    def particle_cfl(self):
        """per-species maximum CFL number of the current particles (the value
        UpdateJMassMatrix prints)"""
        out = np.zeros(len(self.wl.species))
        self._check(self.lib.amps_gpu_particle_cfl(self.h, ptr(out, C.c_double)), "particle_cfl")
        return out

    def UpdateJMassMatrix(self):
        e = C.c_double()
        self._check(self.lib.amps_gpu_update_j_mass_matrix(self.h, C.byref(e)),
                    "UpdateJMassMatrix")
        return e.value

    def TimeStep(self, tol=None, maxit=200, precond=0):
        st = _capi.SolveStats()
        tol = self.wl.tol if tol is None else tol
        self._check(self.lib.amps_gpu_field_solve(self.h, tol, maxit, precond, C.byref(st)),
                    "ECSIM::TimeStep")
        return st

    def PicTimeStep(self, tol=None, maxit=200, precond=0):
        st = _capi.StepStats()
        tol = self.wl.tol if tol is None else tol
        self._check(self.lib.amps_gpu_step(self.h, tol, maxit, precond, C.byref(st)),
                    "PIC::TimeStep")
        return st

    def push_deposit(self, want_energy=True):
        e = C.c_double()
        self._check(self.lib.amps_gpu_push_deposit(self.h, C.byref(e) if want_energy else None),
                    "push_deposit")
        return e.value

    # ---- field-solve options and the learned preconditioner ----
    def set_inner_fp64(self, on=True):
        """GMRES inner operator in FP64 (True) or FP32 with FP64 refinement (False)."""
        self._check(self.lib.amps_gpu_set_inner_fp64(self.h, 1 if on else 0), "set_inner_fp64")

    def precond_num_sets(self):
        """Weight sets of the network: 1 on a uniform mesh, one per level on AMR."""
        n = C.c_int()
        self._check(self.lib.amps_gpu_precond_num_sets(self.h, C.byref(n)), "precond_num_sets")
        return n.value

    def precond_select(self, wset):
        """Weight set that load / weights / train / loss_grad / forward act on."""
        self._check(self.lib.amps_gpu_precond_select(self.h, int(wset)), "precond_select")

    def precond_interface_jacobi(self, on=True):
        """Jacobi instead of the network on blocks at refinement interfaces;
        returns the number of such blocks."""
        n = C.c_int()
        self._check(self.lib.amps_gpu_precond_interface_jacobi(self.h, 1 if on else 0, C.byref(n)),
                    "precond_interface_jacobi")
        return n.value

    def precond_sample_sets(self, first=0, count=None):
        if count is None:
            count = self.precond_num_samples() - first
        out = np.empty(count, np.int32)
        self._check(self.lib.amps_gpu_precond_sample_sets(self.h, first, count, ptr(out, C.c_int32)),
                    "precond_sample_sets")
        return out

    def precond_load(self, w1, w2, w3):
        ws = [np.ascontiguousarray(w, np.float32) for w in (w1, w2, w3)]
        for w, shp in zip(ws, PRECOND_SHAPES):
            if w.shape != shp:
                raise ValueError("weight shape %s, expected %s" % (w.shape, shp))
        self._check(self.lib.amps_gpu_precond_load(self.h, *[ptr(w, C.c_float) for w in ws]),
                    "precond_load")

    def precond_weights(self):
        ws = [np.empty(shp, np.float32) for shp in PRECOND_SHAPES]
        self._check(self.lib.amps_gpu_precond_get(self.h, *[ptr(w, C.c_float) for w in ws]),
                    "precond_get")
        return ws

    def precond_use_tensor_cores(self, on=True):
        self._check(self.lib.amps_gpu_precond_use_tensor_cores(self.h, 1 if on else 0),
                    "precond_use_tensor_cores")

    def precond_harvest(self, capacity):
        self._check(self.lib.amps_gpu_precond_harvest(self.h, int(capacity)), "precond_harvest")

    def precond_num_samples(self):
        n = C.c_longlong()
        self._check(self.lib.amps_gpu_precond_num_samples(self.h, C.byref(n)), "num_samples")
        return n.value

    def precond_samples(self, first=0, count=None):
        if count is None:
            count = self.precond_num_samples() - first
        x = np.empty((count, 1000, 3), np.float32)
        e = np.empty((count, 512, 3), np.float32)
        self._check(self.lib.amps_gpu_precond_get_samples(self.h, first, count, ptr(x, C.c_float),
                                                          ptr(e, C.c_float)), "get_samples")
        return x, e

    def precond_train(self, epochs, batch=64, lr=1e-3, seed=1):
        loss = np.zeros(epochs, np.float32)
        self._check(self.lib.amps_gpu_precond_train(self.h, epochs, batch, lr, seed,
                                                    ptr(loss, C.c_float)), "precond_train")
        return loss

    def precond_loss_grad(self, x, e):
        x = np.ascontiguousarray(x, np.float32)
        e = np.ascontiguousarray(e, np.float32)
        g = [np.empty(shp, np.float32) for shp in PRECOND_SHAPES]
        loss = C.c_float()
        self._check(self.lib.amps_gpu_precond_loss_grad(
            self.h, len(x), ptr(x, C.c_float), ptr(e, C.c_float), C.byref(loss),
            *[ptr(q, C.c_float) for q in g]), "precond_loss_grad")
        return loss.value, g

    def precond_forward(self, x, tensor_cores=False):
        x = np.ascontiguousarray(x, np.float32)
        y = np.empty((len(x), 512, 3), np.float32)
        self._check(self.lib.amps_gpu_precond_forward(self.h, len(x), ptr(x, C.c_float),
                                                      1 if tensor_cores else 0, ptr(y, C.c_float)),
                    "precond_forward")
        return y

    # ---- launch configuration ----
    def set_graphs(self, on=True):
        self._check(self.lib.amps_gpu_set_graphs(self.h, 1 if on else 0), "set_graphs")

    def set_arrivals_chunk(self, chunk):
        """stage arrivals 16 or 32 at a time (ends an autotuner comparison)"""
        self._check(self.lib.amps_gpu_set_arrivals_chunk(self.h, int(chunk)), "set_arrivals_chunk")

    def particle_tuning(self):
        """the arrivals chunk in use, the particle steps the autotuner still
        compares, and the mean ms per arrivals launch of 16 and 32"""
        chunk, pending = C.c_int(), C.c_int()
        ms = np.zeros(2)
        self._check(self.lib.amps_gpu_get_particle_tuning(self.h, C.byref(chunk), C.byref(pending),
                                                          ptr(ms, C.c_double)), "particle_tuning")
        return {"arrivals_chunk": chunk.value, "pending_steps": pending.value,
                "arrivals_ms_16_32": ms.round(4).tolist()}

    def autotune(self):
        """Times candidate launch shapes of the field kernels; returns the
        candidates' times and the chosen (threads per CTA, reduction CTAs).
        Also arms the arrivals comparison of the next 6 particle steps
        (particle_tuning)."""
        ms = np.zeros(6)
        self._check(self.lib.amps_gpu_autotune(self.h, ptr(ms, C.c_double)), "autotune")
        tb, red = C.c_int(), C.c_int()
        self._check(self.lib.amps_gpu_get_tuning(self.h, C.byref(tb), C.byref(red)), "get_tuning")
        return {"operator_ms_tb64_128_256": ms[:3].round(4).tolist(),
                "sweep_ms_cta76_152_304": ms[3:].round(4).tolist(),
                "threads_per_cta": tb.value, "reduction_ctas": red.value}

    # ---- timing ----
    def set_kernel_timing(self, on=True):
        self._check(self.lib.amps_gpu_set_kernel_timing(self.h, 1 if on else 0), "timing")

    def reset_kernel_times(self):
        self._check(self.lib.amps_gpu_reset_kernel_times(self.h), "reset timing")

    def kernel_times(self):
        cap = 64
        names = (C.c_char_p * cap)()
        ms = np.zeros(cap)
        cnt = np.zeros(cap, np.int64)
        n = C.c_int()
        self._check(self.lib.amps_gpu_get_kernel_times(self.h, names, ptr(ms, C.c_double),
                                                       cnt.ctypes.data_as(C.POINTER(C.c_longlong)),
                                                       cap, C.byref(n)), "kernel times")
        return {names[i].decode(): (float(ms[i]), int(cnt[i])) for i in range(n.value)}


PRECOND_SHAPES = ((27, 3, 32), (27, 32, 32), (27, 32, 3))


class PinnedArrays:
    """Page-locked host arrays (cudaHostAlloc) viewed as numpy arrays, for
    host <-> device copies at full link bandwidth."""

    def __init__(self):
        self.rt = C.CDLL("libcudart.so")
        self.ptrs = []

    def empty(self, shape, dtype=np.float64):
        dt = np.dtype(dtype)
        nbytes = int(np.prod(shape)) * dt.itemsize
        p = C.c_void_p()
        if self.rt.cudaHostAlloc(C.byref(p), C.c_size_t(max(nbytes, 1)), 0) != 0:
            raise MemoryError("cudaHostAlloc of %d bytes failed" % nbytes)
        self.ptrs.append(p)
        buf = (C.c_byte * max(nbytes, 1)).from_address(p.value)
        return np.frombuffer(buf, dtype=dt, count=int(np.prod(shape))).reshape(shape)

    def free(self):
        for p in self.ptrs:
            self.rt.cudaFreeHost(p)
        self.ptrs = []


def init_precond_weights(seed=0, out_scale=1e-3):
    """Seeded initial weights of the block network: layers 1-2 scaled by
    1/sqrt(fan-in), the output layer by out_scale/sqrt(fan-in) so that the
    untrained preconditioner is Jacobi plus a small correction."""
    rng = np.random.default_rng(seed)
    ws = []
    for l, shp in enumerate(PRECOND_SHAPES):
        fan = shp[0] * shp[1]
        sc = (out_scale if l == 2 else 1.0) / np.sqrt(fan)
        ws.append((sc * rng.standard_normal(shp)).astype(np.float32))
    return ws


def trace_dipole(x, p, q, m0, b_eq, r_e, b_ext, r_in, r_out, max_steps, dphi_max=0.15,
                 dt_max=1.0, precision=0, device=0):
    """Batched relativistic Boris tracing (SI). x, p are (n,3) float64 arrays,
    updated in place.  Returns (status, steps, total_steps, kernel_ms)."""
    lib = _capi.load()
    n = len(x)
    assert x.dtype == np.float64 and p.dtype == np.float64 and x.flags.c_contiguous
    status = np.zeros(n, np.int32)
    steps = np.zeros(n, np.int64)
    ext = np.ascontiguousarray(b_ext, np.float64)
    tot = C.c_longlong()
    ms = C.c_double()
    st = lib.amps_gpu_trace_dipole(device, n, ptr(x, C.c_double), ptr(p, C.c_double),
                                   ptr(status, C.c_int32), ptr(steps, C.c_int64), q, m0, b_eq,
                                   r_e, ptr(ext, C.c_double), r_in, r_out, max_steps, dphi_max,
                                   dt_max, precision, C.byref(tot), C.byref(ms))
    if st != 0:
        raise AmpsGpuError(st, "amps_gpu_trace_dipole")
    return status, steps, tot.value, ms.value
