"""ctypes declarations of libamps_gpu.so (include/amps_gpu.h).

The shared library is the product; this module only binds it.  Importing it
fails loudly when the library has not been built: there is no CPU fallback.
The host-side mesh builder and initial condition (amps_amr_*, amps_ic_*) live
in libamps_host.so, on which libamps_gpu.so depends; load_host() binds that
library alone, for callers that build meshes and particles without a GPU.
"""
import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libamps_gpu.so")
HOST_LIB_PATH = os.path.join(_HERE, "libamps_host.so")

MAX_SPECIES = 8

STATUS = {
    0: "OK",
    1: "INVALID_ARG",
    2: "OUT_OF_DOMAIN_PARTICLES",
    3: "GMRES_NOT_CONVERGED",
    4: "DEVICE_TIMEOUT",
    5: "CUDA_ERROR",
    6: "CAPACITY_EXCEEDED",
    7: "NO_DEVICE",
}


class AmpsGpuError(RuntimeError):
    def __init__(self, status, msg=""):
        self.status = status
        super().__init__("%s (%d)%s" % (STATUS.get(status, "?"), status, (": " + msg) if msg else ""))


class Config(C.Structure):
    _fields_ = [
        ("nbx", C.c_int), ("nby", C.c_int), ("nbz", C.c_int),
        ("x0", C.c_double * 3), ("dx", C.c_double * 3),
        ("nspec", C.c_int),
        ("charge", C.c_double * MAX_SPECIES),
        ("mass", C.c_double * MAX_SPECIES),
        ("weight", C.c_double * MAX_SPECIES),
        ("dt", C.c_double), ("theta", C.c_double),
        ("particle_capacity", C.c_longlong),
        ("track_ids", C.c_int), ("device", C.c_int),
    ]


class RecordLayout(C.Structure):
    """amps_gpu_record_layout: the caller's particle record (ParticleDataLength
    and the offsets of velocity, position, species, weight correction or -1)"""
    _fields_ = [("record_length", C.c_int), ("off_velocity", C.c_int), ("off_position", C.c_int),
                ("off_species", C.c_int), ("off_weight", C.c_int)]

    @classmethod
    def basic(cls, weight_correction=False):
        """picParticleBasicOffset.cpp: next, prev, v, x, species [, weight correction]"""
        return cls(80, 16, 40, 64, 72) if weight_correction else cls(65, 16, 40, 64, -1)


class SolveStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("converged", C.c_int),
                ("rel_residual", C.c_double), ("wave_energy", C.c_double)]


class StepStats(C.Structure):
    _fields_ = [("solve", SolveStats), ("particle_energy", C.c_double),
                ("out_of_block", C.c_longlong), ("ulp_face", C.c_longlong)]


class DiveStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("rel_residual", C.c_double),
                ("gauss_before", C.c_double), ("gauss_after", C.c_double),
                ("moved", C.c_longlong)]


P = C.c_void_p
D = C.POINTER(C.c_double)
F = C.POINTER(C.c_float)
U8 = C.POINTER(C.c_uint8)
I32 = C.POINTER(C.c_int32)
U32 = C.POINTER(C.c_uint32)
I64 = C.POINTER(C.c_int64)
LL = C.POINTER(C.c_longlong)

# name -> (restype, argtypes); every symbol declared in include/amps_gpu.h
SIGNATURES = {
    "amps_amr_build": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, D, C.c_double, P, C.c_int,
                                 C.POINTER(P)]),
    "amps_amr_info": (C.c_int, [P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "amps_amr_tables": (C.c_int, [P, I32, I32, I32, I32, D, I32]),
    "amps_amr_destroy": (C.c_int, [P]),
    "amps_amr_build_open": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, D, C.c_double, P, C.c_int,
                                      C.POINTER(C.c_int), C.c_int, C.POINTER(P)]),
    "amps_amr_build_open_faces": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, D, C.c_double, P,
                                            C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                            C.POINTER(P)]),
    "amps_amr_boundary_tables": (C.c_int, [P, C.POINTER(C.c_int), I32, I32, I32, D]),
    "amps_amr_nested_leaves": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                         C.c_double, P, C.c_int]),
    "amps_gpu_create": (C.c_int, [C.POINTER(Config), C.POINTER(P)]),
    "amps_gpu_create_amr": (C.c_int, [C.POINTER(Config), P, C.POINTER(P)]),
    "amps_gpu_mesh_sizes": (C.c_int, [P, LL, LL, LL]),
    "amps_gpu_export_cell_moments": (C.c_int, [P, D, D]),
    "amps_gpu_destroy": (C.c_int, [P]),
    "amps_gpu_last_error": (C.c_char_p, [P]),
    "amps_gpu_get_stream": (C.c_int, [P, C.POINTER(P)]),
    "amps_gpu_synchronize": (C.c_int, [P]),
    "amps_gpu_import_particles": (C.c_int, [P, C.c_longlong, D, D, U8, D]),
    "amps_gpu_import_particles_local": (C.c_int, [P, C.c_longlong, F, F, U8, I32]),
    "amps_gpu_import_particles_local_weighted": (C.c_int, [P, C.c_longlong, F, F, U8, I32, F]),
    "amps_gpu_set_species_moments": (C.c_int, [P, C.c_int]),
    "amps_gpu_set_open_axes": (C.c_int, [P, C.c_int, C.c_int, C.c_int]),
    "amps_gpu_deleted_particles": (C.c_int, [P, LL]),
    "amps_gpu_add_injection": (C.c_int, [P, C.c_int, C.c_int, C.c_double, D, C.c_double]),
    "amps_gpu_clear_injection": (C.c_int, [P]),
    "amps_gpu_set_injection_seed": (C.c_int, [P, C.c_ulonglong]),
    "amps_gpu_injected_particles": (C.c_int, [P, LL]),
    "amps_gpu_export_species_moments": (C.c_int, [P, D]),
    "amps_gpu_restart_particle_bytes": (C.c_int, [P, C.POINTER(RecordLayout), C.c_int, LL]),
    "amps_gpu_write_restart_particles": (C.c_int, [P, C.POINTER(RecordLayout), I32, P, C.c_int, P,
                                                   C.c_longlong, LL]),
    "amps_gpu_read_restart_particles": (C.c_int, [P, C.POINTER(RecordLayout), P, C.c_longlong, P,
                                                  C.c_int, LL]),
    "amps_gpu_particle_checksum": (C.c_int, [P, C.POINTER(RecordLayout), I32,
                                             C.POINTER(C.c_ulonglong)]),
    "amps_gpu_export_particles": (C.c_int, [P, D, D, U8, I32, I32, U32, LL]),
    "amps_gpu_num_particles": (C.c_int, [P, LL]),
    "amps_gpu_import_fields": (C.c_int, [P, D, D, D, D, D]),
    "amps_gpu_export_fields": (C.c_int, [P, D, D, D, D, D]),
    "amps_gpu_import_moments": (C.c_int, [P, D, D]),
    "amps_gpu_export_moments": (C.c_int, [P, D, D]),
    "amps_gpu_move_particles": (C.c_int, [P, LL]),
    "amps_gpu_move_particles_relativistic": (C.c_int, [P, C.c_double, C.c_double, LL]),
    "amps_gpu_move_particles_boris": (C.c_int, [P, C.c_double]),
    "amps_gpu_particle_cfl": (C.c_int, [P, C.POINTER(C.c_double)]),
    "amps_gpu_write_tecplot": (C.c_int, [P, C.c_char_p]),
    "amps_gpu_div_e_correction": (C.c_int, [P, C.c_double, C.c_int, C.c_int, C.POINTER(DiveStats)]),
    "amps_gpu_export_div_e": (C.c_int, [P, D, D, D, D]),
    "amps_gpu_update_j_mass_matrix": (C.c_int, [P, D]),
    "amps_gpu_field_solve": (C.c_int, [P, C.c_double, C.c_int, C.c_int, C.POINTER(SolveStats)]),
    "amps_gpu_step": (C.c_int, [P, C.c_double, C.c_int, C.c_int, C.POINTER(StepStats)]),
    "amps_gpu_push_deposit": (C.c_int, [P, D]),
    "amps_gpu_update_j_mass_matrix_noalloc": (C.c_int, [C.POINTER(Config), C.c_longlong, P, P,
                                                        P, P, P, P, P, P, P]),
    "amps_gpu_set_inner_fp64": (C.c_int, [P, C.c_int]),
    "amps_gpu_precond_load": (C.c_int, [P, F, F, F]),
    "amps_gpu_precond_get": (C.c_int, [P, F, F, F]),
    "amps_gpu_precond_use_tensor_cores": (C.c_int, [P, C.c_int]),
    "amps_gpu_precond_harvest": (C.c_int, [P, C.c_longlong]),
    "amps_gpu_precond_num_samples": (C.c_int, [P, LL]),
    "amps_gpu_precond_get_samples": (C.c_int, [P, C.c_longlong, C.c_longlong, F, F]),
    "amps_gpu_precond_sample_sets": (C.c_int, [P, C.c_longlong, C.c_longlong, I32]),
    "amps_gpu_precond_num_sets": (C.c_int, [P, C.POINTER(C.c_int)]),
    "amps_gpu_precond_select": (C.c_int, [P, C.c_int]),
    "amps_gpu_precond_interface_jacobi": (C.c_int, [P, C.c_int, C.POINTER(C.c_int)]),
    "amps_gpu_precond_train": (C.c_int, [P, C.c_int, C.c_int, C.c_float, C.c_ulonglong, F]),
    "amps_gpu_precond_loss_grad": (C.c_int, [P, C.c_longlong, F, F, F, F, F, F]),
    "amps_gpu_precond_forward": (C.c_int, [P, C.c_longlong, F, C.c_int, F]),
    "amps_gpu_set_graphs": (C.c_int, [P, C.c_int]),
    "amps_gpu_autotune": (C.c_int, [P, D]),
    "amps_gpu_get_tuning": (C.c_int, [P, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "amps_gpu_set_arrivals_chunk": (C.c_int, [P, C.c_int]),
    "amps_gpu_set_b_center": (C.c_int, [P, C.c_int]),
    "amps_gpu_get_particle_tuning": (C.c_int, [P, C.POINTER(C.c_int), C.POINTER(C.c_int), D]),
    "amps_gpu_set_kernel_timing": (C.c_int, [P, C.c_int]),
    "amps_gpu_get_kernel_times": (C.c_int, [P, C.POINTER(C.c_char_p), D, LL, C.c_int,
                                            C.POINTER(C.c_int)]),
    "amps_gpu_reset_kernel_times": (C.c_int, [P]),
    "amps_ic_count": (C.c_longlong, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
    "amps_ic_maxwellian": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, D,
                                     C.c_ulonglong, C.c_int, F, F, U8, I32]),
    "amps_gpu_trace_dipole": (C.c_int, [C.c_int, C.c_longlong, D, D, I32, I64, C.c_double,
                                        C.c_double, C.c_double, C.c_double, D, C.c_double,
                                        C.c_double, C.c_longlong, C.c_double, C.c_double,
                                        C.c_int, LL, D]),
}

_lib = None
_host = None


def load_host():
    """Load and bind libamps_host.so (AMR mesh builder, initial condition)."""
    global _host
    if _host is not None:
        return _host
    if not os.path.exists(HOST_LIB_PATH):
        raise ImportError("libamps_host.so is not built (%s); run __graft_entry__.build()"
                          % HOST_LIB_PATH)
    lib = C.CDLL(HOST_LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        if name.startswith(("amps_amr_", "amps_ic_")):
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
    _host = lib
    return lib


def load():
    """Load and bind libamps_gpu.so (raises if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libamps_gpu.so is not built (%s); run __graft_entry__.build()" % LIB_PATH)
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def ptr(a, ctype):
    """numpy array -> ctypes pointer (None passes through)."""
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ctype))
