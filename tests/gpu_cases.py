"""Shared seeded inputs for the GPU parity tests (oracle comparisons)."""
import numpy as np

import amps_gb300 as A
from tests import oracle_lib as O


def smooth_field(shape_cells, rng, amp, kmax=2):
    """Random smooth periodic vector field on the corner grid (FP64, (n,3))."""
    NX, NY, NZ = shape_cells
    I, J, K = np.meshgrid(np.arange(NX), np.arange(NY), np.arange(NZ), indexing="ij")
    out = np.zeros((NX, NY, NZ, 3))
    for d in range(3):
        for _ in range(4):
            k = rng.integers(-kmax, kmax + 1, 3)
            ph = rng.uniform(0, 2 * np.pi)
            out[..., d] += amp * rng.uniform(0.3, 1.0) * np.cos(
                2 * np.pi * (k[0] * I / NX + k[1] * J / NY + k[2] * K / NZ) + ph)
    # global corner index I + NX*(J + NY*K): transpose to K,J,I order then flatten
    return np.ascontiguousarray(out.transpose(2, 1, 0, 3).reshape(-1, 3))


def make_case(nb=(2, 2, 2), ppc=8, seed=100, e_amp=2e-3, b_amp=0.05, vscale=1.0):
    wl = A.electron_proton_plasma("case", *nb, ppc, 3)
    wl.seed = seed
    ic = A.make_initial_condition(wl, nthreads=4)
    if vscale != 1.0:
        ic["v"] = (ic["v"] * np.float32(vscale)).astype(np.float32)
    x = A.physical_positions(wl.mesh, ic["u"], ic["block"])
    rng = np.random.default_rng(seed)
    f = A.initial_fields(wl)
    shp = wl.mesh.shape
    f["E_n"] = smooth_field(shp, rng, e_amp)
    f["E_half"] = smooth_field(shp, rng, e_amp)
    f["B_center"] = f["B_center"] + smooth_field(shp, rng, b_amp)
    f["B_corner_prev"] = f["B_corner_prev"] + smooth_field(shp, rng, b_amp)
    f["B_corner_cur"] = f["B_corner_cur"] + smooth_field(shp, rng, b_amp)
    return wl, ic, x, f


def gpu_ctx(wl, ic, x, f, capacity=None, wcorr=None):
    ctx = A.EcsimContext(wl, capacity=capacity, track_ids=True)
    ctx.import_particles(x, ic["v"].astype(np.float64), ic["spec"], wcorr)
    ctx.import_fields(**f)
    return ctx


def oracle_state(wl, ic, x, f, wcorr=None):
    return O.OracleState(wl, x, ic["v"].astype(np.float64), ic["spec"], f, wcorr)


def by_id(exp):
    order = np.argsort(exp["id"])
    return {k: v[order] for k, v in exp.items()}


def face_distance(x, dx=1.0):
    """Distance (cells) of each position to the nearest cell face, min over axes."""
    u = x / dx
    return np.min(np.abs(u - np.rint(u)), axis=1)


def rel_err(a, b):
    den = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / (den if den > 0 else 1.0))
