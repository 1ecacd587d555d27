"""Benchmark of the AMPS particle hot path on GB300: particle-steps/s of
push + re-bin + deposit (Lapenta2017 mover + ECSIM UpdateJMassMatrix).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--workload NAME]

Default workload: the two-level AMR plasma (64^3 base cells in 8^3-cell
blocks, central 1/8 of the volume refined 2x, electrons + protons at 128
particles per species per base cell: 67,108,864 particles, 960 blocks).
Uniform periodic workloads (WORKLOADS in amps_gb300.ecsim) run with the same
command.

A step is one pass of push + re-bin + deposit over every particle of the
workload (inputs resident in HBM; the particle arrays, ~1.7 GB, exceed the
129 MB L2, so no L2 flush is needed).  The timed region is bracketed by a
barrier and device synchronisation and timed with CUDA events on the library's
stream; the max over ranks is reported.  N > 1 runs independent replicas (the
path is not sharded), value = all ranks' particle-steps / max time.

--impl reference times the reference CPU path on the host cores: the FP64
restatement of Lapenta2017 + re-binning + ProcessCell (oracle/, pinned to the
reference's own ProcessCell and Lapenta2017 compiled from its sources) over
every particle of the same workload on all host threads (uniform workloads:
one replica of the plasma per host thread).
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s (push+deposit)"
# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of the
# particle-step kernels on the default workload, from a one-pass ncu capture
# of this bench command; "version" names the kernel revision it was taken on
MEASURED_TRAFFIC = {"amr_64c_128ppc": {"version": "push_deposit packed-FMA 3x3 tiles on SoA "
                                                  "records, FP32 chunk sums, unrolled full chunks; "
                                                  "arrivals from a "
                                                  "per-layer cell list",
                                       "push_deposit": 4.663e9, "arrivals": 1.015e9}}
UNIT = "particle-steps/s"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def init_dist(ws):
    if ws <= 1:
        return None
    import torch.distributed as dist
    backend = os.environ.get("AMPS_DIST_BACKEND", "nccl")
    dist.init_process_group(backend)
    return dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, val):
    if dist is None:
        return val
    import torch
    t = torch.tensor([float(val)], dtype=torch.float64)
    if dist.get_backend() == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(dist, val):
    if dist is None:
        return val
    import torch
    t = torch.tensor([float(val)], dtype=torch.float64)
    if dist.get_backend() == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def replica_throughput(dist, units, ms):
    """Whole-job throughput of N independent replicas: the units all ranks
    processed over the slowest rank's time.  Returns (units/s, max ms)."""
    ms_max = max_over_ranks(dist, ms)
    return sum_over_ranks(dist, units) / (ms_max / 1e3), ms_max


# ---------------------------------------------------------------------------
class CudaEvents:
    """CUDA events on an external stream through the runtime library."""

    def __init__(self):
        self.rt = C.CDLL("libcudart.so")

    def event(self):
        e = C.c_void_p()
        assert self.rt.cudaEventCreate(C.byref(e)) == 0
        return e

    def record(self, e, stream):
        assert self.rt.cudaEventRecord(e, C.c_void_p(stream)) == 0

    def elapsed_ms(self, a, b):
        self.rt.cudaEventSynchronize(b)
        ms = C.c_float()
        assert self.rt.cudaEventElapsedTime(C.byref(ms), a, b) == 0
        return ms.value

    def sync(self):
        self.rt.cudaDeviceSynchronize()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------------------
def kernel_bytes(n, ncell, nb, name, b_center=False):
    """Algorithmic bytes per launch of each particle-step kernel: what the
    kernel must read and write given the slotted cell layout (n particles,
    ncell cells, nb blocks; b_center: B from the cell centres)."""
    ctas = nb * 8
    if name == "push_deposit":
        # particles: read u,v (24) + species (1), write u,v (24); per cell: base, cnt
        # (8), stay (4), partials 267 floats (27 monomials x 9 + 8 corners x 3);
        # stencils 23.3 + 11.7 KB per CTA (centre B: 23.3 + 2 x 16 KB)
        return n * 49 + ncell * (12 + 267 * 4) + ctas * (23328 + (32000 if b_center else 11664))
    if name == "arrivals":
        # per cell: base, base+1, cnt, stay, arr (20) and cnt/arr writes (8); the
        # ~1% arrivals and their partial read-modify-write; stencil per CTA
        return ncell * 28 + ctas * 11664
    if name == "assemble":
        # read the partials (64 monomial blocks + 8 current rows per corner, from
        # 8 cells: each cell's 267 floats are read by its 8 corners, mostly from
        # L2); write M (243 FP32) + J (3 FP64)
        return ncell * 267 * 4 + ncell * (243 * 4 + 3 * 8)
    if name == "pack_stencils":
        return ncell * 9 * 8 * 27 // 8 + nb * (23328 + 11664)
    return None


# FP32 operations of one push + deposit of a particle (the fused kernel's
# algorithm): trilinear weights 16 + E/B gather 96 + Lapenta2017 ~40 + position
# 6; deposit weights 16 + alpha ~30 + alpha v 18 + J 48 + 27 weight monomials 54
# + mass matrix 27 x 9 FMA 486 + kinetic energy 6
FLOP_PER_PARTICLE = 816


def cpu_replica_rate(wl_name, steps, seconds_budget, threads):
    """FP64 oracle (Lapenta2017 + ProcessCell + re-binning) on per-thread
    single-block periodic replicas of the workload's plasma.  Returns
    particle-steps/s over all threads."""
    import amps_gb300 as A
    from tests import oracle_lib as O
    base = A.WORKLOADS[wl_name]()
    rep = A.electron_proton_plasma("cpu_replica", 1, 1, 1, base.ppc, steps)
    states = []
    for t in range(threads):
        rep.seed = 100 + 2 * t + 1
        ic = A.make_initial_condition(rep, nthreads=1)
        x = A.physical_positions(rep.mesh, ic["u"], ic["block"])
        f = A.initial_fields(rep)
        states.append(O.OracleState(rep, x, ic["v"].astype(np.float64), ic["spec"], f))
    counts = [0] * threads
    deadline = [None]

    def work(i):
        st = states[i]
        while time.time() < deadline[0]:
            st.push()
            st.deposit()
            counts[i] += len(st.spec)

    deadline[0] = time.time() + seconds_budget
    t0 = time.time()
    th = [threading.Thread(target=work, args=(i,)) for i in range(threads)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    dt = time.time() - t0
    n = rep.nparticles
    return sum(counts) / dt, {"replica_particles": n, "threads": threads, "seconds": dt,
                              "particle_steps": sum(counts)}


def setup_workload(name, device, track_ids=False):
    """Context with the workload's particles and initial fields imported.
    Returns (ctx, info)."""
    import amps_gb300 as A
    from amps_gb300 import amr
    t_ic = time.time()
    if name in amr.AMR_WORKLOADS:
        wl = amr.AMR_WORKLOADS[name]()
        mesh = wl.mesh()
        ic = wl.initial_condition(mesh, seed=100, nthreads=os.cpu_count() or 8)
        t_ic = time.time() - t_ic
        n = len(ic["spec"])
        ctx = A.EcsimContext(wl.plasma, capacity=n, track_ids=track_ids, device=device,
                             amr_mesh=mesh)
        f = amr.amr_initial_fields(mesh, wl.b0)
        info = {"workload": name, "particles": n, "cells": mesh.ncells, "blocks": mesh.nblocks,
                "corners": mesh.ncorners, "hanging_corners": mesh.nhanging,
                "levels": wl.lmax + 1, "fine_blocks": int(np.sum(mesh.level > 0)),
                ("ppc_per_species_per_cell" if wl.per_cell else "ppc_per_species_base_cell"): wl.ppc,
                "amr": True, "tol": wl.tol}
        if wl.per_cell:
            info["weights"] = "weight correction 8^-level per particle (uniform density)"
    else:
        wl = A.WORKLOADS[name]()
        ic = A.make_initial_condition(wl, nthreads=os.cpu_count() or 8)
        t_ic = time.time() - t_ic
        n = wl.nparticles
        ctx = A.EcsimContext(wl, capacity=n, track_ids=track_ids, device=device)
        f = A.initial_fields(wl)
        info = {"workload": name, "particles": n, "cells": wl.mesh.ncells,
                "blocks": wl.mesh.nblocks, "ppc_per_species": wl.ppc, "amr": False,
                "tol": wl.tol}
    ctx.import_particles_local(ic["u"], ic["v"], ic["spec"], ic["block"], ic.get("wcorr"))
    ctx.import_fields(**f)
    info["ic_seconds"] = round(t_ic, 2)
    return ctx, info


def precond_ab(workload, device, nsamples=20000, epochs=20, lr=2e-3, dt=None, reps=3):
    """Learned vs plain vs Jacobi GMRES on one uniform workload: train the block
    network on nsamples pairs harvested from Jacobi solves of seeded plasma
    states, then time the field solve and the full ECSIM step from identical
    held-out states (host wall clock around calls that synchronise)."""
    import amps_gb300 as A
    from amps_gb300 import precond as PC
    wl = A.WORKLOADS[workload]()
    if dt is not None:
        wl.dt = dt
    ctx, info = PC.build_trained_context(wl, nsamples=nsamples, epochs=epochs, batch=64, lr=lr,
                                         device=device, e_amp=1e-3, b_amp=0.02)
    ctx.precond_use_tensor_cores(True)
    names = {0: "plain", 1: "jacobi", 2: "learned"}
    solve = {k: [] for k in names.values()}
    step = {k: [] for k in names.values()}
    iters = {k: [] for k in names.values()}
    for seed in (5001, 5002, 5003):
        PC.random_state(ctx, wl, seed, e_amp=1e-3, b_amp=0.02)
        ctx.PicTimeStep(tol=wl.tol, maxit=400, precond=1)   # evolve once from the seeded state
        f0 = ctx.export_fields()
        p0 = ctx.export_particles(ids=False)
        for pc, nm in names.items():
            ts, tp = [], []
            for _ in range(reps):
                ctx.import_fields(**f0)
                ctx.synchronize()
                t = time.perf_counter()
                st = ctx.TimeStep(tol=wl.tol, maxit=400, precond=pc)
                ctx.synchronize()
                ts.append((time.perf_counter() - t) * 1e3)
                if not st.converged:
                    raise RuntimeError("%s solve did not converge" % nm)
            iters[nm].append(st.iterations)
            for _ in range(reps):
                ctx.import_particles(p0["x"], p0["v"], p0["spec"])
                ctx.import_fields(**f0)
                ctx.UpdateJMassMatrix()
                ctx.synchronize()
                t = time.perf_counter()
                ctx.PicTimeStep(tol=wl.tol, maxit=400, precond=pc)
                ctx.synchronize()
                tp.append((time.perf_counter() - t) * 1e3)
            solve[nm].append(min(ts))
            step[nm].append(min(tp))
    ctx.close()
    med = lambda v: float(np.median(v))
    out = {"workload": workload, "dt": wl.dt, "tol": wl.tol, "pairs": info["samples"],
           "solves_harvested": info["solves"], "train_seconds": round(info["train_seconds"], 2),
           "loss_first_last": [info["loss"][0], info["loss"][-1]],
           "gmres_iterations": {k: iters[k] for k in iters},
           "field_solve_ms": {k: round(med(v), 3) for k, v in solve.items()},
           "ecsim_step_ms": {k: round(med(v), 3) for k, v in step.items()},
           "inference": "BF16 tcgen05 kernel, FP32 accumulate; flexible GMRES"}
    out["step_speedup_learned_vs_plain"] = round(out["ecsim_step_ms"]["plain"] /
                                                 out["ecsim_step_ms"]["learned"], 3)
    out["step_speedup_learned_vs_jacobi"] = round(out["ecsim_step_ms"]["jacobi"] /
                                                  out["ecsim_step_ms"]["learned"], 3)
    return out


def run_precond_kernel(args):
    """Inference of the block network alone (BF16 tcgen05 kernel) on
    args.precond_kernel random blocks: FLOP rate against the dense bf16 peak."""
    import amps_gb300 as A
    ws, rank, local = dist_env()
    wl = A.electron_proton_plasma("precond_kernel", 1, 1, 1, 1, 1)
    ctx = A.EcsimContext(wl, capacity=16, track_ids=False, device=local)
    ctx.precond_load(*A.init_precond_weights(seed=3, out_scale=1.0))
    rng = np.random.default_rng(1)
    S = args.precond_kernel
    x = rng.standard_normal((S, 1000, 3)).astype(np.float32)
    ctx.set_kernel_timing(True)
    for _ in range(args.warmup):
        ctx.precond_forward(x, tensor_cores=True)
    ctx.reset_kernel_times()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.precond_forward(x, tensor_cores=True)
    wall = time.perf_counter() - t0
    kt = ctx.kernel_times()
    ms, n = kt.get("precond_forward_tc", (float("nan"), 1))
    # useful FLOP per block (padded GEMM rows not counted): 2 x voxels x taps x cin x cout
    flop = 2 * 27 * (1000 * 3 * 32 + 1000 * 32 * 32 + 512 * 32 * 3)
    tflops = S * flop / (ms / n / 1e3) / 1e12
    d = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    peak = d.get("bf16_tflops", 1900.0)
    print(json.dumps({"metric": "precond inference (BF16 tcgen05)", "blocks": S, "steps": args.steps,
                      "kernel_ms_per_launch": ms / n, "useful_tflops": tflops,
                      "bf16_peak_tflops": peak, "frac": tflops / peak,
                      "wall_ms_per_call": wall * 1e3 / args.steps}), flush=True)
    ctx.close()


def tracer_line(n32, n64, device):
    """Batched relativistic test-particle tracing (cutoff workload): particle-steps/s
    in FP32 on n32 particles and FP64 on the first n64 of them; status agreement."""
    from amps_gb300 import tracer as T
    starts = T.sphere_starts(n32, 7)
    x32, p32, st32, s32, tot32, ms32 = T.trace_cutoff(n32, precision=1, device=device, starts=starts)
    # FP64 on the first n64 of the same particles
    x64, p64, st64, s64, tot64, ms64 = T.trace_cutoff(n64, precision=0, device=device, starts=starts)
    same = float(np.mean(st32[:n64] == st64))
    short = s64 < 10000
    same_short = float(np.mean(st32[:n64][short] == st64[short])) if short.any() else None
    return {"workload": "cutoff tracing: protons on r=1.1 R_E, isotropic, 0.1-20 GV log-uniform, "
                        "dipole B_eq=3.1e-5 T + 5 nT southward, stop r<1, r>10 R_E or 1e5 steps",
            "fp32": {"particles": n32, "particle_steps": int(tot32), "kernel_ms": ms32,
                     "particle_steps_per_s": tot32 / (ms32 / 1e3)},
            "fp64": {"particles": n64, "particle_steps": int(tot64), "kernel_ms": ms64,
                     "particle_steps_per_s": tot64 / (ms64 / 1e3)},
            "status_agreement_fp32_vs_fp64": same,
            "status_agreement_lifetime_below_1e4_steps": same_short,
            "status_fraction_fp32": {str(k): float(np.mean(st32[:n64] == k)) for k in (0, 1, 2)},
            "status_fraction_fp64": {str(k): float(np.mean(st64 == k)) for k in (0, 1, 2)},
            "status": "0 step budget, 1 r < 1 R_E, 2 r > 10 R_E"}


def restart_line(ctx):
    """Restart particle section of the bench state (SaveParticleData layout,
    basic 65-byte records) and the reference's particle CRC32 checksum, each
    through the C ABI with host buffers (wall clock); the section read back
    must give the same checksum."""
    from amps_gb300._capi import RecordLayout
    from amps_gb300.ecsim import PinnedArrays
    lay = RecordLayout.basic(False)
    ctx.particle_checksum(lay)
    t0 = time.perf_counter()
    ck = ctx.particle_checksum(lay)
    t1 = time.perf_counter()
    sec = ctx.write_restart_particles(lay)
    t2 = time.perf_counter()
    n = ctx.read_restart_particles(sec, lay)
    t3 = time.perf_counter()
    ck2 = ctx.particle_checksum(lay)
    gb = sec.size / 1e9
    out = {"particles": int(n), "section_bytes": int(sec.size), "checksum": "0x%x" % ck,
           "checksum_after_read_back_equal": ck == ck2,
           "checksum_ms": round((t1 - t0) * 1e3, 2), "checksum_records_per_s": n / (t1 - t0),
           "pageable": {"write_ms": round((t2 - t1) * 1e3, 2), "read_ms": round((t3 - t2) * 1e3, 2),
                        "write_gb_per_s": gb / (t2 - t1), "read_gb_per_s": gb / (t3 - t2)},
           "timing": "wall clock, host buffers, C ABI"}
    pin = PinnedArrays()
    try:
        buf = pin.empty(sec.size, np.uint8)
        ctx.write_restart_particles(lay, out=buf)
        t4 = time.perf_counter()
        ctx.write_restart_particles(lay, out=buf)
        t5 = time.perf_counter()
        ctx.read_restart_particles(buf, lay)
        t6 = time.perf_counter()
        out["page_locked"] = {"write_ms": round((t5 - t4) * 1e3, 2), "read_ms": round((t6 - t5) * 1e3, 2),
                              "write_gb_per_s": gb / (t5 - t4), "read_gb_per_s": gb / (t6 - t5),
                              "bytes_equal": bool(np.array_equal(buf, sec))}
    finally:
        pin.free()
    # the same CRC walk on one host core (the oracle's sequential restatement of
    # GetParticleDataCheckSum) over a 2M-record sample of synthetic particles
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from tests import oracle_lib as O
    m = 2_000_000
    rng = np.random.default_rng(0)
    xs, vs = rng.uniform(0, 64, (m, 3)), rng.standard_normal((m, 3))
    sp, blk, cel = np.zeros(m, np.uint8), np.zeros(m, np.int32), rng.integers(0, 512, m).astype(np.int32)
    t7 = time.perf_counter()
    O.particle_checksum(lay, 1, xs, vs, sp, blk, cel)
    t8 = time.perf_counter()
    out["cpu_baseline"] = {"checksum_records_per_s": m / (t8 - t7), "cores": 1, "kind": "port",
                           "sample": "oracle CRC32 walk over 2,000,000 synthetic 65-byte records"}
    return out


def cpu_leg(workload, device, tol=None):
    """The CPU baseline leg: one full ECSIM step (UpdateJMassMatrix, field
    solve, push + re-bin + deposit) of an AMR workload on the GPU and in the
    FP64 AMR oracle from the same particles (the oracle starts from the GPU's
    FP32-stored state).  Returns (cpu_baseline, parity): the oracle's push +
    deposit rate on one core, and the relative errors (max norm over the max
    entry) of fields, per-cell moments, particles and energies, with the
    block/cell mismatches checked against the face rule (tests/parity.py)."""
    import amps_gb300 as A
    from amps_gb300 import amr
    from tests import oracle_amr as OA
    from tests import parity as P
    wl = amr.AMR_WORKLOADS[workload]()
    tol = tol or wl.tol
    mesh = wl.mesh()
    ic = wl.initial_condition(mesh, seed=100, nthreads=os.cpu_count() or 8)
    n = len(ic["spec"])
    f = amr.amr_initial_fields(mesh, wl.b0)
    ctx = A.EcsimContext(wl.plasma, capacity=n, track_ids=True, device=device, amr_mesh=mesh)
    ctx.import_particles_local(ic["u"], ic["v"], ic["spec"], ic["block"], ic.get("wcorr"))
    ctx.import_fields(**f)
    e0 = ctx.export_particles()
    order = np.argsort(e0["id"])
    x0 = e0["x"][order]
    ctx.UpdateJMassMatrix()
    st = ctx.PicTimeStep(tol=tol, maxit=400, precond=1)
    cfl_gpu = ctx.particle_cfl()
    g = ctx.export_fields()
    gJ, gM = ctx.export_cell_moments()
    e1 = ctx.export_particles()
    o1 = np.argsort(e1["id"])
    ctx.close()
    wc = None if ic["wcorr"] is None else ic["wcorr"].astype(np.float64)
    ao = OA.AmrOracle(mesh, wl.species, wl.dt, wl.theta, x0, ic["v"].astype(np.float64), ic["spec"],
                      wcorr=wc)
    ao.Bcen[:] = f["B_center"]
    ao.Bprev[:] = f["B_corner_prev"]
    ao.Bcur[:] = f["B_corner_cur"]
    ao.deposit()
    it, wave = ao.field_solve(tol=tol, maxit=400)
    t0 = time.perf_counter()
    ao.push()
    t1 = time.perf_counter()
    pe = ao.deposit()
    t2 = time.perf_counter()

    def rel(a, b):
        den = np.max(np.abs(b))
        return float(np.max(np.abs(a - b)) / (den if den > 0 else 1.0))
    L = np.array(mesh.nfine, float) * mesh.dxf
    d = e1["x"][o1] - ao.x
    d -= L * np.rint(d / L)
    gb, gc = e1["block"][o1], e1["cell"][o1]
    rep = P.mismatch_report(e1["x"][o1], gb, gc, ao.x, ao.block, ao.cell, mesh.block_origins(),
                            mesh.block_dx(), L)
    same = (gb == ao.block) & (gc == ao.cell)
    # a particle filed in the neighbouring cell moves its contribution between
    # the two cells' partials (same corners, same corner moments): compare the
    # per-cell partials of the cells no such particle touches
    touched = np.zeros(mesh.ncells, bool)
    touched[(gb * 512 + gc)[~same]] = True
    touched[(ao.block * 512 + ao.cell)[~same]] = True
    keep = ~touched
    b0 = np.array(wl.b0)
    # the oracle's per-species CFL of the same particles (ProcessCell's cflCell)
    key = ao.block.astype(np.int64) * 512 + ao.cell
    cfl_orc = []
    for s in range(len(wl.species)):
        m = ao.spec == s
        u, inv = np.unique(key[m], return_inverse=True)
        sums = np.bincount(inv, weights=np.sqrt(np.sum(ao.v[m] ** 2, axis=1)) * wl.dt)
        cnt = np.bincount(inv)
        diag = np.sqrt(3.0) * mesh.block_dx()[u // 512]
        cfl_orc.append(float(np.max(sums / (cnt * diag))))
    parity = {
        "workload": workload, "particles": n, "tol": tol,
        "rel_err_E_n": rel(g["E_n"], ao.E_n), "rel_err_E_half": rel(g["E_half"], ao.E_half),
        "rel_err_B_center": rel(g["B_center"] - b0, ao.Bcen - b0),
        "rel_err_B_corner": rel(g["B_corner_cur"] - b0, ao.Bcur - b0),
        "rel_err_cell_J": rel(gJ.reshape(-1, 24)[keep], ao.cellJ.reshape(-1, 24)[keep]),
        "rel_err_cell_M": rel(gM.reshape(-1, 324)[keep], ao.cellM.reshape(-1, 324)[keep]),
        "cells_excluded_face_particles": int(touched.sum()),
        "max_position_err_dx0": float(np.max(np.abs(d)) / mesh.dx0),
        "rel_err_v": rel(e1["v"][o1], ao.v),
        "block_cell_mismatches": rep["mismatches"],
        "mismatch_max_offset_ulps": round(rep["max_offset_ulps"], 3),
        "face_rule_holds": rep["face_rule_holds"],
        "particle_energy_rel": abs(st.particle_energy - pe) / pe,
        "wave_energy_rel": abs(st.solve.wave_energy - wave) / wave,
        "cfl_rel": float(np.max(np.abs(cfl_gpu - np.array(cfl_orc)) / np.array(cfl_orc))),
        "gmres_iterations_gpu_oracle": [int(st.solve.iterations), int(it)],
        "norm": "max |gpu - oracle| / max |oracle| per array",
    }
    cpu = {"value": n / (t2 - t0), "unit": UNIT, "cores": 1, "kind": "port",
           "sample": "FP64 AMR oracle (Lapenta2017 + re-binning across levels + ProcessCell, "
                     "restated line by line and pinned to the reference's compiled ProcessCell/"
                     "Lapenta2017) on one core: one push + deposit of %s (%d particles), %.1f s"
                     % (workload, n, t2 - t0)}
    return cpu, parity


def field_solve_ab(ctx, tol, ev, stream, reps=3):
    """Jacobi vs learned field solve from the same state (fields restored
    between solves; the moments do not change): iterations and CUDA-event
    times."""
    f0 = ctx.export_fields()
    out = {}
    for pc, nm in ((1, "jacobi"), (2, "learned")):
        ms, its = [], []
        for _ in range(reps):
            ctx.import_fields(**f0)
            a, b = ev.event(), ev.event()
            ev.record(a, stream)
            st = ctx.TimeStep(tol=tol, maxit=400, precond=pc)
            ev.record(b, stream)
            ms.append(ev.elapsed_ms(a, b))
            its.append(st.iterations)
        out[nm] = {"iterations": its[-1], "ms": round(float(np.median(ms)), 3)}
    ctx.import_fields(**f0)
    out["speedup"] = round(out["jacobi"]["ms"] / out["learned"]["ms"], 3)
    return out


# ---------------------------------------------------------------------------
def run_gpu(args):
    import amps_gb300 as A
    ws, rank, local = dist_env()
    dist = init_dist(ws)
    ev = CudaEvents()
    ctx, info = setup_workload(args.workload, local)
    npart, ncell, nblk = info["particles"], info["cells"], info["blocks"]
    tol = info["tol"]
    if args.b_center:
        # the reference's default build: B seen by the particles from the cell centres
        ctx.set_b_center(True)
    info["b_field"] = "cell centres" if args.b_center else "corners"
    # one field solve so the push sees a self-consistent E^{n+theta}
    ctx.UpdateJMassMatrix()
    tuning = ctx.autotune()
    solve = ctx.TimeStep(tol=tol, maxit=200, precond=1)
    # the autotuner's arrivals comparison runs on the next particle steps
    while ctx.particle_tuning()["pending_steps"] > 0:
        ctx.push_deposit(want_energy=False)
    tuning.update(ctx.particle_tuning())
    stream = ctx.stream()
    ctx.set_graphs(args.graphs > 0)
    for _ in range(args.warmup):
        ctx.push_deposit(want_energy=False)
    ctx.synchronize()
    a, b = ev.event(), ev.event()
    clk = ClockSampler(local)
    barrier(dist)
    ev.sync()
    clk.start()
    ev.record(a, stream)
    for _ in range(args.steps):
        ctx.push_deposit(want_energy=False)
    ev.record(b, stream)
    ev.sync()
    ms = ev.elapsed_ms(a, b)
    clocks = clk.stop()
    barrier(dist)
    # per-kernel breakdown (roofline): the same steps again with event timing
    ctx.set_kernel_timing(True)
    ctx.reset_kernel_times()
    n_kt = max(3, args.steps // 4)
    for _ in range(n_kt):
        ctx.push_deposit(want_energy=False)
    ktimes = ctx.kernel_times()
    ctx.set_kernel_timing(False)
    value, ms_max = replica_throughput(dist, float(npart) * args.steps, ms)

    # full ECSIM step (field solve + push + deposit), Jacobi GMRES
    t_step = []
    for _ in range(2):
        a2, b2 = ev.event(), ev.event()
        ev.record(a2, stream)
        s = ctx.PicTimeStep(tol=tol, maxit=200, precond=1)
        ev.record(b2, stream)
        t_step.append(ev.elapsed_ms(a2, b2))
    gmres_it = s.solve.iterations

    # energy conservation over many full ECSIM steps (theta = 0.5)
    energy = None
    if args.energy_steps > 0:
        pc = args.energy_precond
        training = solve_ab = None
        if pc == 2:
            # the network learns from this run's own Jacobi solves (one weight
            # set per refinement level), then replaces Jacobi
            from amps_gb300 import precond as PC
            training = PC.train_in_situ(ctx, args.train_samples, tol=tol, epochs=20, batch=64,
                                        lr=2e-3, seed=0)
            ctx.precond_use_tensor_cores(True)
            solve_ab = field_solve_ab(ctx, tol, ev, stream)
        tot = []
        its = []
        t0 = time.perf_counter()
        for _ in range(args.energy_steps):
            s = ctx.PicTimeStep(tol=tol, maxit=400, precond=pc)
            tot.append(s.particle_energy + s.solve.wave_energy)
            its.append(s.solve.iterations)
        wall = time.perf_counter() - t0
        tot = np.array(tot)
        energy = {"steps": args.energy_steps, "precond": {1: "jacobi", 2: "learned"}[pc],
                  "total_energy_first": float(tot[0]),
                  "total_energy_last": float(tot[-1]),
                  "max_relative_drift": float(np.max(np.abs(tot - tot[0])) / abs(tot[0])),
                  "gmres_iterations_mean": float(np.mean(its)),
                  "wall_ms_per_step": wall * 1e3 / args.energy_steps,
                  "cuda_graphs": args.graphs > 0}
        if training is not None:
            energy["precond_training"] = training
            energy["field_solve_jacobi_vs_learned"] = solve_ab

    # end to end through the reference-facing C ABI with host FP64 buffers in
    # page-locked memory: per step the host hands in the fields the push and
    # the deposit read (E^{n+theta}, corner B prev/cur) and reads back the
    # moments the field solve needs: corner J and the 243-term corner mass
    # matrix, the node data UpdateJMassMatrix leaves at JxOffsetIndex /
    # MassMatrixOffsetIndex (on AMR meshes summed over the cells of every
    # unique corner) -- the drop-in for MoveParticles + UpdateJMassMatrix with
    # the particles resident on the device
    e2e = None
    e2e_particles = None
    if args.e2e_steps > 0:
        import amps_gb300 as A
        pin = A.PinnedArrays()
        f0 = ctx.export_fields()
        hf = {k: pin.empty(f0[k].shape) for k in ("E_half", "B_corner_prev", "B_corner_cur")}
        for k in hf:
            hf[k][:] = f0[k]
        hJ, hM = pin.empty((ctx.ncorners, 3)), pin.empty((ctx.ncorners, 243))
        # one untimed step first: the export's corner lists, copy stream and
        # per-block volumes are set up on its first call
        ctx.import_fields(**hf)
        ctx.push_deposit(want_energy=False)
        ctx.export_moments(out=(hJ, hM))
        ctx.synchronize()
        t_exp = 0.0  # the export calls alone (each returns with its copies complete)
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            ctx.import_fields(**hf)
            ctx.push_deposit(want_energy=False)
            t1 = time.perf_counter()
            ctx.export_moments(out=(hJ, hM))
            t_exp += time.perf_counter() - t1
        ctx.synchronize()
        e2e_s = time.perf_counter() - t0
        bi = int(sum(a.nbytes for a in hf.values()))
        bo = int(hJ.nbytes + hM.nbytes)
        e2e = {"value": npart * args.e2e_steps / e2e_s, "unit": UNIT,
               "h2d_bytes_per_step": bi, "d2h_bytes_per_step": bo, "steps": args.e2e_steps,
               "ms_per_step": round(e2e_s / args.e2e_steps * 1e3, 3),
               "export_ms": round(t_exp / args.e2e_steps * 1e3, 3),
               "export_gbs": round(bo * args.e2e_steps / t_exp / 1e9, 1),
               "host_memory": "page-locked (cudaHostAlloc)",
               "api": "amps_gpu_import_fields (E_half, B corner prev/cur) + amps_gpu_push_deposit + "
                      "amps_gpu_export_moments (corner J, M)"}
        pin.free()
        # the heavier round trip: every particle in and out through the FP64 AoS-style API
        exp = ctx.export_particles(ids=False)
        hx, hv, hs = exp["x"], exp["v"], exp["spec"]
        t0 = time.perf_counter()
        for _ in range(max(1, args.e2e_steps // 5)):
            ctx.import_particles(hx, hv, hs)
            ctx.push_deposit(want_energy=True)
            out = ctx.export_particles(ids=False)
            hx, hv = out["x"], out["v"]
        ctx.synchronize()
        tp = time.perf_counter() - t0
        e2e_particles = {"value": npart * max(1, args.e2e_steps // 5) / tp, "unit": UNIT,
                         "h2d_bytes_per_step": npart * 49, "d2h_bytes_per_step": npart * 57,
                         "host_memory": "pageable (numpy)",
                         "api": "amps_gpu_import_particles + amps_gpu_push_deposit + "
                                "amps_gpu_export_particles"}

    # roofline of the dominant kernel
    peak, peak_kind = measured_peaks()
    per = {k: v for k, v in ktimes.items()}
    top = max(per, key=lambda k: per[k][0])
    ms_top, launches = per[top]
    nl = max(1, launches)
    nbytes = kernel_bytes(npart, ncell, nblk, top, bool(args.b_center))
    traffic = args.traffic
    traffic_src = "--traffic" if traffic is not None else None
    if traffic is None and top in MEASURED_TRAFFIC.get(args.workload, {}):
        traffic = MEASURED_TRAFFIC[args.workload][top]
        traffic_src = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of this command, kernel "
                       "revision: " + MEASURED_TRAFFIC[args.workload]["version"])
    roof = None
    if nbytes:
        achieved = nbytes / (ms_top / nl / 1e3) / 1e9
        roof = {"kernel": top, "bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                "traffic": traffic, "traffic_source": traffic_src,
                "algorithmic_bytes_per_launch": int(nbytes),
                "avg_launch_ms": round(ms_top / nl, 4)}
        if top == "push_deposit":
            # the deposition is FP32-issue bound: its FP32 pipe rate beside the HBM one
            nsm = C.c_int()
            ev.rt.cudaDeviceGetAttribute(C.byref(nsm), 16, local)  # cudaDevAttrMultiProcessorCount
            mhz = (clocks or {}).get("sm_mhz") or 2070.0
            fp32_peak = nsm.value * 128 * 2 * mhz * 1e6 / 1e12
            tflops = npart * FLOP_PER_PARTICLE / (ms_top / nl / 1e3) / 1e12
            roof["fp32"] = {"achieved_tflops": round(tflops, 2), "peak_tflops": round(fp32_peak, 1),
                            "frac": round(tflops / fp32_peak, 4),
                            "flop_per_particle": FLOP_PER_PARTICLE,
                            "peak_source": "SMs x 128 FP32 lanes x 2 x median SM clock"}
    shares = {k: round(v[0] / sum(x[0] for x in per.values()), 4) for k, v in per.items()}
    # kernels per step (from the event-timed pass) x timed steps
    gpu_launches = int(round(sum(v[1] for v in per.values()) / n_kt * args.steps))

    cpu = parity = None
    if rank == 0 and ws == 1 and args.cpu_seconds > 0:
        if info["amr"]:
            cpu, parity = cpu_leg(args.parity_workload, local)
        else:
            rate, ci = cpu_replica_rate(args.workload, 1, args.cpu_seconds, 1)
            smp = "FP64 oracle Lapenta2017+ProcessCell on a periodic 8^3-cell replica of the " \
                  "same plasma (%d particles), %.1f s" % (ci["replica_particles"], ci["seconds"])
            cpu = {"value": rate, "unit": UNIT, "cores": 1, "kind": "port", "sample": smp}
    trc = None
    if rank == 0 and args.tracer > 0:
        trc = tracer_line(args.tracer, max(1, args.tracer // 256), local)
    rst = restart_line(ctx) if (rank == 0 and args.restart) else None
    pab = None
    if rank == 0 and args.precond_ab:
        pab = {"config": precond_ab("ecsim_32c_64ppc", local)}
        if args.precond_stiff:
            pab["stiff_dt_1_over_wpe"] = precond_ab("ecsim_32c_64ppc", local, dt=1.0)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (FP64 field solve)",
            "data": "synthetic (seeded Maxwellian electron-proton plasma, LCG of rnd.h)",
            "config": dict(info, **{
                "parallelism": "replicas" if ws > 1 else "single GPU",
                "l2": "inputs larger than L2 (no flush)",
                "ecsim_step_ms": round(min(t_step), 3), "gmres_iterations": gmres_it,
                "gmres_precond": "jacobi", "first_solve_iterations": solve.iterations,
                "cuda_graphs": args.graphs > 0, "autotune": tuning}),
            "e2e": e2e, "e2e_particle_roundtrip": e2e_particles,
            "roofline": roof, "kernel_shares": shares, "cpu_baseline": cpu, "parity": parity,
            "precond_ab": pab, "tracer": trc, "energy": energy, "restart": rst,
            "clocks": clocks, "gpu_launches": gpu_launches,
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()


def reference_amr_workload(name, threads, steps, warmup, budget):
    """The reference CPU path on the GPU arm's own AMR workload: the FP64 AMR
    oracle (Lapenta2017 + re-binning + ProcessCell, pinned to the reference's
    compiled ProcessCell/Lapenta2017) on `threads` host threads, one push +
    deposit per step.  Each step is a bounded sample of the workload: the
    particles of every m-th block, pushed, and those blocks' ProcessCell, with m
    the smallest stride at which the warm-up and timed steps take about `budget`
    seconds (m = 1, every particle, when the whole workload fits).  The sample's
    particles are put back before every step, outside the timed region, so
    every step does the same work.  Returns the per-step seconds, the particles
    per step, the stride and the workload's particle count."""
    from amps_gb300 import amr
    from tests import oracle_amr as OA
    wl = amr.AMR_WORKLOADS[name]()
    mesh = wl.mesh()
    ic = wl.initial_condition(mesh, seed=100, nthreads=threads)
    nb = mesh.nblocks
    f = amr.amr_initial_fields(mesh, wl.b0)

    def sample(m):
        sel = np.arange(nb) % m == 0
        pick = sel[ic["block"]]
        blk = ic["block"][pick]
        x = mesh.block_origins()[blk] + ic["u"][pick].astype(np.float64) * mesh.block_dx()[blk][:, None]
        wc = None if ic["wcorr"] is None else ic["wcorr"][pick].astype(np.float64)
        ao = OA.AmrOracle(mesh, wl.species, wl.dt, wl.theta, x, ic["v"][pick].astype(np.float64),
                          ic["spec"][pick], wcorr=wc)
        ao.Bprev[:] = f["B_corner_prev"]
        ao.Bcur[:] = f["B_corner_cur"]
        start = [a.copy() for a in (ao.x, ao.v, ao.block, ao.cell)]
        return ao, sel.astype(np.uint8), start

    # calibration on every 8th block: seconds per step of the whole workload
    ntot = len(ic["spec"])
    ao, sel, start = sample(8)
    t0 = time.perf_counter()
    ao.push_deposit_mt(threads, sel)
    full = (time.perf_counter() - t0) * ntot / len(ao.spec)
    m = max(1, int(np.ceil((steps + warmup) * full / budget)))
    if m != 8:
        del ao
        ao, sel, start = sample(m)
    del ic
    times = []
    for it in range(warmup + steps):
        for a, a0 in zip((ao.x, ao.v, ao.block, ao.cell), start):
            a[:] = a0
        t0 = time.perf_counter()
        ao.push_deposit_mt(threads, sel)
        if it >= warmup:
            times.append(time.perf_counter() - t0)
    return times, len(ao.spec), m, ntot


def run_reference(args):
    ws, rank, local = dist_env()
    if rank != 0:
        return
    from amps_gb300 import amr
    threads = os.cpu_count() or 1
    if args.workload in amr.AMR_WORKLOADS:
        times, n, m, ntot = reference_amr_workload(args.workload, threads, args.steps, args.warmup,
                                             args.ref_budget)
        value = n * len(times) / sum(times)
        part = ("all %d particles of %s, pushed, and ProcessCell of every block"
                % (n, args.workload) if m == 1 else
                "the %d particles of one block in %d of %s (%.3g of the workload), pushed, and "
                "those blocks' ProcessCell" % (n, m, args.workload, n / ntot))
        sample = ("FP64 AMR oracle (Lapenta2017 + re-binning across levels + ProcessCell, pinned to "
                  "the reference's compiled ProcessCell/Lapenta2017) on %d host threads (push over "
                  "particle ranges, deposit over block ranges): per step %s, %.2f s per step" %
                  (threads, part, sum(times) / len(times)))
        same = True
    else:
        rates = []
        for _ in range(args.steps):
            r, info = cpu_replica_rate(args.workload, 1, args.ref_seconds, threads)
            rates.append(r)
        value = float(np.mean(rates))
        sample = ("FP64 oracle port of Lapenta2017 + ProcessCell + re-binning, one periodic "
                  "8^3-cell replica of the same plasma per host thread (%d threads, %d particles "
                  "each), %g s per step" % (threads, info["replica_particles"], args.ref_seconds))
        same = False
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "same_config": same},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    # ~1 s of timed steps on the default workload, so that the clock sampler
    # (200 ms period) sees the timed region several times
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="amr_64c_128ppc")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--ref-seconds", type=float, default=8.0)
    ap.add_argument("--ref-budget", type=float, default=90.0,
                    help="reference arm on an AMR workload: seconds of warm-up + timed steps; "
                         "each step is a sample of the workload's blocks sized to fit")
    ap.add_argument("--precond-ab", type=int, default=1,
                    help="learned vs plain vs Jacobi GMRES on the 32^3 plasma (1 = on)")
    ap.add_argument("--precond-stiff", type=int, default=1,
                    help="also the same A/B at dt = 1/omega_pe")
    ap.add_argument("--graphs", type=int, default=1, help="particle step as a CUDA graph")
    ap.add_argument("--b-center", type=int, default=0,
                    help="1: the particles see B from the cell centres "
                         "(_PIC_FIELD_SOLVER_B_CENTER_BASED_; uniform workloads)")
    ap.add_argument("--oracle-check", action="store_true",
                    help="run only the CPU baseline leg (one full ECSIM step on the GPU and "
                         "the FP64 oracle, parity errors) on --parity-workload")
    ap.add_argument("--parity-workload", default="amr_64c_32ppc",
                    help="AMR workload of the CPU baseline leg: the headline mesh at 32 "
                         "particles per species per base cell by default (16.8M particles)")
    ap.add_argument("--energy-steps", type=int, default=50,
                    help="also run this many full ECSIM steps and report the energy drift "
                         "(0 = off)")
    ap.add_argument("--energy-precond", type=int, default=1, choices=(1, 2),
                    help="preconditioner of those steps: 1 Jacobi, 2 the learned network "
                         "(trained first on the run's own Jacobi solves)")
    ap.add_argument("--train-samples", type=int, default=20000,
                    help="block pairs harvested for the in-run training (--energy-precond 2)")
    ap.add_argument("--tracer", type=int, default=16777216,
                    help="also run the cutoff tracing workload with this many particles (FP32; "
                         "FP64 on 1/256 of them); 0 = off")
    ap.add_argument("--restart", type=int, default=1,
                    help="also time the restart particle section write/read and checksum")
    ap.add_argument("--precond-kernel", type=int, default=0,
                    help="time only the tensor-core inference kernel on this many blocks")
    ap.add_argument("--traffic", type=float, default=None,
                    help="DRAM bytes per launch of the top kernel from an ncu capture "
                         "(default: the committed capture of the default workload)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "gb300":
        args.warmup = 3
    if args.oracle_check:
        cpu, parity = cpu_leg(args.parity_workload, 0)
        print(json.dumps({"cpu_baseline": cpu, "parity": parity}), flush=True)
        return
    if args.impl == "reference":
        run_reference(args)
    elif args.precond_kernel > 0:
        run_precond_kernel(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
