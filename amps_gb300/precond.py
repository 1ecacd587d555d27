"""Training workflow of the learned GMRES preconditioner (the kernels and the
C ABI are amps_gpu_precond_* in include/amps_gpu.h).

harvest_training_pairs: Jacobi field solves on seeded random plasma states of a
uniform workload, with the context harvesting (A e, e) block pairs from every
Arnoldi step and (b, x) from every converged solve.
train: Adam on the device with the library's own forward/backward kernels.
train_in_situ: the same on the context's own run (any mesh): Jacobi ECSIM
steps harvest the pairs, then every weight set (one per refinement level) is
trained on the pairs of its level.
"""
import time

import numpy as np

from .ecsim import (PRECOND_SHAPES, EcsimContext, init_precond_weights, initial_fields,
                    make_initial_condition)


def random_state(ctx, wl, seed, e_amp=0.0, b_amp=0.0):
    """Seeded plasma (Maxwellian particles of wl with this seed) plus optional
    random corner/centre field perturbations; deposits the moments."""
    wl.seed = int(seed)
    ic = make_initial_condition(wl, nthreads=8)
    ctx.import_particles_local(ic["u"], ic["v"], ic["spec"], ic["block"])
    f = initial_fields(wl)
    if e_amp > 0.0 or b_amp > 0.0:
        rng = np.random.default_rng(seed)
        n = wl.mesh.ncells
        f["E_n"] = f["E_n"] + e_amp * rng.standard_normal((n, 3))
        for k in ("B_center", "B_corner_prev", "B_corner_cur"):
            f[k] = f[k] + b_amp * rng.standard_normal((n, 3))
    ctx.import_fields(**f)
    ctx.UpdateJMassMatrix()
    return ic


def harvest_training_pairs(ctx, wl, nsamples, seed0=1000, steps_per_state=4, tol=1e-8,
                           e_amp=0.0, b_amp=0.0):
    """Fill the context's sample buffer with nsamples block pairs from Jacobi
    solves (ECSIM steps of several seeded states).  Returns the number of
    solves and states used."""
    ctx.precond_harvest(nsamples)
    solves = states = 0
    while ctx.precond_num_samples() < nsamples:
        random_state(ctx, wl, seed0 + states, e_amp, b_amp)
        states += 1
        for _ in range(steps_per_state):
            ctx.PicTimeStep(tol=tol, maxit=400, precond=1)
            solves += 1
            if ctx.precond_num_samples() >= nsamples:
                break
    return {"solves": solves, "states": states, "samples": ctx.precond_num_samples()}


def train(ctx, epochs=20, batch=64, lr=1e-3, seed=1):
    t0 = time.time()
    loss = ctx.precond_train(epochs, batch, lr, seed)
    ctx.synchronize()
    return loss, time.time() - t0


def train_in_situ(ctx, nsamples, tol=1e-8, max_steps=20, epochs=20, batch=64, lr=2e-3, seed=0):
    """Harvest nsamples block pairs from the context's own Jacobi ECSIM steps
    (at most max_steps; the run advances), then train each weight set on the
    pairs of its level from seeded initial weights.  Returns a summary."""
    t0 = time.time()
    ctx.precond_harvest(nsamples)
    steps = 0
    while ctx.precond_num_samples() < nsamples and steps < max_steps:
        ctx.PicTimeStep(tol=tol, maxit=400, precond=1)
        steps += 1
    n = ctx.precond_num_samples()
    sets = ctx.precond_sample_sets(0, n)
    t_h = time.time() - t0
    out = {"harvest_steps": steps, "samples": int(n), "harvest_seconds": round(t_h, 2),
           "epochs": epochs, "batch": batch, "sets": []}
    t1 = time.time()
    for s in range(ctx.precond_num_sets()):
        ns = int(np.sum(sets == s))
        ctx.precond_select(s)
        ctx.precond_load(*init_precond_weights(seed + s))
        entry = {"set": s, "samples": ns}
        if ns > 0:
            loss = ctx.precond_train(epochs, min(batch, ns), lr, seed + 100 + s)
            entry["loss_first_last"] = [float(loss[0]), float(loss[-1])]
        else:
            ctx.precond_load(*[np.zeros(shp, np.float32) for shp in PRECOND_SHAPES])
        out["sets"].append(entry)
    ctx.precond_select(0)
    ctx.synchronize()
    out["train_seconds"] = round(time.time() - t1, 2)
    ctx.precond_harvest(0)
    return out


def build_trained_context(wl, nsamples=20000, epochs=20, batch=64, lr=1e-3, seed=0,
                          capacity=None, device=0, e_amp=0.0, b_amp=0.0):
    """Context for wl with a network trained on nsamples harvested pairs."""
    ctx = EcsimContext(wl, capacity=capacity or wl.nparticles, track_ids=False, device=device)
    ctx.precond_load(*init_precond_weights(seed))
    t0 = time.time()
    info = harvest_training_pairs(ctx, wl, nsamples, e_amp=e_amp, b_amp=b_amp)
    info["harvest_seconds"] = time.time() - t0
    loss, secs = train(ctx, epochs, batch, lr, seed + 1)
    info.update({"loss": loss.tolist(), "train_seconds": secs, "epochs": epochs, "batch": batch})
    ctx.precond_harvest(0)
    return ctx, info
