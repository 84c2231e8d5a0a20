#!/usr/bin/env python
"""Throughput of the jax-sph hot path on GB300: particle-steps/s.

Workload: 3D Taylor-Green vortex, 64^3 = 262,144 particles on the periodic
(2 pi)^3 lattice, Wendland C2 kernel (h = dx, cutoff 2h), standard SPH with
transport velocity (tvf = 1), Re = 1600, float32, the reference's exact
neighbour set every step. One step = one si_euler step (kick, drift,
neighbour update, WCSPH forward, bc_fn). The neighbour update filters Verlet
candidates (cutoff plus a skin, rebuilt on the GPU's own decision once a
particle has moved half the skin) with the reference's membership test. Synthetic input: the reference's own initial condition
(lattice + analytic velocity field), built by ``jaxsph_gb300.cases.tgv``.

Default (our arm): resident rollout (``sph_step`` CUDA graphs), each timed step
bracketed by CUDA events on the launching stream, L2 flushed (256 MiB write)
between steps outside the events. ``--impl reference`` times the CPU
restatement of the reference step (the oracle; JAX itself is not installable
here) on all host threads. Under torchrun every rank runs an independent
replica (weak scaling, no collective on the data path).
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "jax-sph_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402
import torch  # noqa: E402

METRIC = "particle-steps/s on 1 GB300: batched/adjoint vs plain at stated FP64 error"
UNIT = "particle-steps/s"
WORKLOAD = ("3D Taylor-Green vortex 64^3 = 262,144 particles, periodic (2pi)^3, WC2K h=dx "
            "cutoff 2h, SPH + transport velocity (tvf=1), Re=1600, c0=10, float32, "
            "the reference's neighbour set every step")
# Algorithmic bytes per particle (float32 / int32), the minimum unique state traffic
STEP_BYTES = 128          # fused 3D TVF step: reads r,u,dudt,dvdt,m,eta,tag; writes r,u,v,dudt,dvdt,rho,p
FORCE_BYTES = 76          # force pass: reads r,m,u,v,rho,p,eta (52 B); writes dudt,dvdt (24 B)
DENSITY_BYTES = 24        # density pass: reads r,m (16 B); writes rho,p (8 B)
KICK_BYTES = 104          # kick-drift: reads r,m,u,v,dudt,dvdt,eta,tag (56 B); writes r,u,v (48 B)
# The kernels of one step, with their algorithmic bytes per particle and what
# one ncu capture of the same kernel on the 64^3 workload measured
# (profiles/lean_passes_tgv3d_64.md): DRAM bytes per particle per launch
# (dram__bytes_read.sum + dram__bytes_write.sum, cold caches), FMA-pipe and
# issue activity.
KERNELS = {
    "kick": {"kernel": "k_kick", "alg_bytes": KICK_BYTES,
             "ncu": {"dram_bytes": 100.6, "fma_pipe": 0.067, "issue_active": 0.280}},
    "rebuild": {"kernel": "k_hash_count + scan + k_scatter + k_permute + k_verlet_lean "
                          "(every few steps, per-step average)", "alg_bytes": None, "ncu": None},
    "density": {"kernel": "k_density_lean", "alg_bytes": DENSITY_BYTES,
                "ncu": {"dram_bytes": 118.4, "fma_pipe": 0.249, "issue_active": 0.658}},
    "force": {"kernel": "k_force_lean", "alg_bytes": FORCE_BYTES,
              "ncu": {"dram_bytes": 149.2, "fma_pipe": 0.426, "issue_active": 0.688}},
    # the force pass with its senders staged in shared memory (--force-variant staged)
    # (profiles/k_force_staged_tgv3d_64.md)
    "force_staged": {"kernel": "k_force_staged", "alg_bytes": FORCE_BYTES,
                     "ncu": {"dram_bytes": 153.2, "fma_pipe": 0.253, "issue_active": 0.523}},
}
# Status bits of the device status word (include/sph_gb300.h), for the line.
STATUS_BITS = {0x1: "NEIGHBOR_LIST_OVERFLOW", 0x2: "CELL_LIST_OVERFLOW",
               0x4: "CELL_SIZE_TOO_SMALL", 0x8: "MALFORMED_BOX", 0x100: "ERR_INVALID_ARG",
               0x200: "ERR_CUDA", 0x400: "ERR_TIMEOUT", 0x800: "ERR_NONFINITE",
               0x1000: "WARN_BOX_EDGE", 0x2000: "INFO_MOVED", 0x4000: "ERR_HOST"}


def status_report(code):
    """The status word of the timed steps, decoded. The two overflow bits are
    the reference's capacity tests (jax_md/partition.py:385-392, :956-976):
    its driver would allocate larger buffers and redo the step; here nothing
    is truncated on the GPU, so the steps' results stand and only the
    capacities are re-allocated (after the timed region)."""
    names = [v for k, v in STATUS_BITS.items() if code & k]
    out = {"word": code, "bits": names}
    if code & 0x3:
        out["note"] = ("reference capacity exceeded as the flow evolved: capacities "
                       "re-allocated after the timed steps; no result depends on them")
    return out


FP64_STEPS = 5  # steps of the float64 comparison run


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def init_dist(ws, backend):
    if ws > 1 and not torch.distributed.is_initialized():
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        torch.distributed.init_process_group(backend=backend)


def max_over_ranks(x, ws, device):
    if ws == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def barrier(ws):
    if ws > 1:
        torch.distributed.barrier()


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p is not None:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()

    def summary(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


# ------------------------------------------------------------------ CPU timings
def cpu_oracle_rate(n_side, max_steps, budget_s, threads, warmup=1, warmup_budget_s=60.0):
    """Oracle float32 si_euler steps on the same 3D TGV state, all host threads.

    ``warmup`` untimed steps run first (the first one allocates the neighbour
    list), stopping early once ``warmup_budget_s`` is spent; returns the rate,
    the timed steps, their seconds, the particle count and the warm-up steps
    that ran."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from jaxsph_gb300 import cases
    from oracle_setup import oracle_case
    import oracle

    torch.set_num_threads(threads)
    setup = cases.tgv(dim=3, dx=2 * np.pi / n_side)
    with torch.no_grad():  # a plain rollout: no autograd graphs kept
        solver, fns, bc, st = oracle_case(setup, torch.float32)
        nb = fns.allocate(st["r"])
        t0 = time.perf_counter()
        warm = 0
        while warm < max(1, warmup):
            st, nb = oracle.sph.si_euler_advance(setup.dt, setup.tvf, st, nb, fns, solver, bc)
            warm += 1
            if time.perf_counter() - t0 > warmup_budget_s:
                break
        t0 = time.perf_counter()
        steps = 0
        while steps < max_steps:
            st, nb = oracle.sph.si_euler_advance(setup.dt, setup.tvf, st, nb, fns, solver, bc)
            steps += 1
            if time.perf_counter() - t0 > budget_s:
                break
        dt = time.perf_counter() - t0
    return setup.n * steps / dt, steps, dt, setup.n, warm


def workload_config(args, n, ws):
    """The ``config`` object both arms print (identical dicts)."""
    return {"workload": (WORKLOAD if args.n_side == 64 else
                         WORKLOAD.replace("64^3 = 262,144", f"{args.n_side}^3 = {n:,}")),
            "n_particles": n, "parallelism": f"replicas x{ws}", "verlet_skin": args.skin,
            "l2": "flushed between timed steps (256 MiB write outside the events)"}


def fp64_error(setup, steps, device, threads):
    """The GPU rollout's error against a float64 run: ``steps`` si_euler steps
    of the case on the GPU (float32) and in the float64 oracle (the CPU
    restatement of the reference step) from the same initial state; max over
    particles of |r - r64| (minimum image) / box, |u - u64| / max|u64| and
    |rho - rho64| / rho_ref."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from jaxsph_gb300 import simulate
    from oracle_setup import oracle_rollout
    import oracle

    sim = simulate.Simulation(setup, device=device)
    sim.run(steps, check_every=1)
    got = sim.state()[0]
    del sim
    torch.set_num_threads(threads)
    with torch.no_grad():
        ref = oracle_rollout(setup, steps, torch.float64)
        ref32 = oracle_rollout(setup, steps, torch.float32)
    side = torch.as_tensor(setup.box, dtype=torch.float64)

    def errors(st):
        dr = oracle.space.periodic_displacement(side, st["r"].double().cpu() - ref["r"])
        return {"r_max_over_box": float(dr.abs().max() / side.max()),
                "u_max_rel": float((st["u"].double().cpu() - ref["u"]).abs().max()
                                   / ref["u"].abs().max()),
                "rho_max_rel": float((st["rho"].double().cpu() - ref["rho"]).abs().max()
                                     / setup.eos.rho_ref)}

    # the float32 oracle's own distance from the float64 run: what float32
    # rounding of the same algorithm alone gives
    return dict(errors(got), steps=steps,
                against="float64 oracle (CPU restatement of the reference step)",
                float32_oracle=errors(ref32))


def reference_arm(args, ws, rank):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    rate, steps, secs, n, warm = cpu_oracle_rate(64, max(1, args.steps), 150.0, threads,
                                                 warmup=max(3, args.warmup))
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": args.gpus,
        "steps": steps, "warmup": warm, "ms_per_step": 1000.0 * secs / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (reference initial condition of the 3D TGV)",
        "config": workload_config(args, n, args.gpus),
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{steps} float32 oracle si_euler steps of the full 64^3 "
                                   f"case (time-bounded, 150 s budget, after {warm} warm-up "
                                   f"steps)"},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "reference jax[cpu] is not installable here (no JAX, no network); "
                "the oracle restatement of the reference step stands in",
    }
    print(json.dumps(line))


# ------------------------------------------------------------------ GPU arm
def e2e_rate(setup, steps, device):
    """The public drop-in API with host buffers: every step the ``si_euler``
    advance takes its state from pinned host memory and returns the new state
    in pinned host memory (DMA copies in and out inside the one library
    call, which returns once the result is in host memory)."""
    from jaxsph_gb300 import integrator, simulate

    wc = simulate.make_solver(setup)
    fns = simulate.make_neighbor_fns(setup, wc)
    _, shift = setup.space()
    adv = integrator.si_euler(setup.tvf, wc.forward_wrapper(), shift, setup.bc_fn, None)
    keys_in = ("r", "tag", "u", "v", "dudt", "dvdt", "drhodt", "rho", "p", "mass", "eta", "nw")
    host = {k: setup.state[k].to(torch.int32 if k == "tag" else torch.float32)
            .contiguous().pin_memory() for k in keys_in}
    # the bytes that cross the host link each step: the step reads neither v
    # (the kick recomputes it), the old p, drho/dt (a summation carries it
    # over) nor nw (no walls); the results are r, u, v, dudt, dvdt, rho, p
    moved_in = ("r", "tag", "u", "dudt", "dvdt", "rho", "mass", "eta")
    moved_out = ("r", "u", "v", "dudt", "dvdt", "rho", "p")
    h2d = sum(host[k].numel() * host[k].element_size() for k in moved_in)
    d2h = sum(host[k].numel() * host[k].element_size() for k in moved_out)
    nb = fns.allocate(host["r"])
    st = host
    for _ in range(3):  # warm-up (engine creation, pinned output blocks)
        st, nb = adv(setup.dt, st, nb)
    torch.cuda.synchronize()
    assert all(st[k].device.type == "cpu" and st[k].is_pinned() for k in moved_out)
    times, redone = [], 0
    for _ in range(steps):
        t0 = time.perf_counter()
        st_new, nb_new = adv(setup.dt, st, nb)
        if nb_new.did_buffer_overflow:
            # the reference driver's protocol (simulate.py:118-128): allocate
            # at the step's input positions and redo the step
            nb = fns.allocate(st["r"])
            st_new, nb_new = adv(setup.dt, st, nb)
            redone += 1
        st, nb = st_new, nb_new
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    t = float(np.mean(times))
    return setup.n / t, h2d, d2h, t, redone


def timed_steps(sim, steps):
    """Per-step CUDA-event times (ms) of a resident Simulation."""
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    torch.cuda.synchronize()
    for k in range(steps):
        starts[k].record()
        sim.engine.step(1)
        ends[k].record()
    torch.cuda.synchronize()
    return [s.elapsed_time(e) for s, e in zip(starts, ends)]


def batched_form(device, steps, n_instances=256, fp64=True):
    """The batched form on its own workload: 256 cavity/channel instances with
    log-uniform particle counts as one resident batch (one CUDA graph per step,
    autotuned block size) versus the same instances run one after another on
    the plain per-instance path."""
    from jaxsph_gb300 import cases, simulate

    batch = cases.cavity_channel_batch(n_instances, seed=0)
    n_total = sum(s.n for s in batch)
    sim = simulate.Simulation(batch, device=device, autotune=True)
    sim.run(3, check_every=1)
    ms = timed_steps(sim, steps)  # the batch state (~1 GB) exceeds L2
    batched = n_total * steps / (sum(ms) * 1e-3)
    plain_ms, plain_steps = 0.0, max(3, steps // 10)
    diffs = []
    for s in batch:
        one = simulate.Simulation(s, device=device)
        one.run(3, check_every=1)
        plain_ms += sum(timed_steps(one, plain_steps)) / plain_steps
        del one
    # bit-for-bit agreement of batched and plain runs on a sample of instances
    # (canonical pair order: the batch rebuilds candidate lists when any of
    # its cases needs it)
    check = simulate.Simulation(batch, device=device, canonical_order=True)
    check.run(5)
    ref_states = check.state()
    for k in (0, 1, n_instances // 2, n_instances - 1):
        one = simulate.Simulation(batch[k], device=device, canonical_order=True)
        one.run(5)
        a, b = ref_states[k], one.state()[0]
        diffs.append(max(float((a[x].double() - b[x].double()).abs().max()) for x in ("r", "u", "rho")))
    errors = None
    if fp64:
        # the batched result against float64 runs of the same instances
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        from oracle_setup import oracle_rollout
        import oracle

        errs = {"r_max_over_box": 0.0, "u_max_rel": 0.0, "rho_max_rel": 0.0}
        with torch.no_grad():
            for k in (0, n_instances - 1):
                ref = oracle_rollout(batch[k], 5, torch.float64)
                got = ref_states[k]
                side = torch.as_tensor(batch[k].box, dtype=torch.float64)
                dr = oracle.space.periodic_displacement(side, got["r"].double().cpu() - ref["r"])
                scale_u = max(float(ref["u"].abs().max()), batch[k].u_ref)
                e = {"r_max_over_box": float(dr.abs().max() / side.max()),
                     "u_max_rel": float((got["u"].double().cpu() - ref["u"]).abs().max())
                                  / scale_u,
                     "rho_max_rel": float((got["rho"].double().cpu() - ref["rho"]).abs().max()
                                          / batch[k].eos.rho_ref)}
                errs = {x: max(errs[x], e[x]) for x in errs}
        errors = dict(errs, steps=5, instances=[0, n_instances - 1],
                      against="float64 oracle (CPU restatement of the reference step)")
    per_instance = n_total / (plain_ms * 1e-3)
    return {"workload": f"{n_instances} lid-driven cavities / Poiseuille channels (2D, QSK, SPH, "
                        f"wall BC), fluid particles log-uniform 1e3-4e4, {n_total:,} particles",
            "value": batched, "unit": UNIT, "steps": steps, "block_size": sim.block_size,
            "per_instance_value": per_instance, "speedup_vs_per_instance": batched / per_instance,
            "max_abs_diff_vs_per_instance": max(diffs),
            "launches_per_step": sim.engine.launch_count(), "error_vs_fp64": errors}


def oracle_gradient(setup, u0, target, steps):
    """Loss and gradient w.r.t. u0 through the float64 oracle rollout, the
    neighbour list frozen per step (jax.grad(..., allow_int=True))."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from jaxsph_gb300 import adjoint
    from oracle_setup import oracle_case
    import oracle

    solver, fns, bc, st = oracle_case(setup, torch.float64)
    u = u0.detach().double().cpu().clone().requires_grad_(True)
    st = dict(st, u=u, v=u)
    nb = fns.allocate(st["r"].detach())
    side = torch.as_tensor(setup.box, dtype=torch.float64)
    for _ in range(steps):
        st = dict(st)
        st["u"] = st["u"] + setup.dt * st["dudt"]
        st["v"] = st["u"] + setup.tvf * 0.5 * setup.dt * st["dvdt"]
        st["r"] = oracle.space.periodic_shift(side, st["r"], setup.dt * st["v"])
        nb = fns.update(st["r"].detach(), nb)
        st = bc(solver.forward(st, nb.idx))
    loss = adjoint.position_mse(st["r"], target.double().cpu(), setup.box)
    (g,) = torch.autograd.grad(loss, u)
    return float(loss), g


def _min_image(d, box):
    side = torch.as_tensor(box, dtype=d.dtype, device=d.device)
    return d - side * torch.round(d / side)


def adjoint_form(device, steps=100, checkpoint_every=10, fp64=True):
    """The differentiable form on its own workload: gradient of the final
    positions' mean squared distance to a target rollout (another seed) with
    respect to the initial velocity of a 128^2 perturbed 2D TGV, through the
    hand-written adjoint with checkpointing, versus the plain forward rollout."""
    from jaxsph_gb300 import adjoint, cases, simulate

    a = cases.tgv_perturbed(n_side=128, seed=1)
    b = cases.tgv_perturbed(n_side=128, seed=2)
    target = adjoint.AdjointRollout(b, steps, checkpoint_every).forward(b.state["u"].to(device))
    roll = adjoint.AdjointRollout(a, steps, checkpoint_every, device=device, autotune=True)
    u0 = a.state["u"].to(device)

    def gradient():
        u = u0.clone().requires_grad_(True)
        loss = adjoint.position_mse(adjoint.rollout(u, roll), target, a.box)
        (g,) = torch.autograd.grad(loss, u)
        return loss, g

    # warm-up: one whole gradient (graphs, allocations, the autograd engine's
    # and torch's own first-use costs stay out of the timed region)
    gradient()
    torch.cuda.synchronize()
    reps = 3
    t0 = time.perf_counter()
    for _ in range(reps):
        loss, g = gradient()
    torch.cuda.synchronize()
    t_grad = (time.perf_counter() - t0) / reps
    # where a gradient's time goes (CUDA events on the current stream): the
    # forward rollout with its checkpoints, the recomputation of every
    # segment with its tape, and the reverse sweeps
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record()
    r_final = roll.forward(u0)
    f1.record()
    segs = []
    # d/dr of the mean squared minimum-image distance
    lam_r = 2.0 * _min_image(r_final - target, a.box) / a.n
    roll.backward(lam_r, timer=segs)
    torch.cuda.synchronize()
    phases = {"forward_rollout_ms": f0.elapsed_time(f1),
              "recompute_with_tape_ms": sum(e[0].elapsed_time(e[1]) for e in segs),
              "reverse_sweep_ms": sum(e[1].elapsed_time(e[2]) for e in segs)}
    err = None
    if fp64:
        loss64, g64 = oracle_gradient(a, u0, target, steps)
        err = {"grad_rel_l2": float((g.double().cpu() - g64).norm() / g64.norm()),
               "loss_rel": abs(float(loss) - loss64) / abs(loss64),
               "against": "torch autograd through the float64 oracle rollout "
                          "(neighbour lists frozen per step)"}
    plain = simulate.Simulation(a, device=device, autotune=True)
    plain.run(3)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plain.run(steps)
    torch.cuda.synchronize()
    t_plain = time.perf_counter() - t0
    return {"workload": f"2D TGV 128^2 = {a.n:,} particles, TGV + Fourier perturbation "
                        f"(sigma 0.1, |k| <= 8), SPH tvf=0 QSK, {steps}-step rollout, "
                        f"gradient of the final-position MSE w.r.t. the initial velocity",
            "value": a.n * steps / t_grad, "unit": UNIT,
            "note": "forward (with checkpoints) + reverse sweep, wall clock",
            "checkpoint_every": checkpoint_every, "block_size": roll.sim.block_size,
            "plain_block_size": plain.block_size, "loss": float(loss.detach()),
            "grad_norm": float(g.norm()), "timed_gradients": reps,
            "phases": dict(phases, plain_rollout_ms=1e3 * t_plain),
            "plain_forward_value": a.n * steps / t_plain,
            "ratio_vs_plain_forward": t_plain / t_grad, "error_vs_fp64": err}


def gpu_arm(args, ws, rank, local):
    from jaxsph_gb300 import _lib, cases, simulate

    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    setup = cases.tgv(dim=3, dx=2 * np.pi / args.n_side)
    sim = simulate.Simulation(setup, device=device, skin=args.skin)
    variants = {"gather": _lib.FORCE_GATHER, "staged": _lib.FORCE_STAGED}
    sim.engine.set_force_variant(variants[args.force_variant])
    # warm-up through run(): it polls the status word and re-allocates the
    # capacities on overflow, as the reference driver does
    sim.run(max(args.warmup, 3), check_every=1)
    torch.cuda.synchronize()
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=device)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    rebuilds0, per_rebuild = sim.engine.rebuild_stats()
    barrier(ws)
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        for k in range(args.steps):
            flush.fill_(k & 0xFF)
            starts[k].record()
            sim.engine.step(1)
            ends[k].record()
        torch.cuda.synchronize()
    barrier(ws)
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = max_over_ranks(float(np.sum(step_ms)), ws, device)
    status = sim.engine.read_status(clear=False)
    sim._poll()  # the reference driver's response: re-allocate on an overflow bit
    rebuilds = sim.engine.rebuild_stats()[0] - rebuilds0
    launches = sim.engine.launch_count() * args.steps + rebuilds * per_rebuild
    n = setup.n
    value = n * args.steps * ws / (total_ms / 1000.0)
    # per-kernel times, measured with CUDA events on the stream the kernels
    # are launched on (eager steps; the host reads each rebuild decision)
    _, dens_ms, _, force_ms, kick_ms, rb_ms = sim.engine.profile(20, split=True)
    # the other force-pass variant on the same state (same results, other time)
    other = "staged" if args.force_variant == "gather" else "gather"
    sim.engine.set_force_variant(variants[other])
    force_other_ms = sim.engine.profile(20, split=True)[3]
    sim.engine.set_force_variant(variants[args.force_variant])
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        peaks = json.load(open(peaks_path))
        hbm, peak_src = float(peaks["hbm_gbs"]), "measured"
    else:
        hbm, peak_src = 6800.0, "fallback"
    times = {"kick": kick_ms, "rebuild": rb_ms, "density": dens_ms, "force": force_ms}
    kernels = dict(KERNELS)
    if args.force_variant == "staged":
        kernels["force"] = dict(KERNELS["force_staged"])
    table = {}
    for name, ms in times.items():
        k = kernels[name]
        row = {"kernel": k["kernel"], "ms": ms, "alg_bytes_per_particle": k["alg_bytes"]}
        if k["alg_bytes"] and ms > 0:
            gbs = k["alg_bytes"] * n / (ms * 1e-3) / 1e9
            row.update(achieved_gbs=gbs, frac=gbs / hbm)
        if k["ncu"]:
            row["ncu"] = k["ncu"]
        table[name] = row
    # the dominant single kernel (the rebuild is several kernels)
    dom = max(("kick", "density", "force"), key=lambda x: times[x])
    d = table[dom]
    ncu = kernels[dom]["ncu"] or {}
    step_ms_mean = total_ms / args.steps
    step_achieved = STEP_BYTES * n / (step_ms_mean * 1e-3) / 1e9
    cfg = workload_config(args, n, ws)  # identical to the reference arm's
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": step_ms_mean, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (reference initial condition of the 3D TGV)",
        "config": cfg,
        # the dominant kernel's algorithmic bytes over its CUDA-event time,
        # against the measured HBM copy bandwidth; what binds it is the
        # instruction issue (ncu: issue active, FMA pipe), not DRAM
        "roofline": {"bound": "issue", "kernel": d["kernel"], "achieved": d.get("achieved_gbs"),
                     "peak": hbm, "unit": "GB/s", "frac": d.get("frac"),
                     "peak_source": peak_src + " HBM copy bandwidth",
                     "alg_bytes_per_particle": d["alg_bytes_per_particle"],
                     "traffic": (ncu["dram_bytes"] * n if ncu.get("dram_bytes") else None),
                     "traffic_source": "ncu dram bytes per particle of the same kernel at 64^3",
                     "fp32_pipe_frac": ncu.get("fma_pipe"),
                     "issue_active": ncu.get("issue_active"),
                     "step": {"alg_bytes_per_particle": STEP_BYTES, "achieved": step_achieved,
                              "frac": step_achieved / hbm}},
        "kernels": table,
        "force_variant": args.force_variant,
        "force_variants_ms": {args.force_variant: force_ms, other: force_other_ms},
        "candidate_rebuilds": rebuilds,
        "status": status_report(status),
        "gpu_launches": launches,
        "clocks": clocks.summary(),
    }
    del sim
    threads = os.cpu_count() or 1
    if rank == 0 and ws == 1 and not args.no_cpu:
        line["error_vs_fp64"] = fp64_error(setup, FP64_STEPS, device, threads)
    if rank == 0 and ws == 1 and not args.no_e2e:
        rate, h2d, d2h, t, redone = e2e_rate(setup, min(args.steps, 30), device)
        line["e2e"] = {"value": rate, "unit": UNIT, "h2d_bytes_per_step": h2d,
                       "d2h_bytes_per_step": d2h, "steps_redone_on_overflow": redone,
                       "path": "si_euler drop-in advance on a pinned host state: each step "
                               "reads its inputs from and writes its result to host memory"}
    forms = [] if args.no_forms else [f for f in args.forms.split(",") if f]
    if rank == 0 and forms:
        line["forms"] = {}
        if "batched" in forms:
            line["forms"]["batched"] = batched_form(device, args.batched_steps,
                                                    fp64=not args.no_cpu)
        if "adjoint" in forms:
            line["forms"]["adjoint"] = adjoint_form(device, fp64=not args.no_cpu)
    if rank == 0 and ws == 1 and not args.no_cpu:
        # a bounded sample: steps of the full case until ~10 s of CPU work
        rate, steps, secs, n_cpu, warm = cpu_oracle_rate(64, 40, 10.0, threads, warmup=3,
                                                         warmup_budget_s=10.0)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": f"{steps} float32 oracle si_euler step(s) of the full "
                                          f"64^3 case after {warm} warm-up step(s) "
                                          f"({secs:.1f} s)"}
    if rank == 0:
        print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    # the configuration's rollout: 500 steps of the 3D TGV
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the batched/adjoint form measurements on their own workloads")
    ap.add_argument("--forms", default="batched,adjoint",
                    help="comma-separated forms to measure on their own workloads")
    ap.add_argument("--skin", type=float, default=0.1,
                    help="Verlet skin as a fraction of the cutoff (0: rebuild every step)")
    ap.add_argument("--batched-steps", type=int, default=1000,
                    help="steps of the batched form (the configuration's 1,000)")
    ap.add_argument("--force-variant", default="gather", choices=["gather", "staged"],
                    help="how the force pass reads its senders: gathered from global memory "
                         "(default) or staged in shared memory one plane of cells at a time")
    ap.add_argument("--n-side", type=int, default=64,
                    help="particles per side of the 3D TGV lattice (64 = the benchmark case)")
    args = ap.parse_args()
    ws, rank, local = dist_env()
    if args.impl == "reference":
        init_dist(ws, "gloo")
        reference_arm(args, ws, rank)
        return
    init_dist(ws, "nccl")
    gpu_arm(args, ws, rank, local)
    if ws > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
