"""Benchmark: FP64-accurate energy+gradient evaluations per second on one GB300.

Workload (metric "grad evals/s" on one GB300 at 163k vertices): a level-7
icosphere (163,842 vertices, 327,680 faces), vertices jittered by 13% of the
mean edge length (seed 0), the energy of the very-large-mesh configuration
(kb 20, ka 1e6, kv 1e6, kc 0, kt 1e5, kr 1e3, reduced-volume target 0.65,
smooth tether lc0/lc1 = 1.15/0.85 mean edge, repulsion cut-off 0.8 mean edge
via the cell list, exclusion 2).  One step = 10 x (positions displaced by
N(0, 1e-4), one energy+gradient evaluation) + one cell-list rebuild, the
evaluation loop of the large-mesh configuration applied to the 163k mesh.
The displacements are drawn before timing (a pool of 10, applied with the
sign alternating from step to step so the positions do not drift).

value:  device-resident evaluations (positions, gradient and energy in HBM),
        every evaluation and rebuild timed with CUDA events on the launching
        stream, L2 flushed (256 MB write) before each timed piece; the
        stencils in double-word arithmetic on the FP32 pipe (the library's
        default; FP64 results within 1e-10 of the FP64 oracle, tested at this
        mesh), FP64 global sums and penalties.
e2e:    the same evaluations through the public API as the reference's
        drivers call it (trimem_gb300.core: write the positions into
        TriMesh.points(), EnergyManager.energy and .gradient), i.e. host
        positions uploaded and the gradient read back every evaluation; the
        fused energy_gradient call beside it.
cpu_baseline / --impl reference: the reference algorithm restated on the
        host cores (the reference itself cannot be built: its OpenMesh
        submodule is empty), all threads, energy() + gradient() per
        evaluation like the reference's Python drivers (built -O3 -fopenmp
        with FP contraction; the parity build's rate beside it); chain_step:
        chain steps of the same restatement from the chains' start state.

Secondary objects on the same line (measured after the timed region):
roofline        the whole evaluation against HBM (132 algorithmic bytes
                per vertex), per-stage times of one cold evaluation (CUDA
                events inside the library), DRAM traffic and issue-slot
                activity from the committed ncu summary
fp32_stencil, df64_stencil   the other stencil precisions: time and error
surrogate_force the learned force: time, and its tensor-core FLOP rate
level6          the 40,962-vertex evaluation loop, GPU and CPU
batch_replicas  64 membranes of 642-40,962 vertices in one batch
hmc_chain       device chains (HMC move + flip sweep, 2,000 steps) from the
                committed equilibrated state of the 0.65-target membrane:
                per-move times, acceptance, ESS/s of the bending energy and
                the reduced volume, quarter means and a drift test of the
                bending trace
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

LEVEL = 7
EVALS_PER_STEP = 10
# stencil precision of the headline evaluations (tm_energy_set_stencil_precision)
HEADLINE_STENCIL = 2
METRIC = "grad evals/s (FP64 energy+gradient, 163,842-vertex icosphere)"
UNIT = "evals/s"


def workload():
    from trimem_gb300.workloads import very_large_mesh

    return very_large_mesh()


def config():
    return {"workload": "icosphere L7 (163842 vertices), FP64 energy+gradient, cell-list rebuild every 10 evals, "
                        "N(0,1e-4) displacement between evals (pre-drawn pool of 10, sign alternating per step)",
            "vertices": 163842, "faces": 327680, "evals_per_step": EVALS_PER_STEP,
            "l2": "flushed (256 MB write) before every timed evaluation and rebuild",
            "parallelism": "replicas"}


# the committed ncu summary of the headline (double-word) evaluation's
# stages: DRAM bytes per stage and the issue-slot activity of each stage's
# main kernel
TRAFFIC_PROFILE = "profiles/eval_kernels_L7_df64_sections.md"
PIPE_NAME = "issue"
PIPE_METRIC = "smsp__issue_active"


def read_traffic():
    """DRAM bytes per launch of each evaluation stage, and the pipe activity
    of its main kernel (percent), from the committed ncu summary
    TRAFFIC_PROFILE: lines "<stage> <bytes>" and "<pipe> <stage> <pct>"."""
    out, pipe = {}, {}
    try:
        for line in open(os.path.join(ROOT, TRAFFIC_PROFILE)):
            parts = line.split()
            if len(parts) == 2 and parts[0].startswith("k_") and parts[1].isdigit():
                out[parts[0]] = int(parts[1])
            if len(parts) == 3 and parts[0] == PIPE_NAME and parts[1].startswith("k_"):
                pipe[parts[1]] = float(parts[2])
    except (OSError, ValueError):
        pass
    return out, pipe


def read_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


class Clocks:
    """nvidia-smi samples during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu=0):
        self.proc = None
        self.gpu = gpu

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            time.sleep(0.5)  # nvidia-smi's start-up, before the timed region begins
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out = ""
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            v = [x.strip() for x in l.split(",")]
            try:
                sm.append(float(v[0]))
                mx = float(v[1])
            except ValueError:
                continue
            for n, x in zip(names, v[3:7]):
                if x.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(p, f, prm, budget_s=15.0, max_evals=400, warmup=1):
    """Oracle (reference algorithm on the host cores, all threads): warmup
    untimed evaluations, then evaluations until max_evals or budget_s.  The
    process loads the oracle's timing build (-O3 -fopenmp, the compiler's
    default FMA contraction) unless TRIMEM_ORACLE_BUILD says otherwise."""
    from oracle import oracle as O

    nthreads = os.cpu_count() or 1
    O.set_threads(nthreads)
    mo = O.Mesh(p, f)
    eo = O.Energy(mo, O.default_params(**prm))
    eo.time_energy_gradient(mo, max(int(warmup), 1))  # untimed warm-up evaluations
    n, t = 0, 0.0
    rng = np.random.default_rng(1)
    x = mo.points()
    disp = [rng.normal(0, 1e-4, size=x.shape) for _ in range(EVALS_PER_STEP)]  # drawn before timing
    while n < max_evals and t < budget_s:
        t0 = time.perf_counter()
        if n % EVALS_PER_STEP == 0:
            eo.update_repulsion(mo)
        if (n // EVALS_PER_STEP) % 2 == 0:
            x += disp[n % EVALS_PER_STEP]
        else:
            x -= disp[n % EVALS_PER_STEP]
        eo.energy(mo)
        eo.gradient(mo)
        t += time.perf_counter() - t0
        n += 1
    return {"value": n / t, "unit": UNIT, "cores": O.get_threads(), "kind": "port", "build": O.BUILD,
            "sample": f"{n} evaluations (energy + gradient calls, one cell-list rebuild per 10, displacement "
                      f"N(0,1e-4)) of the 163,842-vertex workload, {t:.1f} s, OpenMP {O.get_threads()} threads"}


def cpu_baseline_parity_build(budget_s=8.0):
    """The same CPU sample with the oracle's parity build (no FMA
    contraction), in a child process; returns its evaluations/s."""
    env = dict(os.environ, TRIMEM_ORACLE_BUILD="parity")
    r = subprocess.run([sys.executable, os.path.abspath(__file__), "--cpu-sample", str(budget_s)], env=env,
                       capture_output=True, text=True, timeout=600)
    try:
        out = json.loads(r.stdout.strip().splitlines()[-1])
        return {"value": out["value"], "unit": UNIT, "build": out["build"], "sample": out["sample"]}
    except Exception:
        return {"error": (r.stderr or r.stdout)[-300:]}


def cpu_chain_step(state, n_steps=2, n_leapfrog=20, dt=5e-6, ratio=0.2):
    """Chain steps of the chains' workload on the host cores with the oracle
    (the reference algorithm restated, all threads): per step a neighbour-list
    rebuild, an HMC move of n_leapfrog velocity-Verlet steps (m 1, T 1: 21
    gradients and 2 energies, the reference's integrator) and a parallel flip
    sweep (the reference's pflip restated, OpenMP with try-locks)."""
    from oracle import oracle as O

    O.set_threads(os.cpu_count() or 1)
    mo = O.Mesh(state["x"], state["faces"])
    eo = O.Energy(mo, O.default_params(**state["prm"]))
    if state.get("initial") is not None:  # the chain's reference properties
        eo.set_initial_props(state["initial"])
    x = mo.points()  # a view of the oracle mesh's positions
    rng = np.random.default_rng(3)
    t_hmc = t_flip = 0.0
    acc = flips = 0
    for _ in range(n_steps):
        t0 = time.perf_counter()
        eo.update_repulsion(mo)
        x0 = x.copy()
        pm = rng.standard_normal(x.shape)
        h0 = eo.energy(mo) + 0.5 * float((pm * pm).sum())
        a = -eo.gradient(mo)
        for _ in range(n_leapfrog):
            x += pm * dt + (0.5 * dt * dt) * a
            a1 = -eo.gradient(mo)
            pm += (0.5 * dt) * (a + a1)
            a = a1
        h1 = eo.energy(mo) + 0.5 * float((pm * pm).sum())
        if rng.random() <= np.exp(min(0.0, h0 - h1)):
            acc += 1
        else:
            x[:] = x0
        t1 = time.perf_counter()
        flips += O.flip_parallel(mo, eo, ratio, int(rng.integers(1 << 31)))
        t_flip += time.perf_counter() - t1
        t_hmc += t1 - t0
    sec = t_hmc + t_flip
    return {"steps": n_steps, "seconds": round(sec, 3), "steps_per_s": round(n_steps / sec, 4),
            "ms_per_move": {"hmc": round(t_hmc * 1e3 / n_steps, 1), "flip": round(t_flip * 1e3 / n_steps, 1)},
            "acceptance": acc / n_steps, "flips_accepted_per_sweep": flips / n_steps,
            "cores": O.get_threads(), "kind": "port",
            "sample": f"{n_steps} chain steps (HMC move of {n_leapfrog} velocity-Verlet steps at dt {dt:g} + pflip "
                      f"sweep ratio {ratio}) from the chains' warmed 163,842-vertex state"}


def level6_leg(stream, flush, n_evals=100, cpu=True):
    """The 40,962-vertex evaluation loop (level-6 icosphere, kb 30, volume
    target 0.8, the other parameters as the headline workload): FP64
    energy+gradient evaluations with an N(0, 1e-4) displacement before each
    and a cell-list rebuild every 10, each evaluation timed with CUDA events
    after an L2 flush; beside it the CPU restatement on the host cores."""
    import ctypes

    import torch

    from trimem_gb300 import capi, meshgen
    from trimem_gb300.workloads import workload_params

    p6, f6 = meshgen.jittered_icosphere(6, seed=0)
    prm6 = workload_params(p6, f6)
    mesh = capi.Mesh(p6, f6)
    en = capi.Energy(mesh, capi.params(**prm6))
    L = capi.lib()
    x = torch.tensor(p6, dtype=torch.float64, device="cuda").contiguous()
    g = torch.empty_like(x)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(66)
    disp = [1e-4 * torch.randn(tuple(x.shape), dtype=torch.float64, device="cuda", generator=gen)
            for _ in range(EVALS_PER_STEP)]
    ptr = lambda t: ctypes.c_void_p(t.data_ptr())
    sp = ctypes.c_void_p(stream)
    ms = []
    for i in range(n_evals + 10):
        if i % EVALS_PER_STEP == 0:
            capi.check(L.tm_energy_update_repulsion_device(en.h, mesh.h, ptr(x), sp))
        x.add_(disp[i % EVALS_PER_STEP], alpha=1.0 if (i // EVALS_PER_STEP) % 2 == 0 else -1.0)
        flush.fill_(1.0)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        capi.check(L.tm_energy_eval_device(en.h, mesh.h, ptr(x), ptr(g), None, sp))
        b.record()
        if i >= 10:  # the first ten are warm-up
            ms.append((a, b))
    torch.cuda.synchronize()
    eval_ms = sum(a.elapsed_time(b) for a, b in ms) / len(ms)
    out = {"workload": "icosphere L6 (40962 vertices), FP64 energy+gradient, displacement N(0,1e-4) per eval, "
                       "cell-list rebuild every 10 evals, L2 flushed before each",
           "vertices": len(p6), "evals": n_evals, "eval_ms": round(eval_ms, 5),
           "gpu_evals_per_s": round(1e3 / eval_ms, 1)}
    if cpu:
        cb = cpu_baseline(p6, f6, prm6, budget_s=8.0, max_evals=200)
        out.update(cpu_evals_per_s=round(cb["value"], 3), cpu_cores=cb["cores"],
                   gpu_over_cpu=round(1e3 / eval_ms / cb["value"], 1))
    return out


def batch_members(n_per_level=16, levels=(3, 4, 5, 6)):
    """The 64 membranes of the batch configuration: (points, faces, params)."""
    from trimem_gb300 import meshgen
    from trimem_gb300.workloads import workload_params

    rng = np.random.default_rng(2024)
    reps = []
    for lv in levels:
        for k in range(n_per_level):
            p, f = meshgen.jittered_icosphere(lv, seed=100 * lv + k)
            reps.append((p, f, workload_params(p, f, kappa_b=float(rng.uniform(10, 50)),
                                               vfrac=float(rng.uniform(0.6, 0.95)))))
    return reps


def batch_replicas():
    from trimem_gb300 import capi

    reps = batch_members()
    return capi.Batch([(p, f) for p, f, _ in reps], [capi.params(**prm) for _, _, prm in reps])


def batch_leg(stream, n_per_level=16, levels=(3, 4, 5, 6), n_leapfrog=10, n_steps=500, n_seq=20, dt=1e-6):
    """Replica batch of the 64-membrane configuration: 16 replicas each of
    642, 2,562, 10,242 and 40,962 vertices, reduced volume ~ U[0.6, 0.95] and
    kappa_b ~ U[10, 50] (seeded), FP32 stencils with FP64 sums.  n_steps HMC
    steps of n_leapfrog velocity-Verlet steps for all 64 replicas together
    (each step one CUDA graph replay: the size classes' element kernels side
    by side, neighbour lists rebuilt after every step), against the same 64
    replicas as 64 single-mesh device HMC chains run one after another
    (n_seq steps each, same moves, rebuild after every step).  The measure
    is aggregate vertex updates per second: n_leapfrog x vertices per HMC
    step.  The time step is 1e-6: the jittered members reject the
    configuration's 1e-4 (as the CPU-sized membrane does)."""
    import torch

    from trimem_gb300 import capi
    from trimem_gb300.mc.device import DeviceChain

    reps = batch_members(n_per_level, levels)
    n_rep = len(reps)
    nvert = sum(len(p) for p, _, _ in reps)
    b = capi.Batch([(p, f) for p, f, _ in reps], [capi.params(**prm) for _, _, prm in reps])
    tuning = b.tuning()
    b.hmc(3, n_leapfrog, dt, seed=1)  # warm-up and graph capture
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    acc = b.hmc(n_steps, n_leapfrog, dt, seed=1)
    torch.cuda.synchronize()
    t_batch = time.perf_counter() - t0
    # the same replicas one at a time: single-mesh device chains (FP32
    # stencils like the batch), each timed over n_seq steps after a warm-up
    t_seq, acc_seq = 0.0, 0
    for p, f, prm in reps:
        m = capi.Mesh(p, f)
        e = capi.Energy(m, capi.params(**prm))
        e.set_stencil_precision(1)
        x = torch.tensor(p, dtype=torch.float64, device="cuda").contiguous()
        ch = DeviceChain(m, e, x, dt=dt, n_leapfrog=n_leapfrog, flip_ratio=0.0, refresh=1, seed=3, stream=stream)
        ch.run(2)
        torch.cuda.synchronize()
        a0 = ch.accepted
        s0 = time.perf_counter()
        ch.run(n_seq)
        torch.cuda.synchronize()
        t_seq += time.perf_counter() - s0
        acc_seq += ch.accepted - a0
    upd_batch = n_steps * n_leapfrog * nvert / t_batch
    upd_seq = n_seq * n_leapfrog * nvert / t_seq
    return {"replicas": n_rep, "vertices": nvert, "sizes": "642/2562/10242/40962 vertices, 16 replicas each",
            "size_classes": [{"vertices": [c[0], c[1]], "block_split_face_edge_grad": list(c[2:])} for c in tuning],
            "hmc": f"{n_steps} steps x {n_leapfrog} leapfrog, dt {dt:g}, graph replay, rebuild every step",
            "hmc_steps_per_s": round(n_steps / t_batch, 2),
            "vertex_updates_per_s": round(upd_batch, 1),
            "acceptance": round(float(acc.sum()) / (n_steps * n_rep), 3),
            "sequential": {"steps_per_replica": n_seq, "vertex_updates_per_s": round(upd_seq, 1),
                           "seconds": round(t_seq, 3), "acceptance": round(acc_seq / (n_seq * n_rep), 3)},
            "speedup": round(upd_batch / upd_seq, 2),
            "timing": "wall clock around synchronised HMC runs: the batch's n_steps against the sum over the 64 "
                      "single-mesh chains of n_seq steps each (rates compared)"}


def chain_state(stream):
    """The chains' workload and start: the 163,842-vertex membrane with the
    very-large-mesh energy (reduced-volume target 0.65 of the input sphere's
    volume at its area) at equilibrium: the state saved by
    ``python -m trimem_gb300.mc.equilibrate`` (the sphere brought to the
    volume target by rounds of device L-BFGS and flip sweeps, heated by
    long-trajectory HMC moves, then 30,000 steps of the chains' own moves)
    when it is present, else equilibrated_state alone (its chains then still
    relax slowly: the drift test shows it)."""
    from trimem_gb300.mc.device import equilibrated_state
    from trimem_gb300.mc.equilibrate import load_state

    p, f, prm = workload()
    st = load_state(prm, len(p))
    if st is not None:
        return st
    return equilibrated_state(p, f, prm, stream=stream)


DT_CANDIDATES = (5e-5, 2e-5, 1e-5, 5e-6, 2e-6, 1e-6, 5e-7, 2e-7)


def _chain_handles(state, stencil):
    """Mesh (the state's flipped topology with its edge numbering), energy
    (the relaxed state's area / volume targets) and positions of a chain
    state."""
    import torch

    from trimem_gb300 import capi

    mesh = capi.Mesh(state["x"], state["faces"])
    if state.get("topo") is not None:
        mesh.set_topology(state["topo"])
    en = capi.Energy(mesh, capi.params(**state["prm"]))
    if state.get("initial") is not None:
        en.set_initial_props(state["initial"])
    en.set_stencil_precision(stencil)
    x = torch.tensor(state["x"], dtype=torch.float64, device="cuda").contiguous()
    return mesh, en, x


def drift_check(trace):
    """Stationarity of a trace: the difference of its first and last quarter
    means over their combined standard error (each quarter's standard error
    of the mean from its own effective sample size).  |z| < 3 passes."""
    from trimem_gb300.mc.ess import ess

    q = np.array_split(np.asarray(trace, float), 4)
    se = [float(b.std(ddof=1) / np.sqrt(max(ess(b), 1.0))) for b in (q[0], q[3])]
    z = float((q[3].mean() - q[0].mean()) / max(np.hypot(*se), 1e-300))
    return {"z": round(z, 2), "stationary": bool(abs(z) < 3.0)}


def chain_leg(stream, state, stencil, dt=None, n_burn=20, n_steps=2000, weights=None):
    """ESS/s of the bending energy of a device chain: per step one HMC move
    (20 velocity-Verlet steps, m 1, T 1) and one flip sweep (ratio 0.2,
    98,304 attempts), neighbour list rebuilt every step.  dt: the largest of
    DT_CANDIDATES (from 5e-5, the large-mesh runs' step) whose acceptance
    over 12 pilot moves is >= 0.5, unless given.  The trace's quarter means show whether
    it is still drifting (an ESS of a drifting trace is a lower bound)."""
    import torch

    from trimem_gb300 import capi
    from trimem_gb300.mc.device import DeviceChain, tune_dt
    from trimem_gb300.mc.ess import ess

    prm = state["prm"]
    mesh, en, x = _chain_handles(state, stencil)
    sg = capi.Surrogate(mesh, weights) if weights is not None else None
    pilot = None
    if dt is None:
        dt, pilot = tune_dt(mesh, en, x, candidates=DT_CANDIDATES, pilot=12, stream=stream, force=sg)
    ch = DeviceChain(mesh, en, x, dt=dt, n_leapfrog=20, flip_ratio=0.2, seed=11, stream=stream, force=sg)
    ch.run(n_burn)
    torch.cuda.synchronize()
    a0, f0 = ch.accepted, ch.flips
    sec0 = dict(ch.seconds)
    t0 = time.perf_counter()
    trace = ch.run(n_steps)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    bend = prm["kappa_b"] * trace[:, 3]
    e = ess(bend)
    rv = 6.0 * np.sqrt(np.pi) * trace[:, 1] / trace[:, 0] ** 1.5  # reduced volume
    e_rv = ess(rv)
    return {"dt": dt, "pilot_acceptance": pilot, "steps": n_steps, "burn_in": n_burn,
            "seconds": round(t1 - t0, 3), "ms_per_step": round((t1 - t0) * 1e3 / n_steps, 3),
            "acceptance": round((ch.accepted - a0) / n_steps, 3),
            "flips_accepted_per_sweep": round((ch.flips - f0) / n_steps, 1),
            "ms_per_move": {k: round((ch.seconds[k] - sec0[k]) * 1e3 / n_steps, 3) for k in sec0},
            "flip_attempts_per_s": round(int(0.2 * mesh.counts()[1]) * n_steps / max(ch.seconds["flip"] - sec0["flip"], 1e-9), 1),
            "flips_accepted_per_s": round((ch.flips - f0) / max(ch.seconds["flip"] - sec0["flip"], 1e-9), 1),
            "ess_bending": round(e, 2), "ess_per_s": round(e / (t1 - t0), 3),
            "bending_mean": float(bend.mean()), "bending_sd": float(bend.std()),
            "bending_quarter_means": [round(float(b.mean()), 1) for b in np.array_split(bend, 4)],
            "drift": drift_check(bend),
            "ess_reduced_volume": round(e_rv, 2), "ess_reduced_volume_per_s": round(e_rv / (t1 - t0), 3),
            "reduced_volume_mean": float(rv.mean())}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    p, f, prm = workload()
    # a bounded sample: two evaluations per step, at most two minutes
    cb = cpu_baseline(p, f, prm, budget_s=min(max(20.0, 5.0 * args.steps), 120.0),
                      max_evals=max(3, args.steps * 2), warmup=args.warmup)
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config(),
            "cpu_baseline": cb, "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                                        "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_profile(args):
    """Workload construction, one cell-list rebuild, then --profile-evals
    device evaluations at --stencil precision; prints nothing measured."""
    import ctypes

    import torch

    from trimem_gb300 import capi

    if args.profile_batch:
        b = batch_replicas()
        b.hmc(args.profile_batch, 10, 1e-6, seed=1, use_graph=False)
        print("profile batch HMC steps done:", args.profile_batch)
        return
    p, f, prm = workload()
    mesh = capi.Mesh(p, f)
    en = capi.Energy(mesh, capi.params(**prm))
    L = capi.lib()
    x = torch.tensor(p, dtype=torch.float64, device="cuda").contiguous()
    g = torch.empty_like(x)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(7)
    capi.check(L.tm_energy_set_stencil_precision(en.h, args.stencil))
    capi.check(L.tm_energy_update_repulsion_device(en.h, mesh.h, ctypes.c_void_p(x.data_ptr()), None))
    if args.profile_surrogate:
        from trimem_gb300 import surrogate as S

        sg = capi.Surrogate(mesh, np.load(S.WEIGHTS_L7))
        for _ in range(args.profile_surrogate):
            capi.check(L.tm_surrogate_gradient_device(sg.h, en.h, mesh.h, ctypes.c_void_p(x.data_ptr()),
                                                      ctypes.c_void_p(g.data_ptr()), None))
        torch.cuda.synchronize()
        print("profile surrogate evaluations done:", args.profile_surrogate)
        return
    if args.profile_flips:
        # sweeps of ratio 0.2 (98,304 proposals, windows of 4,096) on the
        # chains' equilibrated membrane, each after one HMC move; the sweeps
        # run inside the NVTX range "flip_sweeps" (ncu --nvtx-include
        # "flip_sweeps/" captures only them) and are timed with CUDA events
        # on their stream
        from trimem_gb300.mc.device import DeviceChain

        side = torch.cuda.Stream()
        sp = ctypes.c_void_p(side.cuda_stream)
        state = chain_state(side.cuda_stream)
        mesh, en, x = _chain_handles(state, 2)
        capi.check(L.tm_energy_update_repulsion_device(en.h, mesh.h, ctypes.c_void_p(x.data_ptr()), sp))
        ch = DeviceChain(mesh, en, x, dt=state["info"]["warm_dt"], n_leapfrog=20, flip_ratio=0.0, seed=3,
                         stream=side.cuda_stream)
        ms, accs = [], []
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("flip_sweeps")
        for k in range(args.profile_flips):
            ch.step()
            acc = ctypes.c_int32()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(side)
            capi.check(L.tm_flip_device(mesh.h, en.h, ctypes.c_void_p(x.data_ptr()), 0.2, 7 + k, 1, 4096,
                                        ctypes.byref(acc), sp))
            b.record(side)
            torch.cuda.synchronize()
            ms.append(a.elapsed_time(b))
            accs.append(acc.value)
        torch.cuda.nvtx.range_pop()
        print("profile flip sweeps done:", args.profile_flips, "ms per sweep:", [round(v, 3) for v in ms],
              "accepted:", accs)
        return
    for _ in range(args.profile_evals):
        x.add_(torch.randn(x.shape, dtype=torch.float64, device="cuda", generator=gen), alpha=1e-4)
        capi.check(L.tm_energy_eval_device(en.h, mesh.h, ctypes.c_void_p(x.data_ptr()),
                                           ctypes.c_void_p(g.data_ptr()), None, None))
    torch.cuda.synchronize()
    print("profile evaluations done:", args.profile_evals)


def main():
    # the CPU legs time the oracle's -O3 -fopenmp build (the reference's own
    # compiler settings); the parity build is timed beside it in a child
    # process.  Set before this process first loads the oracle.
    os.environ.setdefault("TRIMEM_ORACLE_BUILD", "timing")
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--e2e-evals", type=int, default=200)
    ap.add_argument("--profile-evals", type=int, default=0,
                    help="only run this many device evaluations (for ncu captures) and exit")
    ap.add_argument("--stencil", type=int, default=0, help="stencil precision of --profile-evals (0, 1, 2)")
    ap.add_argument("--profile-surrogate", type=int, default=0,
                    help="only run this many surrogate force evaluations (for ncu captures) and exit")
    ap.add_argument("--profile-flips", type=int, default=0,
                    help="only run this many flip sweeps (ratio 0.2) on the chains' equilibrated membrane "
                         "(for ncu captures) and exit")
    ap.add_argument("--profile-batch", type=int, default=0,
                    help="only run this many HMC steps of the 64-replica batch (for ncu captures) and exit")
    ap.add_argument("--cpu-sample", type=float, default=0.0,
                    help="only time the CPU sample of the headline workload for this many seconds, print it, exit")
    args = ap.parse_args()
    if args.cpu_sample:
        p, f, prm = workload()
        print(json.dumps(cpu_baseline(p, f, prm, budget_s=args.cpu_sample, max_evals=200)), flush=True)
        return
    if args.impl == "reference":
        return run_reference(args)
    if args.profile_evals or args.profile_surrogate or args.profile_flips or args.profile_batch:
        return run_profile(args)

    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    from trimem_gb300 import capi, load_core

    core = load_core()
    p, f, prm = workload()
    V = len(p)
    mesh = capi.Mesh(p, f)
    en = capi.Energy(mesh, capi.params(**prm))
    L = capi.lib()
    capi.check(L.tm_energy_set_stencil_precision(en.h, HEADLINE_STENCIL))
    # a dedicated stream: the library runs on it and the timing events are
    # recorded on it (the NULL handle would select the library's own stream)
    side = torch.cuda.Stream()
    torch.cuda.set_stream(side)
    stream = side.cuda_stream
    assert stream != 0
    x = torch.tensor(p, dtype=torch.float64, device="cuda").contiguous()
    g = torch.empty_like(x)
    e_dev = torch.empty(1, dtype=torch.float64, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    gen = torch.Generator(device="cuda")
    gen.manual_seed(1234 + rank)
    # N(0, 1e-4) displacements drawn before timing (a pool of EVALS_PER_STEP,
    # applied in turn with the sign alternating from step to step, so the
    # positions wander without drifting): the timed step applies them, the
    # random-number generation is not part of the workload
    disp = [1e-4 * torch.randn(tuple(x.shape), dtype=torch.float64, device="cuda", generator=gen)
            for _ in range(EVALS_PER_STEP)]
    disp_i = [0]

    def rebuild():
        capi.check(L.tm_energy_update_repulsion_device(en.h, mesh.h, ctypes_ptr(x), ctypes_ptr_s(stream)))

    def evaluate():
        k = disp_i[0]
        x.add_(disp[k % EVALS_PER_STEP], alpha=1.0 if (k // EVALS_PER_STEP) % 2 == 0 else -1.0)
        disp_i[0] += 1
        capi.check(L.tm_energy_eval_device(en.h, mesh.h, ctypes_ptr(x), ctypes_ptr(g), ctypes_ptr(e_dev),
                                           ctypes_ptr_s(stream)))

    def timed(fn):
        flush.fill_(1.0)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        return a, b

    def step():
        evs = [timed(rebuild)]
        for _ in range(EVALS_PER_STEP):
            evs.append(timed(evaluate))
        return evs

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        w0 = time.perf_counter()
        all_evs = [step() for _ in range(args.steps)]
        torch.cuda.synchronize()
        w1 = time.perf_counter()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    dev_ms = sum(a.elapsed_time(b) for evs in all_evs for a, b in evs)
    rebuild_ms = sum(evs[0][0].elapsed_time(evs[0][1]) for evs in all_evs) / args.steps
    eval_ms = (dev_ms / args.steps - rebuild_ms) / EVALS_PER_STEP
    dev_ms = max_over_ranks(dev_ms, world, "cuda")
    ms_per_step = dev_ms / args.steps
    value = job_rate(world, EVALS_PER_STEP * args.steps, dev_ms)

    # ---- roofline of the whole evaluation ----------------------------------
    # algorithmic bytes of one FP64 energy+gradient evaluation: 132 per
    # vertex (positions 24, ordered 1-ring CSR 28, flap indices 24, per-vertex
    # (c, a) written and read back between the passes 32, gradient 24), over
    # the measured time of one evaluation of the timed loop
    import ctypes

    kms = []
    for _ in range(5):
        flush.fill_(1.0)
        ms5 = (ctypes.c_float * 5)()
        capi.check(L.tm_energy_eval_timed(en.h, mesh.h, ctypes_ptr(x), ctypes_ptr(g), ms5, ctypes_ptr_s(stream)))
        kms.append(list(ms5))
    kms = np.median(np.array(kms), axis=0)
    names = ["k_face", "k_edge", "k_vertex", "k_grad"]
    F, E = len(f), 3 * len(f) // 2
    # the unique bytes each stage's kernels read and write per launch (their
    # inputs and outputs, including this implementation's face and edge
    # records), for comparison with the per-stage DRAM traffic
    # (double-word stencils: positions split into 32-byte hi/lo records and
    # 12-byte floats first, then read as 32 bytes per vertex)
    stage_bytes = {
        "k_face": 24 * V + 32 * V + 12 * V + 3 * 4 * F + 32 * V + 64 * F + 16 * F,
        "k_edge": 16 * E + 32 * V + 64 * F + 32 * E + 16 * E,
        "k_vertex": 4 * V + 16 * 2 * E + 16 * F + 16 * E + 8 * V + 16 * V,
        "k_grad": 4 * V + 16 * 2 * E + 32 * V + 16 * V + 64 * F + 32 * E + 24 * V + 24 * V,
    }
    peaks = read_peaks()
    hbm = peaks.get("hbm_gbs")
    peak_note = "of measured" if hbm else "of fallback"
    hbm = hbm or 6800.0
    eval_bytes = 132 * V
    achieved = eval_bytes / (eval_ms * 1e-3) / 1e9
    traffic_all, pipe_active = read_traffic()
    traffic = sum(traffic_all.values()) if len(traffic_all) == 4 else None
    dom = int(np.argmax(kms[:4]))
    dname = names[dom]
    roofline = {"bound": "hbm", "kernel": "one energy+gradient evaluation (all its launches)",
                "achieved": round(achieved, 2), "peak": hbm, "unit": "GB/s", "frac": round(achieved / hbm, 5),
                "traffic": traffic, "peak_source": peak_note,
                "algorithmic_bytes": eval_bytes, "algorithmic_bytes_per_vertex": 132,
                "eval_ms": round(eval_ms, 5),
                "traffic_source": "sum over the evaluation's stages of ncu dram__bytes_read.sum + "
                                  "dram__bytes_write.sum (cold-cache captures), " + TRAFFIC_PROFILE,
                "stage_ms_cold": {n: round(float(k), 5) for n, k in zip(names, kms[:4])},
                "eval_ms_cold": round(float(kms[4]), 5),
                "stage_unique_bytes": stage_bytes,
                # what bounds the stencils instead of HBM: the issue slots of
                # the dominant stage's kernel (latency and occupancy limited)
                "issue_bound": {"pipe": PIPE_NAME, "kernel": dname,
                                "pipe_active_frac": (round(pipe_active[dname] / 100.0, 3)
                                                     if dname in pipe_active else None),
                                "source": "ncu " + PIPE_METRIC + ", " + TRAFFIC_PROFILE}}

    # ---- the stencil precisions: speed and error against FP64 -------------
    g64 = g.clone()
    capi.check(L.tm_energy_set_stencil_precision(en.h, 0))
    capi.check(L.tm_energy_eval_device(en.h, mesh.h, ctypes_ptr(x), ctypes_ptr(g64), ctypes_ptr(e_dev),
                                       ctypes_ptr_s(stream)))
    torch.cuda.synchronize()
    e64 = float(e_dev.item())
    def stencil_cold(mode, n=5):
        capi.check(L.tm_energy_set_stencil_precision(en.h, mode))
        ks = []
        for _ in range(n):
            flush.fill_(1.0)
            ms5 = (ctypes.c_float * 5)()
            capi.check(L.tm_energy_eval_timed(en.h, mesh.h, ctypes_ptr(x), ctypes_ptr(g), ms5, ctypes_ptr_s(stream)))
            ks.append(list(ms5))
        capi.check(L.tm_energy_eval_device(en.h, mesh.h, ctypes_ptr(x), ctypes_ptr(g), ctypes_ptr(e_dev),
                                           ctypes_ptr_s(stream)))
        torch.cuda.synchronize()
        ev = float(e_dev.item())
        capi.check(L.tm_energy_set_stencil_precision(en.h, HEADLINE_STENCIL))
        ks = np.median(np.array(ks), axis=0)
        return {"eval_ms_cold": round(float(ks[4]), 5), "evals_per_s_cold": round(1e3 / float(ks[4]), 1),
                "kernel_ms": {n_: round(float(k), 5) for n_, k in zip(names, ks[:4])},
                "energy_rel_err": abs(ev - e64) / abs(e64),
                "grad_rel_err": float(torch.linalg.norm(g - g64) / torch.linalg.norm(g64))}

    df64 = stencil_cold(2)
    capi.check(L.tm_energy_set_stencil_precision(en.h, 1))
    k32 = []
    for _ in range(5):
        flush.fill_(1.0)
        ms5 = (ctypes.c_float * 5)()
        capi.check(L.tm_energy_eval_timed(en.h, mesh.h, ctypes_ptr(x), ctypes_ptr(g), ms5, ctypes_ptr_s(stream)))
        k32.append(list(ms5))
    capi.check(L.tm_energy_eval_device(en.h, mesh.h, ctypes_ptr(x), ctypes_ptr(g), ctypes_ptr(e_dev),
                                       ctypes_ptr_s(stream)))
    torch.cuda.synchronize()
    e32 = float(e_dev.item())
    capi.check(L.tm_energy_set_stencil_precision(en.h, HEADLINE_STENCIL))
    k32 = np.median(np.array(k32), axis=0)
    fp32 = {"eval_ms_cold": round(float(k32[4]), 5), "evals_per_s_cold": round(1e3 / float(k32[4]), 1),
            "kernel_ms": {n: round(float(k), 5) for n, k in zip(names, k32[:4])},
            "energy_rel_err": abs(e32 - e64) / abs(e64),
            "grad_rel_err": float(torch.linalg.norm(g - g64) / torch.linalg.norm(g64))}

    # ---- surrogate force: speed against the exact one, tensor-core share ---
    surrogate = None
    try:
        from trimem_gb300 import surrogate as S

        if os.path.exists(S.WEIGHTS_L7):
            sg = capi.Surrogate(mesh, np.load(S.WEIGHTS_L7))
            gs = torch.empty_like(x)

            def surrogate_force():
                capi.check(L.tm_surrogate_gradient_device(sg.h, en.h, mesh.h, ctypes_ptr(x), ctypes_ptr(gs),
                                                          ctypes_ptr_s(stream)))

            for _ in range(3):
                surrogate_force()
            sms = []
            for _ in range(10):
                a, b = timed(surrogate_force)
                torch.cuda.synchronize()
                sms.append(a.elapsed_time(b))
            s_ms = float(np.median(sms))
            # three message-passing rounds, each a (V x 128) @ (128 x 64) bf16
            # product on the tensor cores (k_dense); the rest is gathers
            dense_flop = 3 * 2 * V * 128 * 64
            bf16 = peaks.get("bf16_tflops")
            surrogate = {"force_ms_cold": round(s_ms, 5), "forces_per_s_cold": round(1e3 / s_ms, 1),
                         "vs_exact_fp64": round(float(kms[4]) / s_ms, 3),
                         "vs_exact_df64": round(df64["eval_ms_cold"] / s_ms, 3),
                         "dense_gflop": round(dense_flop / 1e9, 3),
                         "dense_tflops_over_whole_force": round(dense_flop / (s_ms * 1e-3) / 1e12, 2),
                         "bf16_peak_tflops": bf16, "peak_source": "of measured" if bf16 else None,
                         "frac": round(dense_flop / (s_ms * 1e-3) / 1e12 / bf16, 5) if bf16 else None,
                         "note": "tensor FLOP over the whole force time (a lower bound on k_dense's own rate); "
                                 "the force is bound by the gathers around the dense layers"}
    except Exception as exc:  # the headline line is printed either way
        surrogate = {"error": f"{type(exc).__name__}: {exc}"}

    # ---- end to end through the public API ---------------------------------
    # the reference's drivers write the positions into TriMesh.points() and
    # call EnergyManager.energy and EnergyManager.gradient separately
    # (src/trimem/mc/evaluators.py fun / grad); each call uploads the host
    # positions and evaluates.  The fused energy_gradient call is timed beside.
    cm = core.TriMesh(p, f)
    ep = core.EnergyParams()
    for k in ["kappa_b", "kappa_a", "kappa_v", "kappa_c", "kappa_t", "kappa_r", "area_frac", "volume_frac",
              "curvature_frac"]:
        setattr(ep, k, prm[k])
    ep.bond_params.lc0, ep.bond_params.lc1, ep.bond_params.a0 = prm["bond_lc0"], prm["bond_lc1"], prm["bond_a0"]
    ep.repulse_params.lc1, ep.repulse_params.rlist = prm["rep_lc1"], prm["rlist"]
    estore = core.EnergyManager(cm, ep)
    estore.set_stencil_precision({0: "fp64", 1: "fp32", 2: "df64"}[HEADLINE_STENCIL])
    rng = np.random.default_rng(5)
    host_x = [p + rng.normal(0, 1e-4, size=p.shape) for _ in range(4)]
    pts = cm.points()
    for i in range(3):
        np.copyto(pts, host_x[i % 4])
        estore.energy(cm)
        estore.gradient(cm)
        estore.energy_gradient(cm)
    n_e2e = args.e2e_evals

    def e2e_loop(fused):
        t0 = time.perf_counter()
        for i in range(n_e2e):
            if i % EVALS_PER_STEP == 0:
                estore.update_repulsion(cm)
            np.copyto(pts, host_x[i % 4])
            if fused:
                estore.energy_gradient(cm)
            else:
                estore.energy(cm)
                estore.gradient(cm)
        return n_e2e / (time.perf_counter() - t0)

    globals_bytes = 184  # the device's global sums and energy terms, read back by energy()
    e2e = {"value": e2e_loop(False), "unit": UNIT,
           "h2d_bytes_per_step": EVALS_PER_STEP * 2 * 24 * V + 24 * V,
           "d2h_bytes_per_step": EVALS_PER_STEP * (24 * V + globals_bytes),
           "evals": n_e2e,
           "api": "np.copyto(TriMesh.points(), x); EnergyManager.energy(mesh); EnergyManager.gradient(mesh); "
                  "update_repulsion every 10 evaluations",
           "fused": {"value": e2e_loop(True), "unit": UNIT,
                     "h2d_bytes_per_step": EVALS_PER_STEP * 24 * V + 24 * V,
                     "d2h_bytes_per_step": EVALS_PER_STEP * (24 * V + 8),
                     "api": "np.copyto(TriMesh.points(), x); EnergyManager.energy_gradient(mesh) (one call, "
                            "no counterpart in the reference)"}}

    try:
        level6 = level6_leg(stream, flush, cpu=(rank == 0 and not args.no_cpu))
    except Exception as exc:  # the headline line is printed either way
        level6 = {"error": f"{type(exc).__name__}: {exc}"}

    try:
        batch = batch_leg(stream)
    except Exception as exc:  # the headline line is printed either way
        batch = {"error": f"{type(exc).__name__}: {exc}"}

    chain = {}
    warm = None
    try:
        warm = chain_state(stream)
        chain["start"] = warm["info"]
        plain = chain_leg(stream, warm, 2)
        chain["plain_df64"] = plain
        # the FP64 stencil on the same moves, shorter: its trace follows the
        # double-word one (the same accept and flip decisions)
        chain["plain_fp64"] = chain_leg(stream, warm, 0, dt=plain["dt"], n_steps=500)
        from trimem_gb300 import surrogate as S

        if os.path.exists(S.WEIGHTS_L7):
            # the surrogate chain tunes its own step on the same rule
            chain["surrogate"] = chain_leg(stream, warm, 2, weights=np.load(S.WEIGHTS_L7))
        else:
            chain["surrogate"] = {"error": "no trained weights"}
    except Exception as exc:
        chain["error"] = f"{type(exc).__name__}: {exc}"

    cb = None
    if rank == 0 and not args.no_cpu:
        cb = cpu_baseline(p, f, prm)
        cb["parity_build"] = cpu_baseline_parity_build()
        if warm is not None:
            try:
                cc = cpu_chain_step(warm, dt=warm["info"]["warm_dt"])
                pl = chain.get("plain_df64", {})
                if "ess_bending" in pl:
                    # same moves and the same algorithm: the GPU chain's ESS
                    # per step at the CPU's step rate
                    cc["ess_per_s_at_gpu_ess_per_step"] = round(pl["ess_bending"] / pl["steps"] * cc["steps_per_s"], 5)
                cb["chain_step"] = cc
            except Exception as exc:
                cb["chain_step"] = {"error": f"{type(exc).__name__}: {exc}"}

    # this library's kernels per step: 8 per double-word evaluation (k_split_dw,
    # k_face_dw, k_edge_dw, k_moved, k_rep_fast, k_rep_slow, k_vertex_dw,
    # k_grad_dw) and 14 per cell-list rebuild (box 2, table 1, insert 1,
    # counts 1, scan 3, starts 1, scatter 1, sort 1, near-row check / build /
    # done 3); the displacement and L2-flush kernels are torch's
    launches_per_step = 8 * EVALS_PER_STEP + 14
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config(),
            "timing": {"eval_ms": round(eval_ms, 5), "rebuild_ms": round(rebuild_ms, 5),
                       "wall_ms_per_step_incl_flush": round((w1 - w0) * 1e3 / args.steps, 4),
                       "stencil": HEADLINE_STENCIL},
            "roofline": roofline, "cpu_baseline": cb, "e2e": e2e, "clocks": clk.summary(), "fp32_stencil": fp32, "df64_stencil": df64,
            "surrogate_force": surrogate,
            "level6": level6,
            "batch_replicas": batch,
            "hmc_chain": chain,
            "gpu_launches": launches_per_step * args.steps}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def max_over_ranks(x, world, device):
    """The largest x over the ranks of the process group (x itself alone)."""
    if world <= 1:
        return float(x)
    import torch

    t = torch.tensor([float(x)], device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_rate(world, units_per_rank, ms):
    """Whole-job throughput: every rank processes units_per_rank (replicas,
    weak scaling) within the slowest rank's ms."""
    return world * units_per_rank / (ms / 1e3)


def ctypes_ptr(t):
    import ctypes

    return ctypes.c_void_p(t.data_ptr())


def ctypes_ptr_s(s):
    import ctypes

    return ctypes.c_void_p(s)


if __name__ == "__main__":
    main()
