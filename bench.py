"""Benchmark: batched spin-boson TEMPO trajectories/sec on one GB300.

Workload (the batched TEMPO configuration): 512 spin-boson instances, seeded:
alpha ~ U[0.01, 0.5], omega_c ~ U[1, 10], T ~ U[0, 5], ohmic exponential
cutoff, H = Omega/2 sigma_x with Omega ~ U[0.5, 2], bath operator sigma_z/2,
dkmax ~ U{20..300}, dt = 0.05, epsrel = 1e-6, 500 steps per trajectory,
rho0 = spin up.  Inputs are synthetic (seeded draws of those distributions).

One bench step = 25 TEMPO time steps of every instance (25 kernel launches;
``--launch-steps m`` makes each launch run m steps), so ``--steps 20`` (the
default) times whole 500-step trajectories and ``value`` = whole
trajectories per second of device time.  The headline form is "mixed"
(pivoted QR + one-sided Jacobi, the contractions and the site storage in
double-float on the FP32 pipe; FP64 rank decisions); the
complex128 form is timed on the first steps of the same instances, and the
whole trajectories are compared with the FP64 oracle on a stratified
subsample (committed fixture).  ``e2e`` is the same run through the host
API, with every input uploaded and every state read back inside its timed
region.  ``launch_timeline`` gives, per bench step, its last launch's
per-instance device-clock spans (the longest instance against all
instances' work spread over the SMs).

``--impl reference`` runs the reference's own CPU implementation (the
unmodified OQuPy TempoBackend from baseline/_ref when it is importable, else
the plain-numpy port in oracle/) on a dkmax-stratified sample of the same
batch, one single-threaded process per host core, and states the
whole-trajectory throughput estimated from the measured prefixes.
Other workloads: ``--workload pt | qutrit | surrogate | heavy``.
"""

import argparse
import json
import os
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

NSTEPS_TRAJ = 500
BATCH_SEED = 20261203   # the benchmark batch (one batch, partitioned across ranks)
METRIC = "spin-boson trajectories/sec on 1 GB300, mixed vs complex128, at 1e-6 trace dist"
CHUNK = 25              # TEMPO time steps per bench step: 20 bench steps = whole trajectories


def max_over_ranks(seconds, world):
    """Wall time of the whole job = the slowest rank (NCCL on GPUs, gloo on
    the CPU)."""
    if world <= 1:
        return seconds
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def make_instances(n, seed):
    import numpy as np
    from oqupy_gb300 import bath
    rng = np.random.default_rng(seed)
    sx = np.array([[0, 1], [1, 0]], dtype=complex)
    sz = np.diag([1.0, -1.0]).astype(complex)
    out = []
    for _ in range(n):
        a = rng.uniform(0.01, 0.5)
        wc = rng.uniform(1.0, 10.0)
        T = rng.uniform(0.0, 5.0)
        om = rng.uniform(0.5, 2.0)
        dk = int(rng.integers(20, 301))
        infl, U = bath.influences(a, 1.0, wc, "exponential", T, 0.05, dk, 0.5 * sz)
        p1, p2 = bath.half_step_propagators(0.5 * om * sx, 0.05)
        out.append(dict(hs_dim=2, dkmax=dk, epsrel=1e-6, influences=infl,
                        prop1=p1, prop2=p2,
                        rho0=np.diag([1.0, 0.0]).astype(complex), unitary=U,
                        params=(a, wc, T, om)))
    return out


# ---------------------------------------------------------------------------
# CPU oracle (reference arm / cpu_baseline)
# ---------------------------------------------------------------------------

def stratified_sample(insts, per=32):
    """One instance per ``per``-instance stratum of the batch sorted by dkmax
    (the stratum's middle element): the CPU legs' sample (16 of 512)."""
    order = sorted(range(len(insts)), key=lambda i: (insts[i]["dkmax"], i))
    return [order[min(k + per // 2, len(order) - 1)] for k in range(0, len(order), per)]


def _prefix_worker(args):
    """Steps 1, 2, ... of one instance on the CPU until ``budget`` seconds of
    work are done or the trajectory is complete; per-step seconds.  ``kind``
    "reference": the unmodified OQuPy TempoBackend (tempo_backend.py:577-626)
    from baseline/_ref, its tensornetwork import served by the from-scratch
    stand-in; "port": the plain-numpy oracle restatement."""
    inst, budget, kind = args
    import numpy as np
    D = int(np.asarray(inst["rho0"]).size)
    infl = inst["influences"]
    influence = (lambda dk: infl[dk] if 0 <= dk < len(infl) else None)
    props = (lambda step: (inst["prop1"], inst["prop2"]))
    if kind == "reference":
        for p in (os.path.join(ROOT, "oracle", "tnshim"), os.path.join(ROOT, "baseline", "_ref")):
            if p not in sys.path:
                sys.path.append(p)
        import warnings
        warnings.simplefilter("ignore")
        from oqupy.backends.tempo_backend import TempoBackend
        be = TempoBackend(np.asarray(inst["rho0"]).reshape(-1), influence, inst["unitary"], props,
                          np.ones(D), np.ones(D), inst["dkmax"], inst["epsrel"], config={})
    else:
        from oracle import tempo_oracle as to
        be = to.TempoOracle(np.asarray(inst["rho0"]).reshape(-1), influence, inst["unitary"], props,
                            np.ones(D), np.ones(D), inst["dkmax"], inst["epsrel"])
    be.initialize()
    times, total = [], 0.0
    while total < budget and len(times) < NSTEPS_TRAJ:
        t0 = time.perf_counter()
        be.compute_step()
        dt = time.perf_counter() - t0
        times.append(dt)
        total += dt
    return times


def reference_importable():
    """True when the unmodified reference and its stand-in imports load."""
    code = ("import sys, warnings; warnings.simplefilter('ignore'); "
            f"sys.path += [{os.path.join(ROOT, 'oracle', 'tnshim')!r}, {os.path.join(ROOT, 'baseline', '_ref')!r}]; "
            "from oqupy.backends.tempo_backend import TempoBackend")
    try:
        return subprocess.run([sys.executable, "-c", code], capture_output=True,
                              timeout=300).returncode == 0
    except Exception:
        return False


def extrapolate_trajectory(times, dkmax, nsteps=NSTEPS_TRAJ):
    """Seconds of a whole ``nsteps``-step trajectory from the measured
    per-step seconds of its first ``len(times)`` steps.  A TEMPO step's cost
    grows with the memory window min(t, dkmax + 1) and is stationary once
    the window is full: measured stationary steps are averaged; otherwise
    the growth is a power law in the window, c(t) = c_m (w(t) / t_m)^g,
    fitted (least squares in log-log) to the second half of the measured
    steps, g clipped to [0.5, 3]."""
    import numpy as np
    tau = np.asarray(times, dtype=float)
    tm = len(tau)
    if tm >= nsteps:
        return float(tau[:nsteps].sum())
    full = dkmax + 1
    if tm >= full:
        # window full from step `full` on: the measured stationary steps
        return float(tau.sum() + (nsteps - tm) * tau[max(full - 1, tm - 10):].mean())
    lo = max(2, tm // 2)
    x = np.log(np.arange(lo + 1, tm + 1, dtype=float))
    y = np.log(np.maximum(tau[lo:], 1e-9))
    g, c = np.polyfit(x, y, 1) if tm - lo >= 3 else (1.0, np.log(tau[-1]) - np.log(tm))
    g = float(np.clip(g, 0.5, 3.0))
    cm = float(np.exp(c + g * np.log(tm)))
    t = np.arange(tm + 1, nsteps + 1, dtype=float)
    return float(tau.sum() + np.sum(cm * (np.minimum(t, full) / tm) ** g))


def cpu_whole_trajectories(insts, budget, kind, procs):
    """Whole-trajectory throughput of the batch on ``procs`` host cores,
    estimated from the stratified sample: each sampled instance runs from
    step 1 in its own single-threaded process for ``budget`` seconds of
    work; its whole-trajectory seconds are the measured prefix plus the
    extrapolated rest (``extrapolate_trajectory``); the batch's CPU seconds
    are the stratum sizes times the sampled instances' seconds."""
    import multiprocessing as mp
    import numpy as np
    idx = stratified_sample(insts)
    env_keys = ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS", "MKL_NUM_THREADS")
    old = {k: os.environ.get(k) for k in env_keys}
    for k in env_keys:
        os.environ[k] = "1"
    try:
        t0 = time.perf_counter()
        with mp.get_context("spawn").Pool(min(procs, len(idx))) as pool:
            per = pool.map(_prefix_worker, [(insts[i], budget, kind) for i in idx], chunksize=1)
        wall = time.perf_counter() - t0
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    whole = [extrapolate_trajectory(t, insts[i]["dkmax"]) for t, i in zip(per, idx)]
    measured = [len(t) for t in per]
    stratum = len(insts) / len(idx)
    cpu_s = stratum * float(np.sum(whole))
    rate = len(insts) / (cpu_s / procs)
    frac = float(np.sum([sum(t) for t in per]) / np.sum(whole))
    return {"value": rate, "unit": "trajectories/s", "cores": procs, "kind": kind,
            "sample": (f"{len(idx)} instances (one per {stratum:.0f}-instance dkmax stratum of the batch), "
                       f"each run from step 1 for {budget:.0f} s of single-threaded work (steps "
                       f"{min(measured)}..{max(measured)} of {NSTEPS_TRAJ} measured), the rest of its "
                       f"trajectory extrapolated by a power law in the memory window fitted to the "
                       f"measured steps; {100 * frac:.0f}% of the estimated whole-trajectory seconds "
                       f"measured; batch seconds = {stratum:.0f} x the sample's; {procs} cores"),
            "measured_fraction": frac, "sample_steps_measured": measured, "wall_s": wall}


def _oracle_worker(args):
    """Run one instance through the oracle: W untimed steps, K timed steps."""
    inst, warm, steps = args
    import numpy as np
    from oracle import tempo_oracle as to
    infl = inst["influences"]
    p1, p2 = inst["prop1"], inst["prop2"]
    D = int(np.asarray(inst["rho0"]).size)
    # negative dk asks for the add_correlation_time influence: none here
    o = to.TempoOracle(inst["rho0"].reshape(-1), lambda dk: infl[dk] if dk >= 0 else None,
                       inst["unitary"], lambda s: (p1, p2), np.ones(D),
                       np.ones(D), inst["dkmax"], inst["epsrel"])
    o.initialize()
    for _ in range(warm):
        o.compute_step()
    t0 = time.perf_counter()
    for _ in range(steps):
        o.compute_step()
    return time.perf_counter() - t0


def cpu_oracle_rate(insts, warm, steps, procs):
    """Trajectories/sec of the oracle on ``insts`` (timed steps only) with
    ``procs`` single-threaded worker processes."""
    import multiprocessing as mp
    env_keys = ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS", "MKL_NUM_THREADS")
    old = {k: os.environ.get(k) for k in env_keys}
    for k in env_keys:
        os.environ[k] = "1"
    try:
        ctx = mp.get_context("spawn")
        t0 = time.perf_counter()
        with ctx.Pool(procs) as pool:
            per = pool.map(_oracle_worker, [(i, warm, steps) for i in insts])
        wall = time.perf_counter() - t0
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    cpu_seconds = float(sum(per))
    # instances run concurrently on `procs` cores: whole-machine throughput
    rate = len(insts) * steps / NSTEPS_TRAJ / (cpu_seconds / procs)
    return rate, cpu_seconds, wall


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------

class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.p = None
        import tempfile
        self.path = os.path.join(tempfile.gettempdir(), f"oqupy_gb300_clocks_{os.getpid()}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.QUERY,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

def trace_distance_max(a, b):
    import numpy as np
    d = (a - b).reshape(a.shape[:-1] + (2, 2))
    h = 0.5 * (d + np.conj(np.swapaxes(d, -1, -2)))
    ev = np.linalg.eigvalsh(h)
    return 0.5 * np.abs(ev).sum(axis=-1)


def run_gpu_form(torch, insts, precision, warm, steps, flush, chi_cap=64, e2e_steps=0, qr_cut=0.0):
    """Warm-up, ``steps`` device-timed steps; then, on a fresh batch advanced
    through the same warm-up, ``e2e_steps`` steps of the same window through
    the plugin path (all propagators host->device in one call, one launch,
    the new states device->host), wall-clock timed."""
    import numpy as np
    from oqupy_gb300 import TempoBatch
    b = TempoBatch(insts, precision=precision, chi_cap=chi_cap, out_cap=warm + steps + 1, qr_cut=qr_cut)
    stream = torch.cuda.current_stream()
    for _ in range(warm):
        b.advance(1, stream.cuda_stream)
    torch.cuda.synchronize()
    b.check_status()
    f0 = sum(b.info(i)["flops_alg"] for i in range(b.n))
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    for k in range(steps):
        flush.zero_()                       # evict L2 between timed steps
        ev[k][0].record(stream)
        b.advance(1, stream.cuda_stream)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    ms = [e0.elapsed_time(e1) for e0, e1 in ev]
    b.check_status()
    infos = [b.info(i) for i in range(b.n)]
    flops = sum(x["flops_alg"] for x in infos) - f0
    states = b.states(0, warm + steps + 1)
    nsplit = max(1, sum(x["splits"] for x in infos))
    stats = {"max_bond": max(x["max_bond"] for x in infos), "splits": nsplit,
             "sweeps64_per_split": sum(x["sweeps64"] for x in infos) / nsplit,
             "sweepsff_per_split": sum(x["sweeps32"] for x in infos) / nsplit}
    b.close()
    e2e = None
    if e2e_steps:
        b = TempoBatch(insts, precision=precision, chi_cap=chi_cap, out_cap=warm + e2e_steps + 1,
                       qr_cut=qr_cut)
        for _ in range(warm):
            b.advance(1, stream.cuda_stream)
        torch.cuda.synchronize()
        p1s = [i["prop1"] for i in insts]
        p2s = [i["prop2"] for i in insts]
        us = [i.get("unitary") for i in insts]
        h2d = d2h = 0
        t0 = time.perf_counter()
        for k in range(e2e_steps):
            flush.zero_()
            b.set_all_propagators(p1s, p2s, us, stream.cuda_stream)
            h2d += 2 * sum(np.asarray(p).nbytes for p in p1s)
            b.advance(1, stream.cuda_stream)
            st = b.states(warm + k + 1, 1)
            d2h += st.nbytes
        e2e = (time.perf_counter() - t0, h2d // e2e_steps, d2h // e2e_steps)
        b.check_status()
        b.close()
    return sum(ms), ms, flops, states, stats, e2e


def run_surrogate(args):
    """Learned-surrogate workload: data from the batched TEMPO solver, GPU
    training with the tensor-core kernels, calibration, held-out screening
    with TEMPO fallback above the error budget, and 1e5-point inference.
    Prints one JSON line; ``value`` = held-out points/s after fallback."""
    import numpy as np
    import torch
    from oqupy_gb300 import surrogate as sg
    ns, dk = args.sur_steps, args.sur_dkmax
    t0 = time.perf_counter()
    P = {k: sg.sample_params(n, seed) for k, n, seed in
         (("train", args.sur_train, 101), ("val", args.sur_val, 102), ("test", args.sur_test, 103))}
    Y, tgen = {}, 0.0
    for k in ("train", "val", "test"):
        Y[k], t = sg.tempo_bloch(P[k], ns, dkmax=dk)
        tgen += t
    ngen = sum(len(v) for v in P.values())
    sur = sg.Surrogate(nsteps=ns, dkmax=dk, seed=0, bins=args.sur_bins)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    losses = sur.fit(P["train"], Y["train"], epochs=args.sur_epochs, batch=256)
    torch.cuda.synchronize()
    ttrain = time.perf_counter() - t1
    val_err = sur.calibrate(P["val"], Y["val"])
    clocks = ClockSampler()
    clocks.start()
    screens = {}
    for budget in (1e-3, 1e-2):
        out, fb, tim = sur.screen(P["test"], budget=budget)
        err = np.abs(out - Y["test"]).max(axis=(1, 2))
        screens[f"{budget:g}"] = {
            "points_per_s": tim["points_per_s"], "fallback_frac": float(fb.mean()),
            "max_err_after_fallback": float(err.max()),
            "frac_within_budget": float(np.mean(err <= budget)),
            "surrogate_s": tim["surrogate_s"], "fallback_s": tim["fallback_s"]}

    # inference throughput: 1e5 in-box points, weights and inputs resident
    npts = args.sur_points
    Xp = sur._x(sg.sample_params(npts, 104))
    for _ in range(3):
        sur.net.forward(Xp)
    stream = torch.cuda.current_stream()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    for k in range(args.steps):
        ev[k][0].record(stream)
        sur.net.forward(Xp)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    ms = float(np.mean([a.elapsed_time(b) for a, b in ev]))
    # end to end: host parameters -> device -> forward -> trajectories to host
    host = sg.sample_params(npts, 105)
    torch.cuda.synchronize()
    te = time.perf_counter()
    for _ in range(args.steps):
        res = sur.predict(host)
    e2e_s = (time.perf_counter() - te) / args.steps
    clk = clocks.stop()
    sizes = sur.net.sizes
    flops = 2.0 * npts * sum(a * b for a, b in zip(sizes[:-1], sizes[1:]))
    peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["bf16_tflops"] \
        if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else 1900.0
    achieved = flops / (ms / 1e3) / 1e12
    scr = screens["0.001"]
    line = {"metric": "surrogate screening parameter points/s after TEMPO fallback (1e-3 max Bloch error)",
            "value": scr["points_per_s"], "unit": "points/s", "n_gpus": 1, "steps": args.steps,
            "warmup": 3, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16 (FP32 accumulate, FP32 master weights)",
            "data": "synthetic (seeded TEMPO-generated trajectories)",
            "config": {"workload": f"MLP 5->{sizes[1]}x{len(sizes) - 2} GELU->{sizes[-1]}; "
                                   f"{args.sur_train} train / {args.sur_val} calibration / "
                                   f"{args.sur_test} held-out TEMPO trajectories, {ns} steps dt 0.05, "
                                   f"dkmax {dk}, epsrel 1e-6; H = Omega/2 sx + eps/2 sz; the network learns the "
                                   f"bath's correction to the closed-system precession",
                       "error_bins": f"{args.sur_bins}x{args.sur_bins} (alpha x T)",
                       "l2": "not flushed: inference inputs and weights are the workload's resident state"},
            "inference": {"points_per_s": npts / (ms / 1e3), "points": npts, "ms": ms},
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": None,
                         "kernel": "tc_gemm_kernel (tcgen05 kind::f16), forward of the MLP",
                         "peak_source": "measured cuBLAS bf16 burst"},
            "e2e": {"value": npts / e2e_s, "unit": "points/s (inference only)",
                    "h2d_bytes_per_step": npts * 5 * 4, "d2h_bytes_per_step": int(res.size * 4)},
            "screening": screens,
            "validation_max_err": {"median": float(np.median(val_err)), "p90": float(np.quantile(val_err, 0.9)),
                                   "max": float(val_err.max())},
            "err_map": [float(x) for x in sur.err_map],
            "data_generation": {"trajectories": ngen, "seconds": tgen, "traj_per_s": ngen / tgen},
            "training": {"epochs": args.sur_epochs, "seconds": ttrain, "loss_first": losses[0],
                         "loss_last": losses[-1]},
            "clocks": clk, "gpu_launches": args.steps * (len(sizes) - 1),
            "wall_s": time.perf_counter() - t0}
    print(json.dumps(line))


def _pt_worker(args):
    """CPU oracle PT-TEMPO build of one instance (seconds)."""
    inst = args
    from oracle import tempo_oracle as to
    infl = inst["influences"]
    t0 = time.perf_counter()
    to.pt_tempo_build(2, lambda dk: infl[dk] if 0 <= dk < len(infl) else None,
                      inst["num_steps"], inst["dkmax"], inst["epsrel"])
    return time.perf_counter() - t0


def run_pt(args):
    """PT-TEMPO workload: a batch of process tensors of the spin-boson model
    (omega_c 5, T 1, dt 0.02, sigma_z/2 coupling) at alpha ~ 0.1 U[0.8, 1],
    dkmax 20, 100 steps, epsrel 1e-6 (bonds up to ~25; the alpha 0.3,
    epsrel 1e-7 model reaches bond 168 already at dkmax 20, beyond one CTA
    per split), built in both precision forms; then the process-tensor sweep
    (compute_dynamics) for 8 and for 1024 Hamiltonians a sx + b sz with
    (a, b) ~ U[-2, 2]^2 on one process tensor.  One JSON line; ``value`` =
    mixed-form process-tensor builds per second."""
    import numpy as np
    import torch
    from oqupy_gb300 import bath
    from oqupy_gb300.pt import PtBatch
    n, steps, dk = args.pt_instances, args.pt_steps, args.pt_dkmax
    rng = np.random.default_rng(20261204)
    sz = np.diag([1.0, -1.0]).astype(complex)
    sx = np.array([[0, 1], [1, 0]], dtype=complex)
    insts = []
    for _ in range(n):
        a = 0.1 * rng.uniform(0.8, 1.0)
        infl, _u = bath.influences(a, 1.0, 5.0, "exponential", 1.0, 0.02, dk, 0.5 * sz)
        insts.append(dict(hs_dim=2, num_steps=steps, dkmax=dk, epsrel=1e-6,
                          influences=infl[:min(steps, dk + 1)]))
    res = {}
    clocks = ClockSampler()
    clocks.start()
    for prec in ("mixed", "complex128"):
        b = PtBatch(insts, precision=prec, chi_cap=args.pt_chi_cap)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        b.advance(steps)
        e1.record()
        torch.cuda.synchronize()
        b.check_status()
        ms = e0.elapsed_time(e1)
        infos = [b.info(i) for i in range(n)]
        res[prec] = {"ms": ms, "builds_per_s": n / (ms / 1e3),
                     "max_bond": max(int(x["max_bond"]) for x in infos),
                     "splits": int(sum(x["splits"] for x in infos))}
        if prec == "mixed":
            bm = b
        else:
            bc = b
    # sweep: 8 and 1024 Hamiltonians on process tensor 0
    sweeps = {}
    dims = bc.bond_dimensions(0)
    for nh in (8, 1024):
        ab = rng.uniform(-2, 2, size=(nh, 2))
        props = [bath.half_step_propagators(a * sx + c * sz, 0.02) for a, c in ab]
        p1 = np.array([p[0] for p in props]); p2 = np.array([p[1] for p in props])
        rho0 = np.tile(np.array([1, 0, 0, 0], dtype=complex), (nh, 1))
        bm.dynamics(0, p1, p2, rho0)                  # warm-up (graph build)
        t0 = time.perf_counter()
        reps = 3
        for _ in range(reps):
            out_m = bm.dynamics(0, p1, p2, rho0)
        dt_s = (time.perf_counter() - t0) / reps
        out_c = bc.dynamics(0, p1, p2, rho0)
        td = trace_distance_max(out_m, out_c).max()
        chi = dims.astype(float)
        pt_bytes = float(np.sum(16.0 * chi[:-1] * chi[1:] * 4))
        st_bytes = float(np.sum(16.0 * nh * (chi[:-1] + chi[1:]) * 4))
        flops = float(np.sum(8.0 * nh * chi[:-1] * chi[1:] * 4))
        sweeps[str(nh)] = {"seconds_per_sweep": dt_s, "steps": steps,
                           "us_per_step": dt_s / steps * 1e6,
                           "effective_GBps": (pt_bytes + st_bytes) / dt_s / 1e9,
                           "fp64_GFLOPs": flops / dt_s / 1e9,
                           "mixed_vs_complex128_trace_distance": float(td)}
    clk = clocks.stop()
    cpu = None
    if args.cpu_sample > 0:
        import multiprocessing as mp
        procs = os.cpu_count() or 1
        sample = insts[: min(args.cpu_sample, n)]
        os.environ["OPENBLAS_NUM_THREADS"] = "1"
        with mp.get_context("spawn").Pool(min(procs, len(sample))) as pool:
            per = pool.map(_pt_worker, sample)
        cpu = {"value": min(procs, len(sample)) / float(np.mean(per)), "unit": "process-tensor builds/s",
               "cores": min(procs, len(sample)), "kind": "port",
               "sample": f"{len(sample)} builds, numpy oracle, one process per core"}
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) \
        if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else {"hbm_gbs": 6800.0}
    s1024 = sweeps["1024"]
    from oqupy_gb300 import _native
    fp64_peak = _native.fma_peak_tflops(0)
    line = {"metric": "PT-TEMPO process-tensor builds/s (mixed form) and process-tensor sweep",
            "value": res["mixed"]["builds_per_s"], "unit": "process-tensor builds/s", "n_gpus": 1,
            "steps": steps, "warmup": 0, "ms_per_step": res["mixed"]["ms"] / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c128 (Jacobi in double-float)", "data": "synthetic",
            "config": {"workload": f"{n} process tensors, spin-boson alpha~0.1*U[0.8,1], wc 5, T 1, dt 0.02, "
                                   f"dkmax {dk}, {steps} steps, epsrel 1e-6",
                       "chi_cap": args.pt_chi_cap},
            "build": res, "mixed_speedup_vs_complex128": res["complex128"]["ms"] / res["mixed"]["ms"],
            "sweep": sweeps,
            # the sweep re-reads each PT tensor from L2 for every Hamiltonian: HBM traffic is
            # the tensor once per step, so the bound is the FP64 pipe (complex128 sweep)
            "roofline": {"bound": "fp64-pipe", "achieved": s1024["fp64_GFLOPs"] / 1e3,
                         "peak": fp64_peak, "unit": "TFLOP/s", "frac": s1024["fp64_GFLOPs"] / 1e3 / fp64_peak,
                         "traffic": None, "hbm_effective_GBps": s1024["effective_GBps"],
                         "hbm_peak_GBps": peaks["hbm_gbs"],
                         "kernel": "dyn_step_kernel (1024 Hamiltonians), wall time of the whole sweep call",
                         "peak_source": "measured DFMA throughput (otb_measure_fma_peak)"},
            "cpu_baseline": cpu, "clocks": clk, "gpu_launches": steps * 2}
    print(json.dumps(line))


def make_qutrit_instances(n, seed):
    """Batched qutrit configuration: d = 3, super-ohmic J = 2 alpha w^3 / wc^2
    exp(-w / wc) (zeta = 3), alpha ~ U[0.05, 0.2], wc = 3, T ~ U[0, 2],
    H = seeded GUE 3x3 scaled to spectral norm 1, coupling diag(1, 0, -1),
    dt 0.05, dkmax 100, epsrel 1e-7, rho0 = |0><0|, 300-step trajectories."""
    import numpy as np
    from oqupy_gb300 import bath
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        a = rng.uniform(0.05, 0.2)
        T = rng.uniform(0.0, 2.0)
        g = rng.normal(size=(3, 3)) + 1j * rng.normal(size=(3, 3))
        h = 0.5 * (g + g.conj().T)
        h /= np.linalg.norm(h, 2)
        infl, U = bath.influences(a, 3.0, 3.0, "exponential", T, 0.05, 100, np.diag([1.0, 0.0, -1.0]))
        p1, p2 = bath.half_step_propagators(h, 0.05)
        out.append(dict(hs_dim=3, dkmax=100, epsrel=1e-7, influences=infl, prop1=p1, prop2=p2,
                        rho0=np.diag([1.0, 0.0, 0.0]).astype(complex), unitary=U))
    return out


def run_qutrit(args):
    """Batched-qutrit workload: mixed form on the GPU over a window of steps
    (warm-up W, timed K) against the CPU oracle on the same window.  value =
    300-step trajectories/s at the cost of the timed steps."""
    import numpy as np
    import torch
    n = args.qutrit_instances
    insts = make_qutrit_instances(n, 20261205)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    clocks = ClockSampler()
    clocks.start()
    t_ms, ms, fl, st, stats, e2e_m = run_gpu_form(torch, insts, "mixed", args.warmup, args.steps, flush,
                                                   args.qutrit_chi_cap, args.steps)
    clk = clocks.stop()
    value = n * args.steps / 300 / (t_ms / 1e3)
    e2e_s, h2d, d2h = e2e_m
    cpu = None
    if args.cpu_sample > 0:
        procs = os.cpu_count() or 1
        sample = insts[: min(args.cpu_sample, procs)]
        rate, cpu_s, wall = cpu_oracle_rate(sample, args.warmup, args.steps, procs)
        rate = rate * NSTEPS_TRAJ / 300          # 300-step trajectories
        cpu = {"value": rate, "unit": "trajectories/s", "cores": procs, "kind": "port",
               "sample": f"{len(sample)} instances x steps {args.warmup + 1}..{args.warmup + args.steps}"
                         f" ({cpu_s:.1f} CPU-s), numpy oracle, one process per core"}
    from oqupy_gb300 import _native
    peak_fp32 = _native.fma_peak_tflops(1)
    achieved = fl / (t_ms / 1e3) / 1e12
    line = {"metric": "batched qutrit TEMPO trajectories/sec on 1 GB300 (mixed form)", "value": value,
            "unit": "trajectories/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128 (Jacobi in double-float)", "data": "synthetic",
            "config": {"workload": f"{n} qutrit instances (alpha U[0.05,0.2], wc 3, T U[0,2], zeta 3, GUE H, "
                                   "dkmax 100, dt 0.05, epsrel 1e-7, 300-step trajectories)",
                       "timed_steps": f"{args.warmup + 1}..{args.warmup + args.steps} of 300",
                       "chi_cap": args.qutrit_chi_cap,
                       "l2": "flushed (256 MiB write) before every timed step"},
            "roofline": {"bound": "fp32-pipe", "achieved": achieved, "peak": peak_fp32, "unit": "TFLOP/s",
                         "frac": achieved / peak_fp32, "traffic": None,
                         "kernel": "tempo_kernel<true>", "peak_source": "measured FFMA throughput"},
            "cpu_baseline": cpu,
            "e2e": {"value": n * args.steps / 300 / e2e_s, "unit": "trajectories/s",
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "clocks": clk, "gpu_launches": args.steps, "mixed_stats": stats}
    print(json.dumps(line))


def _accuracy_vs_oracle(states, indices):
    """Per-instance trace distance of whole trajectories against the FP64
    oracle on the committed stratified subsample (tests/golden/
    bench_oracle.npz, made by tests/golden/make_bench_oracle.py), beside
    the oracle's own spread under 1e-15 / 1e-14 input perturbations."""
    import numpy as np
    path = os.path.join(ROOT, "tests", "golden", "bench_oracle.npz")
    if not os.path.exists(path):
        return None
    g = np.load(path)
    pos = {int(i): k for k, i in enumerate(indices)}
    rows = []
    for k, i in enumerate(g["index"]):
        n = g["states"].shape[1]
        if int(i) not in pos or states[pos[int(i)]].shape[0] < n:
            continue
        err = trace_distance_max(states[pos[int(i)]][:n], g["states"][k])
        env = g["envelope"][k]
        rows.append((int(i), int(g["dkmax"][k]), float(err.max()), float(env.max()),
                     bool((err <= np.maximum(1e-6, 10 * env)).all())))
    if not rows:
        return None
    e = np.array([r[2] for r in rows])
    return {"instances": len(rows), "steps": int(g["states"].shape[1] - 1),
            "frac_le_1e-6": float(np.mean(e <= 1e-6)),
            "frac_le_max_1e-6_10x_envelope": float(np.mean([r[4] for r in rows])),
            "median": float(np.median(e)), "max": float(e.max()),
            "per_instance": [{"index": r[0], "dkmax": r[1], "max_trace_distance": r[2],
                              "oracle_envelope_max": r[3]} for r in rows]}


def run_heavy(args):
    """Critical-path instance: the late steps of the batch wait on their
    longest instance, so time that instance alone.  The 512-instance batch
    advances 60 steps in one launch; the instance with the largest
    (window + 1) x bond^3 then runs alone on one CTA (512 threads, 200 KiB):
    steps 1..N-1 in one launch, step N (``--heavy-steps``) in its own
    launch, which is the third ``tempo_kernel`` launch of the process."""
    import numpy as np
    import torch
    from oqupy_gb300.tempo import TempoBatch
    N = int(args.heavy_steps)
    insts = make_instances(args.instances, BATCH_SEED)
    s = torch.cuda.current_stream()
    b = TempoBatch(insts, precision="mixed", chi_cap=args.chi_cap, out_cap=2, block=512, smem_kb=200)
    b.advance(60, s.cuda_stream)
    torch.cuda.synchronize()
    b.check_status()
    bonds = [b.info(i)["max_bond"] for i in range(b.n)]
    b.close()
    cost = [(min(60, x["dkmax"]) + 1) * bonds[i] ** 3 for i, x in enumerate(insts)]
    idx = int(np.argmax(cost))
    h = TempoBatch([insts[idx]], precision="mixed", chi_cap=args.chi_cap, out_cap=N + 1,
                   block=512, smem_kb=200)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    ev[0].record(s)
    h.advance(N - 1, s.cuda_stream)
    ev[1].record(s)
    ev[2].record(s)
    h.advance(1, s.cuda_stream)
    ev[3].record(s)
    torch.cuda.synchronize()
    h.check_status()
    inf = h.info(0)
    h.close()
    print(json.dumps({"workload": "critical-path instance of the batched spin-boson configuration",
                      "instance": idx, "dkmax": int(insts[idx]["dkmax"]), "step": int(inf["step"]),
                      "max_bond": int(inf["max_bond"]),
                      "ms_steps_before": ev[0].elapsed_time(ev[1]),
                      "ms_last_step": ev[2].elapsed_time(ev[3]),
                      "splits": int(inf["splits"]),
                      "sweepsff_per_split": inf["sweeps32"] / max(1, inf["splits"])}))


def tempo_workload_config(n, timed_steps):
    """The batched spin-boson workload's ``config`` (identical in both arms)."""
    return {"workload": (f"batched TEMPO spin-boson, {n} instances (alpha U[0.01,0.5], "
                         "wc U[1,10], T U[0,5], Omega U[0.5,2], dkmax U{20..300}, dt 0.05, "
                         "epsrel 1e-6), whole 500-step trajectories"),
            "instances": n, "seed": BATCH_SEED,
            "bench_step": f"{CHUNK} TEMPO time steps of every instance",
            "timed_steps": f"1..{timed_steps} of {NSTEPS_TRAJ}",
            "l2": "GPU arm: flushed (256 MiB write) before every bench step; site rings >> L2"}


def run_tempo(args, rank, world):
    """The headline workload: whole 500-step trajectories of the batch.

    One bench step = ``CHUNK`` TEMPO time steps of every instance (one
    kernel launch per time step); ``--steps 20`` is the whole trajectory.
    Warm-up steps run on a separate batch of the same size and distribution
    (its own seed), so the timed batch starts at step 1.  Timed region:
    CUDA events on the launching stream around every launch (device time,
    ``value``), nested in a wall-clock region (``e2e``) that also holds the
    handle's creation from host arrays (influences, propagators, initial
    states host->device) and the read-back of every bench step's states
    device->host.  L2 is flushed before every bench step (the batch's site
    rings are also far larger than L2).  Several ranks: one batch, the
    instances partitioned by predicted cost (oqupy_gb300.multigpu), states
    gathered to rank 0 on the host.
    """
    import numpy as np
    import torch
    from oqupy_gb300 import TempoBatch, _native
    from oqupy_gb300 import multigpu as mg
    dev_stream = torch.cuda.current_stream()
    batch_kw = dict(chi_cap=args.chi_cap, qr_cut=args.qr_cut, block=args.block, smem_kb=args.smem_kb)
    t_setup = time.perf_counter()
    insts = make_instances(args.instances, BATCH_SEED)
    setup_s = time.perf_counter() - t_setup       # influences + propagators on the host
    if world > 1:
        costs = mg.probe_costs(insts, steps=20)
        parts = mg.lpt_partition(costs, world)
    else:
        parts = [list(range(len(insts)))]
    local = [insts[i] for i in parts[rank]]
    total_steps = min(args.steps * CHUNK, NSTEPS_TRAJ)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    # warm-up: W bench steps of a separate batch
    warm = TempoBatch(make_instances(len(local), BATCH_SEED + 7919), precision="mixed",
                      out_cap=2, **batch_kw)
    for _ in range(args.warmup):
        warm.advance(CHUNK, dev_stream.cuda_stream)
    torch.cuda.synchronize()
    warm.check_status()
    warm.close()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    from oqupy_gb300.autotune import BucketTuner
    tuner = BucketTuner() if args.autotune and args.launch_steps <= 1 else None
    D = 4
    states = np.zeros((len(local), total_steps + 1, D), dtype=np.complex128)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(total_steps)]
    clocks = ClockSampler()
    barrier()
    clocks.start()
    t0 = time.perf_counter()
    b = TempoBatch(local, precision="mixed", out_cap=CHUNK + 1, **batch_kw)
    h2d = sum(np.asarray(x["influences"]).nbytes + np.asarray(x["prop1"]).nbytes
              + np.asarray(x["prop2"]).nbytes + np.asarray(x["rho0"]).nbytes for x in local)
    d2h = 0
    states[:, 0] = np.array([np.asarray(x["rho0"]).reshape(-1) for x in local])
    done = 0
    ls = max(1, int(args.launch_steps))
    launches = []    # (first step, steps) of every timed launch
    timelines = []   # (step, per-instance device-clock span of that step's launch)
    for k in range(args.steps):
        n = min(CHUNK, total_steps - done)
        if n <= 0:
            break
        flush.zero_()
        if tuner is not None:
            tuner.begin_chunk(b.max_bond() if done else 1)
        cur = None
        j = 0
        while j < n:
            if tuner is not None and tuner.shape_for(j) != cur:
                cur = tuner.shape_for(j)
                b.set_launch(cur[0], cur[1])
            m = min(ls, n - j)
            ev[done + j][0].record(dev_stream)
            b.advance(m, dev_stream.cuda_stream)        # one launch, m steps of every instance
            ev[done + j][1].record(dev_stream)
            launches.append((done + j, m))
            j += m
        chunk_states = b.states(done + 1, n)             # device -> host (synchronises)
        states[:, done + 1: done + 1 + n] = chunk_states
        d2h += chunk_states.nbytes
        if tuner is not None:
            tuner.end_chunk([ev[s0][0].elapsed_time(ev[s0][1]) / m
                             for s0, m in launches if done <= s0 < done + n])
        done += n
        timelines.append((done, b.timeline()))
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    clk = clocks.stop()
    b.check_status()
    # per-step times: a launch of m steps contributes its time / m to each
    ms = np.zeros(done)
    for s0, m in launches:
        ms[s0: s0 + m] = ev[s0][0].elapsed_time(ev[s0][1]) / m
    infos = [b.info(i) for i in range(b.n)]
    b.close()
    flops = float(sum(x["flops_alg"] for x in infos))
    dev_s = max_over_ranks(float(ms.sum()) / 1e3, world)
    e2e_all = max_over_ranks(e2e_s, world)
    frac_traj = done / NSTEPS_TRAJ
    value = len(insts) * frac_traj / dev_s
    all_states = mg.gather_rows(states, parts, len(insts), rank, world)

    # complex128 on the first steps of the same instances (both forms' event
    # times over the same launches)
    c128 = None
    nc = min(args.c128_steps, done)
    if nc > 0 and not args.no_complex128:
        bc = TempoBatch(local, precision="complex128", out_cap=nc + 1, **batch_kw)
        evc = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(nc)]
        torch.cuda.synchronize()
        for j in range(nc):
            if j % CHUNK == 0:
                flush.zero_()
            evc[j][0].record(dev_stream)
            bc.advance(1, dev_stream.cuda_stream)
            evc[j][1].record(dev_stream)
        torch.cuda.synchronize()
        bc.check_status()
        msc = np.array([e0.elapsed_time(e1) for e0, e1 in evc])
        st_c = bc.states(0, nc + 1)
        ic = [bc.info(i) for i in range(bc.n)]
        bc.close()
        td = trace_distance_max(states[:, : nc + 1], st_c).max(axis=1)
        t_mixed = float(ms[:nc].sum())
        t_c = float(msc.sum())
        c128 = {"steps": f"1..{nc}", "complex128_ms_per_step": t_c / nc, "mixed_ms_per_step": t_mixed / nc,
                "mixed_speedup_vs_complex128": t_c / t_mixed,
                "mixed_vs_complex128_trace_distance": {
                    "max": float(td.max()), "median": float(np.median(td)),
                    "frac_le_1e-6": float(np.mean(td <= 1e-6))},
                "complex128_sweeps64_per_split": sum(x["sweeps64"] for x in ic) / max(1, sum(x["splits"] for x in ic))}

    # each chunk's last launch on the device clock, per instance: is a step
    # bound by its longest instance or by the sum of all instances' work?
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    timeline = {"sms": int(sms),
                "note": ("per chunk, the device-clock spans of its last launch: launch_ms close to "
                         "longest_instance_ms means the step waits on one instance's split chain; "
                         "close to instance_ms_sum_over_sms, on the whole batch's work"),
                "steps": []}
    for step_no, tl in timelines:
        dur = (tl[:, 1] - tl[:, 0]) / 1e6
        timeline["steps"].append({
            "step": step_no, "launch_ms": round(float((tl[:, 1].max() - tl[:, 0].min()) / 1e6), 3),
            "longest_instance_ms": round(float(dur.max()), 3),
            "longest_instance": int(np.argmax(dur)),
            "instance_ms_sum_over_sms": round(float(dur.sum() / sms), 3),
            "instance_ms_p50": round(float(np.median(dur)), 3)})
    nsplit = max(1, sum(x["splits"] for x in infos))
    stats = {"max_bond": max(x["max_bond"] for x in infos), "splits": nsplit,
             "sweeps64_per_split": sum(x["sweeps64"] for x in infos) / nsplit,
             "sweepsff_per_split": sum(x["sweeps32"] for x in infos) / nsplit}
    if rank != 0:
        return
    peak_fp32 = _native.fma_peak_tflops(1)
    achieved = flops / (float(ms.sum()) / 1e3) / 1e12
    roofline = {"bound": "fp32-pipe", "achieved": achieved, "peak": peak_fp32, "unit": "TFLOP/s",
                "frac": achieved / peak_fp32, "traffic": None,
                "kernel": "tempo_kernel<true> (QR + double-float Jacobi bond splits)",
                "achieved_def": ("algorithmic flops of the timed launches (complex R-SVD count "
                                 "4 (6 R N^2 + 20 N^3) per split of an R x N matrix + 8 per complex "
                                 "multiply-add of the contractions) / their summed event time"),
                "peak_source": "measured FFMA throughput of this GPU (otb_measure_fma_peak); "
                               "the bound is the FP32 pipe the double-float arithmetic runs on",
                "traffic_note": ("DRAM bytes vary with the memory window over a trajectory; the "
                                 "ncu capture of one launch (step 31, 64 instances) is in profiles/")}
    cpu = None
    if world == 1 and args.cpu_sample > 0:
        cpu = cpu_whole_trajectories(insts, args.cpu_budget, "port", os.cpu_count() or 1)
    acc = _accuracy_vs_oracle(all_states, list(range(len(insts)))) if all_states is not None else None
    line = {"metric": METRIC, "value": value, "unit": "trajectories/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(ms.sum()) / max(1, args.steps),
            "higher_is_better": True, "scaling": "strong" if world > 1 else "weak",
            "vs_baseline": None, "dtype": "c128 storage; splits and contractions in double-float (f32 pairs)",
            "data": "synthetic (seeded draws of the batched spin-boson distribution)",
            "config": tempo_workload_config(len(insts), done),
            "arm": {"precision": "mixed", "parallelism": f"instances x {world} GPUs",
                    "steps_per_launch": ls,
                    "warmup": f"{args.warmup} bench steps on a separate batch (seed {BATCH_SEED + 7919})",
                    "launch": ({"autotuned_per_bond_bucket": tuner.table()} if tuner is not None
                               else {"block": args.block or 256, "smem_kb": args.smem_kb or 56})},
            "roofline": roofline, "cpu_baseline": cpu,
            "e2e": {"value": len(insts) * frac_traj / e2e_all, "unit": "trajectories/s",
                    "h2d_bytes_per_step": int(h2d // max(1, args.steps)),
                    "d2h_bytes_per_step": int(d2h // max(1, args.steps)),
                    "note": ("same run, wall clock: handle creation from host arrays (all inputs "
                             "host->device), every launch, every bench step's states device->host")},
            "clocks": clk, "gpu_launches": len(launches), "mixed_stats": stats,
            "launch_timeline": timeline,
            "setup_seconds": setup_s,
            "ms_per_step_by_block": [float(ms[i:i + 50].sum()) / len(ms[i:i + 50]) for i in range(0, done, 50)],
            "accuracy_vs_fp64_oracle": acc}
    if c128:
        line["complex128_window"] = c128
    print(json.dumps(line))


def run_reference(args, rank, world):
    """``--impl reference``: the reference's own CPU implementation on the
    same batch and metric, all host cores, rank 0 only."""
    if rank != 0:
        return
    procs = os.cpu_count() or 1
    t_setup = time.perf_counter()
    insts = make_instances(args.instances, BATCH_SEED)
    setup_s = time.perf_counter() - t_setup
    kind = "reference" if reference_importable() else "port"
    cpu = cpu_whole_trajectories(insts, args.ref_budget, kind, procs)
    value = cpu["value"]
    line = {"metric": METRIC, "value": value, "unit": "trajectories/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * args.instances / value / NSTEPS_TRAJ * CHUNK,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
            "data": "synthetic (seeded draws of the batched spin-boson distribution)",
            "config": tempo_workload_config(args.instances, min(args.steps * CHUNK, NSTEPS_TRAJ)),
            "arm": {"precision": "complex128", "parallelism": f"one single-threaded process per core x {procs}",
                    "warmup": "none (CPU)"},
            "impl": "reference",
            "cpu_baseline": {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": value, "unit": "trajectories/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "setup_seconds": setup_s,
            "measured_fraction": cpu["measured_fraction"],
            "sample_steps_measured": cpu["sample_steps_measured"]}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20,
                    help=f"timed bench steps; one bench step = {CHUNK} TEMPO time steps of the batch "
                         f"(20 = whole {NSTEPS_TRAJ}-step trajectories)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--instances", type=int, default=512)
    ap.add_argument("--cpu-sample", type=int, default=1,
                    help="0: skip the CPU baseline of the gb300 line")
    ap.add_argument("--cpu-budget", type=float, default=20.0,
                    help="seconds of CPU work per sampled instance (cpu_baseline)")
    ap.add_argument("--ref-budget", type=float, default=60.0,
                    help="seconds of CPU work per sampled instance (--impl reference)")
    ap.add_argument("--no-complex128", action="store_true")
    ap.add_argument("--c128-steps", type=int, default=50,
                    help="first TEMPO steps timed in the complex128 form for the comparison")
    ap.add_argument("--chi-cap", type=int, default=64)
    ap.add_argument("--block", type=int, default=0, help="threads per CTA (0 = the library default)")
    ap.add_argument("--launch-steps", type=int, default=1,
                    help="TEMPO steps per launch (instances are independent: a launch of m steps "
                         "lets every CTA run its instance m steps without a grid-wide wait)")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="fixed launch shape instead of the per-bond-bucket tuner")
    ap.add_argument("--smem-kb", type=int, default=0, help="dynamic shared memory per CTA (0 = default)")
    ap.add_argument("--qr-cut", type=float, default=0.0,
                    help="relative cut of the bond split's QR (0 = the precision form's default)")
    ap.add_argument("--workload", default="tempo", choices=["tempo", "surrogate", "pt", "qutrit", "heavy"])
    ap.add_argument("--heavy-steps", type=int, default=120,
                    help="heavy workload: the step of the critical-path instance that is timed alone")
    ap.add_argument("--qutrit-instances", type=int, default=128)
    ap.add_argument("--qutrit-chi-cap", type=int, default=96)
    ap.add_argument("--pt-instances", type=int, default=304)
    ap.add_argument("--pt-steps", type=int, default=100)
    ap.add_argument("--pt-dkmax", type=int, default=20)
    ap.add_argument("--pt-chi-cap", type=int, default=64)
    ap.add_argument("--sur-train", type=int, default=20000)
    ap.add_argument("--sur-val", type=int, default=2000)
    ap.add_argument("--sur-test", type=int, default=2000)
    ap.add_argument("--sur-steps", type=int, default=500)
    ap.add_argument("--sur-dkmax", type=int, default=8)
    ap.add_argument("--sur-epochs", type=int, default=300)
    ap.add_argument("--sur-bins", type=int, default=4)
    ap.add_argument("--sur-points", type=int, default=100000)
    args = ap.parse_args()
    if args.warmup < 3:
        raise SystemExit("--warmup must be >= 3")
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.workload == "qutrit":
        if rank != 0:
            return
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the qutrit workload's CPU oracle is "
                              "reported as cpu_baseline in the gb300 line"}))
            return
        run_qutrit(args)
        return
    if args.workload == "pt":
        if rank != 0:
            return
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the PT workload's CPU oracle is "
                              "reported as cpu_baseline in the gb300 line"}))
            return
        run_pt(args)
        return
    if args.workload == "heavy":
        if rank == 0 and args.impl != "reference":
            run_heavy(args)
        return
    if args.workload == "surrogate":
        if rank != 0:
            return
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no learned "
                              "surrogate; its TEMPO solve is the fallback timed in this workload"}))
            return
        run_surrogate(args)
        return
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    run_tempo(args, rank, world)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
