"""Benchmark: batched spin-boson TEMPO trajectories/sec on one GB300.

Workload (the batched TEMPO configuration): 512 spin-boson instances, seeded:
alpha ~ U[0.01, 0.5], omega_c ~ U[1, 10], T ~ U[0, 5], ohmic exponential
cutoff, H = Omega/2 sigma_x with Omega ~ U[0.5, 2], bath operator sigma_z/2,
dkmax ~ U{20..300}, dt = 0.05, epsrel = 1e-6, 500 steps per trajectory,
rho0 = spin up.  Inputs are synthetic (seeded draws of those distributions).

One bench step = one TEMPO time step of every instance (one kernel launch).
``value`` = instances x timed steps / 500 / timed seconds, i.e. whole
trajectories per second at the cost of the timed steps; the per-step cost
grows with the memory window (min(step, dkmax+1) sites) and the bonds, so the
timed window is stated in ``config`` and ``--full-trajectories`` times all 500
steps.  The headline form is "mixed" (pivoted QR + Jacobi and the
contractions in double-float on the FP32 pipe, FP64 rank decisions and site
storage); the complex128 form runs the same steps and the trace distance
between the two is reported.

``--impl reference`` times the CPU oracle (a plain-numpy restatement of the
reference TEMPO backend) on the same workload and steps, on all host cores.
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
DRAM_BYTES_PER_INSTANCE_STEP31 = (14.974464e6 + 0.60544e6) / 64
METRIC = "spin-boson trajectories/sec on 1 GB300, mixed vs complex128, at 1e-6 trace dist"


def rank_seed(rank):
    """Every rank draws its own batch of independent instances (weak scaling:
    the ranks share no data and exchange nothing but the timing reduction)."""
    return 20261203 + rank


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


def cpu_oracle_latency(inst, warm, steps, threads):
    """Latency mode: one instance in one process whose BLAS uses ``threads``
    threads; returns the seconds of its ``steps`` timed steps."""
    import multiprocessing as mp
    env_keys = ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS", "MKL_NUM_THREADS")
    old = {k: os.environ.get(k) for k in env_keys}
    for k in env_keys:
        os.environ[k] = str(threads)
    try:
        with mp.get_context("spawn").Pool(1) as pool:
            return float(pool.map(_oracle_worker, [(inst, warm, steps)])[0])
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


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


def run_full_trajectories(args, insts, workload):
    """Mixed form over whole 500-step trajectories of the batch: 3 warm-up
    steps on a separate batch, then a fresh batch timed step by step (CUDA
    events on the launching stream, L2 flushed before every step)."""
    import numpy as np
    import torch
    from oqupy_gb300 import TempoBatch
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    cap = max(args.chi_cap, 96)           # bonds keep growing past the default window
    w = TempoBatch(insts, precision="mixed", chi_cap=cap, out_cap=4)
    for _ in range(max(3, args.warmup if args.warmup < 10 else 3)):
        w.advance(1, stream.cuda_stream)
    torch.cuda.synchronize()
    w.close()
    b = TempoBatch(insts, precision="mixed", chi_cap=cap, out_cap=NSTEPS_TRAJ + 1)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(NSTEPS_TRAJ)]
    clocks = ClockSampler()
    torch.cuda.synchronize()
    clocks.start()
    for k in range(NSTEPS_TRAJ):
        flush.zero_()
        ev[k][0].record(stream)
        b.advance(1, stream.cuda_stream)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = np.array([a.elapsed_time(c) for a, c in ev])
    b.check_status()
    infos = [b.info(i) for i in range(b.n)]
    b.close()
    total = float(ms.sum()) / 1e3
    line = {"metric": METRIC, "value": len(insts) / total, "unit": "trajectories/s", "n_gpus": 1,
            "steps": NSTEPS_TRAJ, "warmup": 3, "ms_per_step": float(ms.mean()), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128 (Jacobi in double-float)",
            "data": "synthetic",
            "config": dict(workload, timed_steps=f"1..{NSTEPS_TRAJ} (whole trajectories)", precision="mixed"),
            "ms_per_step_by_block": [float(ms[i:i + 50].mean()) for i in range(0, NSTEPS_TRAJ, 50)],
            "max_bond": max(int(x["max_bond"]) for x in infos),
            "splits": int(sum(x["splits"] for x in infos)), "clocks": clk,
            "gpu_launches": NSTEPS_TRAJ}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=30)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--instances", type=int, default=512)
    ap.add_argument("--cpu-sample", type=int, default=512)
    ap.add_argument("--no-complex128", action="store_true")
    ap.add_argument("--chi-cap", type=int, default=64)
    ap.add_argument("--qr-cut", type=float, default=0.0,
                    help="relative cut of the bond split's QR (0 = the precision form's default)")
    ap.add_argument("--full-trajectories", action="store_true",
                    help="time whole 500-step trajectories of the batch (mixed form only)")
    ap.add_argument("--workload", default="tempo", choices=["tempo", "surrogate", "pt", "qutrit"])
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
    seed = rank_seed(rank)
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
    if args.workload == "surrogate":
        if rank != 0:
            return
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no learned "
                              "surrogate; its TEMPO solve is the fallback timed in this workload"}))
            return
        run_surrogate(args)
        return

    workload = {"workload": f"batched TEMPO spin-boson, {args.instances} instances (alpha U[0.01,0.5], "
                            "wc U[1,10], T U[0,5], Omega U[0.5,2], dkmax U{20..300}, "
                            "dt 0.05, epsrel 1e-6, 500-step trajectories)",
                "instances_per_gpu": args.instances,
                "timed_steps": f"{args.warmup + 1}..{args.warmup + args.steps} of {NSTEPS_TRAJ}",
                "l2": "flushed (256 MiB write) before every timed step",
                "seed": seed}

    if args.impl == "reference":
        if rank != 0:
            return
        t_setup = time.perf_counter()
        insts = make_instances(args.instances, seed)
        setup_s = time.perf_counter() - t_setup
        procs = os.cpu_count() or 1
        rate, cpu_s, wall = cpu_oracle_rate(insts, args.warmup, args.steps, procs)
        per_step_ms = cpu_s / procs / args.steps * 1e3
        # latency mode: the instance with the longest memory alone, BLAS on all cores
        big = max(insts, key=lambda i: i["dkmax"])
        lat_s = cpu_oracle_latency(big, args.warmup, args.steps, procs)
        line = {"metric": METRIC, "value": rate, "unit": "trajectories/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_step_ms,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "c128", "data": "synthetic", "config": workload, "impl": "reference",
                "cpu_baseline": {"value": rate, "unit": "trajectories/s", "cores": procs,
                                 "kind": "port",
                                 "sample": f"{len(insts)} instances x steps {args.warmup + 1}.."
                                           f"{args.warmup + args.steps}, numpy oracle, one "
                                           f"single-threaded process per core"},
                "e2e": {"value": rate, "unit": "trajectories/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0},
                "setup_seconds": setup_s,
                "latency_mode": {"value": args.steps / NSTEPS_TRAJ / lat_s, "unit": "trajectories/s",
                                 "ms_per_step": lat_s / args.steps * 1e3, "threads": procs,
                                 "sample": f"one instance (dkmax {big['dkmax']}) x steps "
                                           f"{args.warmup + 1}..{args.warmup + args.steps}, "
                                           "BLAS threads = all cores"}}
        print(json.dumps(line))
        return

    import numpy as np
    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    from oqupy_gb300 import _native
    t_setup = time.perf_counter()
    insts = make_instances(args.instances, seed)
    setup_s = time.perf_counter() - t_setup        # influences + propagators on the host
    if args.full_trajectories:
        if rank == 0:
            run_full_trajectories(args, insts, workload)
        return
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    clocks = ClockSampler()
    barrier()
    clocks.start()
    t_mixed, ms_mixed, fl_mixed, st_mixed, stats_mixed, e2e_m = run_gpu_form(
        torch, insts, "mixed", args.warmup, args.steps, flush, args.chi_cap, args.steps, args.qr_cut)
    clk = clocks.stop()
    barrier()
    t_mixed_s = max_over_ranks(t_mixed / 1e3, world)
    value = world * args.instances * args.steps / NSTEPS_TRAJ / t_mixed_s

    res = {}
    if not args.no_complex128:
        t_c, ms_c, fl_c, st_c, stats_c, _ = run_gpu_form(torch, insts, "complex128",
                                                          args.warmup, args.steps, flush,
                                                          args.chi_cap)
        td = trace_distance_max(st_mixed, st_c).max(axis=1)
        res = {"complex128_value": world * args.instances * args.steps / NSTEPS_TRAJ / (t_c / 1e3),
               "complex128_ms_per_step": t_c / args.steps,
               "mixed_speedup_vs_complex128": t_c / t_mixed,
               "mixed_vs_complex128_trace_distance": {
                   "max": float(td.max()), "median": float(np.median(td)),
                   "frac_le_1e-6": float(np.mean(td <= 1e-6))},
               "complex128_stats": stats_c}

    e2e_s, h2d, d2h = e2e_m
    e2e = {"value": world * args.instances * args.steps / NSTEPS_TRAJ / e2e_s,
           "unit": "trajectories/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
           "note": (f"steps {args.warmup + 1}..{args.warmup + args.steps} (the timed window, on a "
                    "second batch advanced through the same warm-up) through the plugin path: "
                    "all propagators host->device in one call, one launch, the new states "
                    "device->host; wall clock")}
    peak_fp32 = _native.fma_peak_tflops(1)
    peak_fp64 = _native.fma_peak_tflops(0)
    achieved = fl_mixed / t_mixed_s / 1e12
    roofline = {"bound": "fp32-pipe", "achieved": achieved, "peak": peak_fp32,
                "unit": "TFLOP/s", "frac": achieved / peak_fp32, "traffic": None,
                "kernel": "tempo_kernel<true> (double-float Jacobi)",
                "achieved_def": "algorithmic flops (complex R-SVD count per split + contractions) / event time",
                "peak_source": "measured FFMA throughput (otb_measure_fma_peak)",
                "fp64_pipe_peak_tflops": peak_fp64}
    if res:
        ach_c = fl_c / (t_c / 1e3) / 1e12
        roofline["complex128"] = {"bound": "fp64-pipe", "achieved": ach_c, "peak": peak_fp64,
                                  "frac": ach_c / peak_fp64}
    # DRAM bytes per launch: ncu capture of the mixed kernel at step 31 for the
    # first 64 instances of this batch (dram__bytes_read.sum + write = 15.58 MB),
    # scaled by the instance count (every instance reads and writes only its
    # own site ring, influences and states)
    roofline["traffic"] = DRAM_BYTES_PER_INSTANCE_STEP31 * args.instances
    roofline["traffic_source"] = ("ncu, step 31, 64 instances, scaled by instances "
                                  "(profiles/tempo_kernel_mixed_step31.md)")

    cpu = None
    if rank == 0 and world == 1 and args.cpu_sample > 0:
        procs = os.cpu_count() or 1
        sample = insts[: args.cpu_sample]
        rate, cpu_s, wall = cpu_oracle_rate(sample, args.warmup, args.steps, procs)
        cpu = {"value": rate, "unit": "trajectories/s", "cores": procs, "kind": "port",
               "sample": f"{len(sample)} instances x steps {args.warmup + 1}..{args.warmup + args.steps}"
                         f" ({cpu_s:.1f} CPU-s), numpy oracle, one process per core"}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "trajectories/s",
                "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": t_mixed / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "c128 (Jacobi in double-float)",
                "data": "synthetic", "config": dict(workload, precision="mixed",
                                                    parallelism=f"instances x {world} GPUs"),
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
                "clocks": clk, "gpu_launches": args.steps, "mixed_stats": stats_mixed,
                "setup_seconds": setup_s,
                "whole_trajectories": ("value is trajectory-equivalents at the cost of the timed "
                                       "steps; per-step cost grows ~15x over a 500-step trajectory "
                                       "(longer memory windows, larger bonds): whole trajectories "
                                       "are timed by `python bench.py --full-trajectories`")}
        line.update(res)
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
