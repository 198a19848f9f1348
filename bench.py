"""Benchmark of the batched WHFast + tidal-effects kernel on GB300.

Workload (``--workload ensemble8``, the default): 4096 independent systems of a
0.08 Msun star and 7 planets (semi-major axes 0.01-0.07 AU, >= 8 mutual Hill
radii apart), constant-time-lag tides + oblate flattening + Kidder GR, WHFast
Jacobi, dt = 0.08 d, FP64, seeded synthetic inputs (posidonius_gb300.ensemble).
One bench step = one WHFast step of every system.  Metric: system-steps/s.

Timed region: one launch of the persistent kernel for K steps (CUDA graph
replay), repeated at least five times and until the timed launches add up
to 100 ms; L2 is flushed before each launch and only the launches are timed,
with CUDA events on the batch's stream; the median launch is reported.  ``e2e`` times the public C ABI with
host buffers: upload of the whole ensemble from pinned memory, K steps,
download of the whole state.

``--impl reference`` times the reference's path on the host cores: the C++
restatement of the Rust FP64 code (the Rust toolchain is not available), all
threads, same workload.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "system-steps/s"
UNIT = "system-steps/s"
L2_FLUSH_BYTES = 512 << 20
MIN_REPEATS = 5         # timed launches of K steps, at least
MIN_TIMED_MS = 1000.0   # and at least this much timed work in all (the clock sampler's 200 ms period)
MAX_REPEATS = 1000


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3000)
    p.add_argument("--warmup", type=int, default=300)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="ensemble8",
                   choices=["ensemble8", "uneven", "single", "gradient", "large", "ias15"])
    p.add_argument("--large-bodies", type=int, default=1024, help="large workload: bodies in the system")
    p.add_argument("--large-coords", default="dh", choices=["dh", "jacobi"],
                   help="large workload: democratic heliocentric or Jacobi coordinates")
    p.add_argument("--grad-steps", type=int, default=10000, help="gradient workload: WHFast steps")
    p.add_argument("--checkpoint-every", type=int, default=100, help="gradient workload: checkpoint interval")
    p.add_argument("--fd-systems", type=int, default=32, help="gradient workload: systems checked against the exact derivatives of the oracle")
    p.add_argument("--no-autotune", action="store_true", help="smallest lane group per system, no tuning")
    p.add_argument("--n-systems", type=int, default=None)
    p.add_argument("--launches", type=int, default=10, help="timed launches (L2 flushed before each)")
    p.add_argument("--mode", default="fast", choices=["fast", "exact"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-derivative", action="store_true",
                   help="large workload: skip the timed derivative run (dissipation-factor tangents)")
    p.add_argument("--derivative-dirs", type=int, default=2, choices=[1, 2, 3, 4],
                   help="large workload: tangent directions of the derivative run (the two planets' "
                        "dissipation factors, then their Love numbers)")
    p.add_argument("--cpu-seconds", type=float, default=10.0)
    p.add_argument("--horizon-steps", type=int, default=100000,
                   help="default line: steps of the energy check at the workload's configured horizon")
    p.add_argument("--horizon-systems", type=int, default=64, help="default line: systems of that check")
    p.add_argument("--adjoint-steps", type=int, default=1000,
                   help="default line: steps of the adjoint / forward timing on the differentiation shape")
    p.add_argument("--no-extras", action="store_true",
                   help="default line: leave out the energy-horizon check and the adjoint / forward timing")
    return p.parse_args()


# DRAM bytes per system and kernel launch, from one ncu capture of each kernel
# (dram__bytes_read.sum + dram__bytes_write.sum over the systems; the state is
# read and written once per launch whatever its step count):
# profiles/whfast_steps_kernel_ensemble8_bench.md (4096 systems: 22.07 MB +
# 0.02 MB) and profiles/ias15_steps_kernel_ensemble8_small.md (1024 systems:
# 12.24 MB + 1.12 MB)
DRAM_BYTES_PER_SYSTEM_LAUNCH = {"ensemble8": 22.09e6 / 4096, "ias15": 13.36e6 / 1024}

EFFECTS = {
    "ensemble8": "CTL tides + oblate flattening + Kidder GR",
    "single": "CTL tides + oblate flattening + Kidder GR",
    "uneven": "each of CTL tides / oblate flattening / Kidder GR on with p = 0.7; 20% circumbinary binaries",
    "ias15": "CTL tides + oblate flattening + Kidder GR",
}


def workload_config(name, n_systems, nmax, world):
    """The line's ``config``: what defines the workload, the same dict on both
    arms (how a run was timed goes under ``timing``)."""
    return {"workload": name, "n_systems": int(n_systems), "bodies_per_system": int(nmax),
            "dt_days": 0.08 if name != "ias15" else "adaptive (IAS15, first trial 0.08)",
            "effects": EFFECTS[name],
            "coordinates": "Jacobi" if name != "ias15" else "inertial (IAS15)",
            "l2": f"flushed ({L2_FLUSH_BYTES >> 20} MiB write) before every timed GPU launch",
            "parallelism": f"replicas x{world} (independent ensembles per GPU)"}


def make_workload(name, n_systems, rank=0):
    from posidonius_gb300 import ensemble as E
    if name == "ias15":
        # the ensemble8 systems integrated by IAS15 from a 0.08 d first step
        seed = E.SEED_BASE + E.WORKLOAD_IDS["ensemble8"] + 1000 * rank
        return E.as_ias15(E.workload_ensemble8(n_systems or 4096, seed=seed), dt=0.08)
    seed = E.SEED_BASE + E.WORKLOAD_IDS[name] + 1000 * rank
    if name == "ensemble8":
        return E.workload_ensemble8(n_systems or 4096, seed=seed)
    if name == "uneven":
        return E.workload_uneven(n_systems or 16384, seed=seed)
    return E.workload_single(seed=seed)


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(world, n_sys, steps, max_ms):
    """Whole-job system-steps/s of `world` independent replicas of n_sys
    systems each, from the slowest rank's time."""
    return world * n_sys * steps / (max_ms * 1e-3)


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0):
        self.dev = device_index
        self.proc = None
        self.lines = []

    def start(self, wait_s=15.0):
        """Start sampling and wait for the first sample, so that nvidia-smi's
        start-up does not overlap the timed region."""
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
            return
        t0 = time.time()
        while not self.lines and time.time() - t0 < wait_s and self.proc.poll() is None:
            time.sleep(0.05)
        self.skip = len(self.lines)

    def discard(self):
        """Forget the samples taken so far (before the timed region)."""
        self.skip = len(self.lines)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, power, reasons = [], [], [], set()
        for line in self.lines[getattr(self, "skip", 0):]:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for name, val in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"),
                                 f[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "power_w_max": max(power),
                "samples": len(sm), "reasons": sorted(reasons)}


def fp64_peak():
    from posidonius_gb300 import _lib
    ms = ctypes.c_double()
    tf = ctypes.c_double()
    best = 0.0
    for _ in range(3):
        _lib.check(_lib.lib().posi_fp64_probe(152 * 8, 256, 20000, ctypes.byref(ms), ctypes.byref(tf)))
        best = max(best, tf.value)
    return best


def newtonian_energy(state, s):
    """Barycentric Newtonian energy of system s (kinetic + pairwise potential)."""
    from posidonius_gb300 import ensemble as E, layout as L
    n = int(state["sys_i64"][s, L.SI_N])
    bf = state["body_f64"][s, :n]
    m = bf[:, L.BF_MASS]
    r = bf[:, L.POS]
    v = bf[:, L.VEL]
    ek = 0.5 * np.sum(m * np.sum(v * v, axis=1))
    ep = 0.0
    for i in range(n):
        for j in range(i + 1, n):
            ep -= E.G * m[i] * m[j] / np.linalg.norm(r[i] - r[j])
    return ek + ep


def pinned_like(state):
    import torch
    out = {}
    for k in ("sys_i64", "sys_f64", "body_i64", "body_f64", "body_ias"):
        if k not in state:
            continue
        t = torch.empty(state[k].shape, dtype=torch.int64 if k.endswith("i64") else torch.float64, pin_memory=True)
        a = t.numpy()
        a[...] = state[k]
        out[k] = a
        out["_t_" + k] = t
    return out


def cpu_leg(ens, steps_hint, seconds, nthreads):
    """Time the oracle on a bounded sample of the workload (all threads)."""
    import oracle
    from posidonius_gb300 import layout as L
    ns_total = ens["n_sys"]
    n_sys = min(ns_total, max(64, nthreads * 16))
    # a strided sample, so that uneven workloads are represented
    idx = np.linspace(0, ns_total - 1, n_sys).astype(np.int64)
    sub = {k: (v[idx] if isinstance(v, np.ndarray) and k != "tables" else v) for k, v in ens.items()}
    sub["n_sys"] = n_sys
    state, _, _ = oracle.run(sub, op=oracle.INITIALIZE, nthreads=nthreads)
    # calibrate: 10 steps, then size the sample for ~`seconds`
    t0 = time.perf_counter()
    state, _, _ = oracle.run(state, max_steps=10, nthreads=nthreads)
    per_step = (time.perf_counter() - t0) / 10
    steps = max(10, int(seconds / max(per_step, 1e-9)))
    t0 = time.perf_counter()
    oracle.run(state, max_steps=steps, nthreads=nthreads)
    dt = time.perf_counter() - t0
    # algorithmic flops per system-step of this workload (counted restatement)
    nf = min(n_sys, 64)
    fidx = np.linspace(0, n_sys - 1, nf).astype(np.int64)
    flo_state, _, _ = oracle.run({k: (v[fidx] if isinstance(v, np.ndarray) and k != "tables" else v)
                                  for k, v in state.items()} | {"n_sys": nf}, op=oracle.ITERATE, max_steps=1)
    _, _, _, cnt = oracle.run(flo_state, max_steps=20, flops=True)
    flops = cnt[0] / (nf * 20)
    return {"value": n_sys * steps / dt, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": f"{n_sys} systems x {steps} "
                      f"{'IAS15' if int(ens['sys_i64'][0, L.SI_INTEGRATOR]) == L.INTEGRATOR_IAS15 else 'WHFast'} "
                      f"steps of the {ens.get('_name', 'ensemble')} workload, "
                      f"C++ restatement of the Rust FP64 path, {nthreads} threads, {dt:.1f} s",
            "flops_per_system_step": flops}


def plain_path(mode, steps=400):
    """Single-system drop-in path on the star + 3 planets workload: one
    posi_iterate(h, 1) call per WHFast step -- the granularity of the
    reference's Integrator::iterate loop (src/main.rs:158-176) -- wall clock."""
    import posidonius_gb300 as pg
    from posidonius_gb300 import layout as L
    one = make_workload("single", 1)
    case = {k: (v[0] if isinstance(v, np.ndarray) and k != "tables" else v) for k, v in one.items()}
    case["n"] = int(one["sys_i64"][0, L.SI_N])
    w = pg.WHFast.from_arrays(case, mode=mode)
    w.initialize_physical_values()
    w.run(20)
    t0 = time.perf_counter()
    done = 0
    for _ in range(steps):
        done += w.iterate(1)[1]
    dt = time.perf_counter() - t0
    w.close()
    return {"value": done / dt, "unit": UNIT, "workload": "single (star + 3 planets)", "steps": done,
            "note": "posi_iterate(h, 1) per WHFast step (one kernel launch + state readback each), wall clock"}


def energy_horizon(workload, n_sys, steps, mode):
    """The whole metric's accuracy half: n_sys systems of the workload
    integrated for `steps` steps (its configured horizon) by the benchmarked
    build, and the relative deviation of every system's barycentric
    Newtonian energy from the oracle's own trajectory at the same step
    (definition 1).  The oracle's sensitivity -- its own trajectory started
    1e-15 (relative) away in position -- is reported beside it: a chaotic
    system's trajectories part whatever the arithmetic.  Definition 3: the
    same systems with every effect off (pure WHFast), the relative drift of
    the Newtonian energy over the run, on the GPU."""
    import oracle
    import posidonius_gb300 as pg
    from posidonius_gb300 import layout as L
    from posidonius_gb300 import ensemble as E
    seed = E.SEED_BASE + E.WORKLOAD_IDS[workload] + 500
    ens = E.workload_ensemble8(n_sys, seed=seed) if workload != "uneven" else E.workload_uneven(n_sys, seed=seed)
    nthreads = os.cpu_count() or 1
    b = pg.Batch(ens, mode=mode)
    b.initialize_physical_values()
    t0 = time.perf_counter()
    b.iterate(steps, min(steps, 25000))
    gpu_s = time.perf_counter() - t0
    got = b.get_state()
    b.close()
    ref, _, _ = oracle.run(ens, max_steps=steps, init_physical=True, nthreads=nthreads)
    nud = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in ens.items()}
    nud["body_f64"][:, :, L.POS] *= 1.0 + 1e-15
    ref2, _, _ = oracle.run(nud, max_steps=steps, init_physical=True, nthreads=nthreads)
    e_ref = np.array([newtonian_energy(ref, s) for s in range(n_sys)])
    d1 = np.abs(np.array([newtonian_energy(got, s) for s in range(n_sys)]) - e_ref) / np.abs(e_ref)
    sens = np.abs(np.array([newtonian_energy(ref2, s) for s in range(n_sys)]) - e_ref) / np.abs(e_ref)
    off = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in ens.items()}
    for f in (L.SI_TIDES, L.SI_FLAT, L.SI_GR):
        off["sys_i64"][:, f] = 0
    for f in (L.BI_TIDES_KIND, L.BI_FLAT_KIND, L.BI_GR_KIND):
        off["body_i64"][:, :, f] = L.EFFECT_DISABLED
    b = pg.Batch(off, mode=mode)
    b.initialize_physical_values()
    e0 = np.array([newtonian_energy(b.get_state(), s) for s in range(n_sys)])
    b.iterate(steps, min(steps, 25000))
    fin = b.get_state()
    b.close()
    d3 = np.abs(np.array([newtonian_energy(fin, s) for s in range(n_sys)]) - e0) / np.abs(e0)
    # definition 2: tides alone (flattening and GR off, their energies are
    # not in the Newtonian sum), the Newtonian plus rotational energy plus
    # the tidal dissipation dE/dt integrated over the run (trapezoid over
    # historic snapshots every H steps, where the kernel refreshes dE/dt)
    H = 50
    tid = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in ens.items()}
    for f in (L.SI_FLAT, L.SI_GR):
        tid["sys_i64"][:, f] = 0
    for f in (L.BI_FLAT_KIND, L.BI_GR_KIND):
        tid["body_i64"][:, :, f] = L.EFFECT_DISABLED
    tid["sys_f64"][:, L.SF_HIST_PERIOD] = H * tid["sys_f64"][:, L.SF_DT]

    def budget(st):
        e = np.array([newtonian_energy(st, s) for s in range(n_sys)])
        bf = st["body_f64"]
        moi = np.where(bf[..., L.BF_MOI] != 0, bf[..., L.BF_MOI], np.inf)
        e += 0.5 * np.sum(np.sum(bf[..., L.ANG] ** 2, axis=-1) / moi, axis=1)
        de = np.nansum(bf[..., L.BF_DENERGY_DT], axis=1)
        return e, de

    b = pg.Batch(tid, mode=mode)
    b.initialize_physical_values()
    e_first, de_prev = budget(b.get_state())
    lost = np.zeros(n_sys)
    dt_chunk = H * tid["sys_f64"][:, L.SF_DT]
    for _ in range(steps // H):
        b.iterate(H, H)
        e_now, de_now = budget(b.get_state())
        lost += 0.5 * (de_prev + de_now) * dt_chunk
        de_prev = de_now
    b.close()
    d2 = np.abs(e_now + lost - e_first) / np.abs(e_first)
    d2_no_loss = np.abs(e_now - e_first) / np.abs(e_first)
    q = lambda x: {"median": float(np.median(x)), "max": float(x.max())}
    return {
        "workload": workload, "systems": n_sys, "steps": steps, "days": steps * 0.08,
        "def1_vs_oracle_trajectory": q(d1) | {"systems_within_1e-10": int((d1 <= 1e-10).sum())},
        "oracle_self_sensitivity_1e-15_nudge": q(sens) | {"systems_within_1e-10": int((sens <= 1e-10).sum())},
        "def2_tides_only_energy_budget_drift": q(d2) | {
            "without_the_integrated_dissipation": q(d2_no_loss),
            "integrated_dissipation_rel": q(np.abs(lost) / np.abs(e_first)),
            "note": f"tides alone; Newtonian + rotational energy + the integral of the reference's tidal dE/dt "
                    f"(trapezoid over historic snapshots every {H} steps), relative drift over the run"},
        "def3_pure_whfast_drift": q(d3),
        "gpu_s": gpu_s,
        "note": "relative deviation of the barycentric Newtonian energy: def 1 from the oracle's own trajectory at "
                "the same step; beside it the oracle against itself started 1e-15 away (systems that part from "
                "themselves part from any other arithmetic too); def 3 the pure-WHFast drift (effects off) "
                "from the start; def 2 with tides alone (flattening and GR potentials are not in the Newtonian sum)",
    }


def adjoint_over_forward(steps, every=100, n_sys=1024):
    """The metric's second half on the differentiation shape (1024 systems
    of a star and 3 planets, checkpoints every `every` steps): backward
    (adjoint) time over forward time of one loss gradient over `steps`
    steps, CUDA events of the library's own forward and backward runs."""
    from posidonius_gb300 import adjoint as A
    from posidonius_gb300 import layout as L
    ens, el, ms, moi, ss = A.gradient_workload(n_sys)
    sig = ens["body_f64"][:, :, L.BF_SIGMA].copy()
    k2 = ens["body_f64"][:, :, L.BF_K2].copy()
    A.adjoint_gradient(ens, el, sig, k2, ms, moi, ss, min(steps, 2 * every), every)  # warm-up
    _, _, _, _, (fwd_ms, bwd_ms, rec_ms, rev_ms), flags = A.adjoint_gradient(ens, el, sig, k2, ms, moi, ss, steps,
                                                                              every)
    return {"value": bwd_ms / fwd_ms, "forward_ms": fwd_ms, "backward_ms": bwd_ms, "steps": steps,
            "checkpoint_every": every, "systems": n_sys, "bodies_per_system": 4,
            "systems_flagged": int((flags != 0).sum()),
            "note": "the gradient workload's shape (bench.py --workload gradient runs it at 1e4 steps with the "
                    "gradient checks); forward = FAST integration with checkpoints, backward = chunk "
                    "re-integration + reverse sweeps"}


def run_reference(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    if args.workload not in EFFECTS:
        print(json.dumps({"impl": "reference", "unavailable": f"the reference arm times the ensemble workloads "
                          f"({', '.join(EFFECTS)}); the {args.workload} line carries its own CPU figures"}), flush=True)
        return
    import oracle
    oracle.build()
    ens = make_workload(args.workload, args.n_systems)
    nthreads = os.cpu_count() or 1
    state, _, _ = oracle.run(ens, op=oracle.INITIALIZE, nthreads=nthreads)
    # exactly W untimed steps, then K timed ones (a bounded sample: at most
    # as many steps of the whole ensemble as fit about a minute)
    warm = max(1, args.warmup)
    t0 = time.perf_counter()
    state, _, _ = oracle.run(state, max_steps=warm, nthreads=nthreads)
    per_step = (time.perf_counter() - t0) / warm
    steps = max(1, min(args.steps, int(60.0 / max(per_step, 1e-9))))
    t0 = time.perf_counter()
    state, _, _ = oracle.run(state, max_steps=steps, nthreads=nthreads)
    dt = time.perf_counter() - t0
    value = ens["n_sys"] * steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": steps,
        "warmup": warm, "ms_per_step": dt * 1e3 / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded; posidonius_gb300.ensemble)",
        "config": workload_config(args.workload, ens["n_sys"], ens["nmax"], world),
        "timing": {"region": f"{steps} steps of the whole ensemble after {warm} untimed ones, wall clock, "
                             f"{nthreads} host threads"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": f"{int(ens['n_sys'])} systems x {steps} steps (C++ restatement of the Rust FP64 "
                                   f"path; Rust toolchain unavailable)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _fd_agreement(adj, fd, fd2, tol=1e-6):
    """Agreement of adjoint gradients [systems, parameters] with central
    differences fd (and fd2, at a second step size), per system, in the
    norm of that system's gradient: e_s = max_j |adj - fd| / max_j |fd| and
    the differences' own noise n_s = max_j |fd - fd2| / max_j |fd|.  Reports
    the median and maximum e_s, the fraction of systems with e_s <= tol, and
    the fraction within the differences' noise (e_s <= 3 n_s + tol)."""
    adj, fd, fd2 = (np.asarray(x, dtype=np.float64).reshape(len(x), -1) for x in (adj, fd, fd2))
    scale = np.abs(fd).max(axis=1)
    ok = scale > 0
    if not ok.any():
        return {"systems": 0}
    e = np.abs(adj - fd).max(axis=1)[ok] / scale[ok]
    nse = np.abs(fd - fd2).max(axis=1)[ok] / scale[ok]
    out = {"systems": int(ok.sum()), "median_rel_err": float(np.median(e)), "max_rel_err": float(e.max()),
           "frac_within_%g" % tol: float(np.mean(e <= tol)),
           "median_fd_noise": float(np.median(nse)),
           "frac_within_fd_noise": float(np.mean(e <= 3 * nse + tol))}
    # per component, where the two quotients agree to 1 % (they resolve it)
    a, f, f2 = adj.ravel(), fd.ravel(), fd2.ravel()
    res = (np.abs(f - f2) <= 1e-2 * np.abs(f)) & (f != 0)
    if res.any():
        rel = np.abs(a - f)[res] / np.abs(f)[res]
        out["resolved_components"] = {"count": int(res.sum()), "of": int(a.size),
                                      "median_rel_err": float(np.median(rel)),
                                      "frac_within_%g" % tol: float(np.mean(rel <= tol)),
                                      "frac_within_1e-4": float(np.mean(rel <= 1e-4))}
    return out


def run_gradient(args):
    """Differentiation workload: forward + adjoint of the loss over K steps,
    the adjoint/forward time ratio, and gradient checks against central
    differences (GPU forward and the CPU restatement)."""
    import torch

    import posidonius_gb300 as pg
    from posidonius_gb300 import adjoint as A
    from posidonius_gb300 import layout as L

    S = args.n_systems or 1024
    K = args.grad_steps
    every = args.checkpoint_every
    ens, el, ms, moi, ss = A.gradient_workload(S)
    sig = ens["body_f64"][:, :, L.BF_SIGMA].copy()
    k2 = ens["body_f64"][:, :, L.BF_K2].copy()
    # warm-up (graph capture, module load), then the timed gradient
    A.adjoint_gradient(ens, el, sig, k2, ms, moi, ss, min(K, 2 * every), every)
    clocks = ClockSampler(0)
    clocks.start()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    loss, g_sig, g_k2, g_el, (fwd_ms, bwd_ms, rec_ms, rev_ms), flags = A.adjoint_gradient(ens, el, sig, k2, ms,
                                                                                           moi, ss, K, every)
    wall = time.perf_counter() - t0
    clock_info = clocks.stop()
    # the forward pass alone, as the batched kernel runs it (no checkpoints)
    b = pg.Batch(ens, mode=pg.FAST)
    b.initialize_physical_values()
    b.iterate(every, every)
    b.set_state(A.initial_ensemble(ens, el, sig, k2, ms, moi, ss))
    b.initialize_physical_values()
    b.iterate(K, every)
    plain_fwd_ms, _ = b.last_timing()
    b.close()
    value = S * K / ((fwd_ms + bwd_ms) * 1e-3)
    # checks on a sample of systems: the adjoint against the exact
    # derivatives of the oracle (its dual-number build), per system, in the
    # max norm of each parameter group; chaotic systems (the oracle's own
    # loss moved by more than 1e-9 by a 1e-13 nudge of the mean anomalies)
    # are also checked at 1e3 steps, inside their predictability horizon
    import oracle
    oracle.build()
    idx = np.linspace(0, S - 1, min(args.fd_systems, S)).astype(np.int64)

    def sub_of(ix):
        d = {k: (v[ix] if isinstance(v, np.ndarray) and k != "tables" else v) for k, v in ens.items()}
        d["n_sys"] = len(ix)
        return d

    def per_system(a, b):
        a, b = (np.asarray(x).reshape(len(x), -1) for x in (a, b))
        return np.abs(a - b).max(axis=1) / np.maximum(np.abs(b).max(axis=1), 1e-300)

    def oracle_runner(e, n):
        out, _, _ = oracle.run(e, max_steps=n, init_physical=True, nthreads=os.cpu_count() or 1)
        return out["body_f64"]

    def vs_dual(ix, ksteps, adj=None):
        sub = sub_of(ix)
        args_ = (sub, el[ix], sig[ix], k2[ix], ms[ix], moi[ix], ss[ix], ksteps)
        if adj is None:
            _, a_sig, a_k2, a_el, _, a_fl = A.adjoint_gradient(*args_, every)
        else:
            a_sig, a_k2, a_el, a_fl = adj
        t0 = time.perf_counter()
        _, d_sig, d_k2, d_el = A.oracle_dual_gradient(*args_)
        dual_s = time.perf_counter() - t0
        l1 = A.loss_of_parameters(*args_, runner=oracle_runner)
        el2 = el[ix].copy()
        el2[..., 5] += 1e-13
        l2 = A.loss_of_parameters(sub, el2, sig[ix], k2[ix], ms[ix], moi[ix], ss[ix], ksteps, runner=oracle_runner)
        sens = np.abs(l2 - l1) / np.abs(l1)
        err = np.maximum.reduce([per_system(a_el, d_el), per_system(a_sig * sig[ix], d_sig * sig[ix]),
                                 per_system(a_k2 * k2[ix], d_k2 * k2[ix])])
        regular = (sens <= 1e-9) & (a_fl == 0)
        return err, regular, a_fl, dual_s, sens

    err, regular, fl, dual_s, sens = vs_dual(idx, K, (g_sig[idx], g_k2[idx], g_el[idx], flags[idx]))
    checks = {f"vs_oracle_dual_{K}_steps": {
        "systems": int(len(idx)), "median_rel_err": float(np.median(err)),
        "frac_within_1e-6": float(np.mean(err <= 1e-6)),
        "predictable_systems": int(regular.sum()),
        "predictable_frac_within_1e-6": float(np.mean(err[regular] <= 1e-6)) if regular.any() else None,
        "predictable_max_rel_err": float(err[regular].max()) if regular.any() else None,
        "chaotic_systems": int((~regular).sum()), "systems_flagged": int((fl != 0).sum()),
        "dual_oracle_s": dual_s}}
    rest = idx[~regular]
    if len(rest):
        ks = min(K, 1000)
        err2, reg2, fl2, _, sens2 = vs_dual(rest, ks)
        ok2 = fl2 == 0
        checks[f"chaotic_systems_at_{ks}_steps"] = {
            "systems": int(len(rest)), "flagged": int((~ok2).sum()),
            "max_rel_err": float(err2[ok2].max()) if ok2.any() else None,
            "frac_within_1e-6": float(np.mean(err2[ok2] <= 1e-6)) if ok2.any() else None,
            "max_oracle_sensitivity": float(sens2.max())}
    checks["note"] = ("relative error per system in the max norm of each parameter group (6 elements per planet; "
                      "sigma and k2 as d loss / d ln p), every parameter at its physical value, against forward-mode "
                      "dual-number derivatives of the oracle's reference-order arithmetic (no step size, no "
                      "difference noise); predictable = the oracle's own loss moves by <= 1e-9 under a 1e-13 "
                      "nudge of the mean anomalies over the run")
    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": K, "warmup": min(K, 2 * every),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded; posidonius_gb300.adjoint.gradient_workload)",
        "config": {"workload": "gradient", "n_systems": S, "bodies_per_system": 4, "dt_days": 0.08,
                   "checkpoint_every": every, "mode": "fast",
                   "loss": "sum e^2 + ((a - a0)/a0)^2 + ((|Omega_p| - |Omega_p0|)/|Omega_p0|)^2",
                   "parameters": "sigma, k2 per body; 6 initial elements per planet",
                   "value_note": "system-steps/s of forward + adjoint together"},
        "adjoint_over_forward": bwd_ms / fwd_ms,
        "forward_ms": fwd_ms, "backward_ms": bwd_ms, "backward_record_ms": rec_ms, "backward_reverse_ms": rev_ms,
        "plain_forward_ms": plain_fwd_ms,
        "adjoint_over_plain_forward": bwd_ms / plain_fwd_ms,
        "wall_s": wall, "systems_flagged": int((flags != 0).sum()),
        "gradient_checks": checks, "clocks": clock_info,
        "gpu_launches": int(2 * ((K + every - 1) // every) * 2),
    }
    # HBM traffic of the checkpoints and step records (the integration itself
    # keeps every system on chip): one state copy per chunk in the forward
    # run; in the backward run one state copy per chunk and the step records,
    # written by the re-integration and read by the reverse sweep (2.69 MB per
    # step for 1024 systems, dram__bytes_read.sum of the reverse kernel,
    # profiles/adj_reverse_kernel_gradient_small.md, scaled by systems)
    from posidonius_gb300 import layout as L
    n_chunks = (K + every - 1) // every
    state_bytes = S * 4 * L.BF_COUNT * 8 + S * (L.SF_COUNT + L.SI_COUNT) * 8
    tape_bytes = 2.69e6 * (S / 1024) * K
    result["hbm"] = {"checkpoint_bytes": n_chunks * state_bytes,
                     "forward_gb_s": n_chunks * state_bytes / (fwd_ms * 1e-3) / 1e9,
                     "step_record_bytes_written_and_read": 2 * tape_bytes,
                     "backward_gb_s": (n_chunks * state_bytes + 2 * tape_bytes) / (bwd_ms * 1e-3) / 1e9,
                     "note": "far below the HBM roof: the forward and reverse kernels are FP64-bound"}
    print(json.dumps(result), flush=True)


def large_derivative(mb, init, K, forward_ms, flush, n_dirs=2):
    """Derivatives of the many-body run with respect to the two tidal
    planets' dissipation factors: one launch of the engine carrying both
    tangent directions over the same K steps (forward mode; two parameters),
    then the loss gradient (torch) from the final state and the tangents.
    n_dirs != 2 times other direction counts (1: the first planet's
    dissipation factor; 3, 4: the planets' Love numbers added)."""
    import torch

    from posidonius_gb300 import adjoint as A
    from posidonius_gb300 import layout as L

    planets = (1, 2)
    seeds = ([(p, L.SEED_SIGMA) for p in planets] + [(p, L.SEED_K2) for p in planets])[:n_dirs]
    host = int(init["sys_i64"][L.SI_HOST])
    idx = [host, *planets]
    b0 = init["body_f64"][idx]
    with torch.no_grad():
        t = lambda x: torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64)
        a0, _ = A.orbital_elements(t(b0[:, L.POS])[None], t(b0[:, L.VEL])[None], t(b0[:, L.BF_MASS])[None])
    a0 = a0[0].numpy()
    spin0 = np.linalg.norm(b0[1:, L.ANG], axis=-1) / b0[1:, L.BF_MOI]
    mb.set_state(init)
    mb.iterate_tangent(3, seeds)              # warm-up
    mb.set_state(init)
    flush.fill_(1.0)
    torch.cuda.synchronize()
    _, tan = mb.iterate_tangent(K, seeds)
    tan_ms = mb.last_timing()
    final = mb.get_state()
    loss, grad = A.tangent_loss_gradient(final["body_f64"], tan[:2], host, planets, a0, spin0)
    # end to end: host state and zero tangents in, K steps, state, tangents and gradient out
    t0 = time.perf_counter()
    mb.set_state(init)
    _, tan2 = mb.iterate_tangent(K, seeds)
    fin2 = mb.get_state()
    A.tangent_loss_gradient(fin2["body_f64"], tan2[:2], host, planets, a0, spin0)
    e2e_s = time.perf_counter() - t0
    sig = init["body_f64"][list(planets), L.BF_SIGMA]
    return {
        "kind": "forward mode: tangents of every body's state along each planet's dissipation factor, both "
                "directions in one launch of the engine; loss gradient = final-state gradient (torch) . tangents",
        "directions": [("dissipation factor" if q == L.SEED_SIGMA else "Love number") + f" of body {b}"
                       for b, q in seeds],
        "parameters": [f"dissipation factor of body {p}" for p in planets][:len(grad)],
        "loss": "sum over the 2 planets of e^2 + ((a - a0)/a0)^2 + ((|Omega| - |Omega0|)/|Omega0|)^2",
        "loss_value": loss, "dloss_dsigma": grad.tolist(), "dloss_dlog_sigma": (grad * sig[:len(grad)]).tolist(),
        "ms": tan_ms, "ms_per_step": tan_ms / K, "over_forward": tan_ms / forward_ms,
        "e2e_s": e2e_s, "gpu_launches": 1,
    }


def run_large(args):
    """Many-body workload: one system of N bodies (star, 2 tidal planets,
    N - 3 small massive bodies), K steps in one cooperative launch."""
    import torch

    import posidonius_gb300 as pg
    from posidonius_gb300 import ensemble as E
    from posidonius_gb300 import layout as L

    N = args.large_bodies
    K = args.steps
    jacobi = args.large_coords == "jacobi"
    case = E.workload_large(N - 3, coords=L.JACOBI if jacobi else L.DEMOCRATIC_HELIOCENTRIC)
    mb = pg.ManyBody(case)
    mb.initialize_physical_values()
    init = mb.get_state()
    W = max(3, min(args.warmup, 50))
    mb.iterate(W)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    mb.set_state(init)
    clocks = ClockSampler(0)
    clocks.start()
    flush.fill_(1.0)
    torch.cuda.synchronize()
    st = mb.iterate(K)
    ms = mb.last_timing()
    clock_info = clocks.stop()
    final = mb.get_state()
    done = int(final["sys_i64"][L.SI_ITERATION])
    value = done / (ms * 1e-3)
    # e2e: host state in, K steps, host state out
    t0 = time.perf_counter()
    mb.set_state(init)
    mb.iterate(K)
    out = mb.get_state()
    e2e_s = time.perf_counter() - t0
    bytes_io = sum(init[k].nbytes for k in ("sys_i64", "sys_f64", "body_i64", "body_f64"))
    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": done, "warmup": W,
        "ms_per_step": ms / max(done, 1), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded; posidonius_gb300.ensemble.workload_large)",
        "config": {"workload": "large", "bodies": N, "dt_days": 0.1,
                   "coordinates": "Jacobi" if jacobi else "democratic heliocentric",
                   "effects": "CTL tides (every body an orbiting tidal body of the star; the small bodies with "
                              "zero dissipation and Love number)", "mode": "fast",
                   "l2": "flushed (512 MiB write) before the timed launch",
                   "pair_interactions_per_step": N * (N - 1)},
        "pair_interactions_per_s": N * (N - 1) * value,
        "e2e": {"value": done / e2e_s, "unit": UNIT, "h2d_bytes_per_step": bytes_io / max(done, 1),
                "d2h_bytes_per_step": bytes_io / max(done, 1), "note": "posi_large_set_state, iterate, get_state"},
        "gpu_launches": 1, "status": int(final["sys_i64"][L.SI_STATUS]), "clocks": clock_info,
    }
    if not args.no_derivative and not jacobi:
        result["derivative"] = large_derivative(mb, init, K, ms, flush, args.derivative_dirs)
    if not args.no_cpu_baseline:
        import oracle
        from oracle.case_json import stack
        oracle.build()
        ens = stack([case])
        state, _, _ = oracle.run(ens, op=oracle.INITIALIZE)
        # a short calibration run, then a sample of about --cpu-seconds
        t0 = time.perf_counter()
        oracle.run(state, max_steps=3, nthreads=1)
        per_step = (time.perf_counter() - t0) / 3
        n_cpu = max(3, int(args.cpu_seconds / max(per_step, 1e-9)))
        t0 = time.perf_counter()
        oracle.run(state, max_steps=n_cpu, nthreads=1)
        cpu_s = time.perf_counter() - t0
        _, _, _, cnt = oracle.run(state, max_steps=1, flops=True)
        flops = float(cnt[0])
        result["cpu_baseline"] = {"value": n_cpu / cpu_s, "unit": UNIT, "cores": 1, "kind": "port",
                                  "sample": f"{n_cpu} WHFast steps of the {N}-body system, C++ restatement of the "
                                            f"Rust FP64 path, one thread (one system does not split), {cpu_s:.1f} s"}
        peak = fp64_peak()
        achieved = flops * done / (ms * 1e-3) / 1e12
        result["roofline"] = {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                              "frac": achieved / peak, "traffic": None, "flops_per_step": flops,
                              "peak_source": "measured in-run: posi_fp64_probe (DFMA chains)",
                              "note": "algorithmic flops of one step (oracle count, + - * / sqrt = 1) x steps / "
                                      "CUDA-event launch time"}
    print(json.dumps(result), flush=True)
    mb.close()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload == "gradient":
        run_gradient(args)
        return
    if args.workload == "large":
        run_large(args)
        return
    world, rank, local = dist_setup(args)
    import torch

    import posidonius_gb300 as pg
    from posidonius_gb300 import layout as L

    torch.cuda.set_device(local)
    ens = make_workload(args.workload, args.n_systems, rank)
    ens["_name"] = args.workload
    mode = pg.FAST if args.mode == "fast" else pg.EXACT
    batch = pg.Batch(ens, mode=mode)
    batch.initialize_physical_values()
    # lane mapping per body count: picked by the autotuner (state unchanged)
    lanes = batch.autotune(probe_steps=20) if not args.no_autotune else {
        int(n): batch.mapping_for(int(n)) for n in np.unique(ens["sys_i64"][:, L.SI_N])}
    def probes(n):
        # IAS15 batches take the smallest lane group without probing
        try:
            return {str(k): v for k, v in batch.autotune_report(n).items()}
        except pg.PosiError:
            return {}

    tuning = None if args.no_autotune else {
        str(n): {"systems": int(np.sum(ens["sys_i64"][:, L.SI_N] == n)), "chosen_lanes": int(g),
                 "probe_ms_by_lanes": probes(n)}
        for n, g in sorted(lanes.items())}
    K = args.steps
    W = max(3, args.warmup)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    clocks = ClockSampler(local)
    clocks.start()
    # warm-up: exactly W steps, in one launch
    batch.iterate(W, W)
    torch.cuda.synchronize()
    clocks.discard()

    # ---- device-timed region -------------------------------------------------
    # one launch of K steps (one CUDA graph replay), L2 flushed before it,
    # CUDA events on the batch's stream; repeated until the timed launches
    # add up to at least MIN_TIMED_MS (and at least MIN_REPEATS times), the
    # median launch reported.  Each repeat continues the integration.
    barrier(world)
    torch.cuda.synchronize()
    times = []
    launches = 0
    while len(times) < MIN_REPEATS or (sum(times) < MIN_TIMED_MS and len(times) < MAX_REPEATS):
        flush.fill_(float(len(times)))
        torch.cuda.synchronize()
        batch.iterate(K, K)
        ms, nl = batch.last_timing()
        times.append(ms)
        launches = nl
    torch.cuda.synchronize()
    barrier(world)
    clock_info = clocks.stop()
    med_ms = max_over_ranks(statistics.median(times), world)
    value = replica_value(world, batch.n_sys, K, med_ms)
    total_ms = med_ms

    # ---- end-to-end through the C ABI with host buffers -----------------------
    state = batch.get_state()
    host = pinned_like(state)
    keys = ("sys_i64", "sys_f64", "body_i64", "body_f64") + (("body_ias",) if "body_ias" in host else ())
    out = {k: host[k].copy() for k in keys}
    out_p = pinned_like(out)
    h2d = sum(host[k].nbytes for k in keys)
    d2h = h2d
    barrier(world)
    torch.cuda.synchronize()
    e2e_times = []
    while len(e2e_times) < MIN_REPEATS or (sum(e2e_times) < MIN_TIMED_MS * 1e-3 and len(e2e_times) < MAX_REPEATS):
        t0 = time.perf_counter()
        batch.set_state(host)
        batch.iterate(K, K)
        batch.get_state(out_p | {"roche": None})
        e2e_times.append(time.perf_counter() - t0)
    barrier(world)
    e2e_s = max_over_ranks(statistics.median(e2e_times), world)
    e2e_value = world * batch.n_sys * K / e2e_s

    # ---- the plain path: one system (star + 3 planets), one launch per step ----
    plain = plain_path(mode)

    # ---- accuracy and roofline --------------------------------------------------
    final = batch.get_state()
    st = final["sys_i64"][:, L.SI_STATUS]
    peak = fp64_peak()
    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": total_ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded; posidonius_gb300.ensemble)",
        "config": workload_config(args.workload, batch.n_sys, batch.nmax, world),
        "timing": {"mode": args.mode, "steps_per_launch": K, "timed_launches": len(times),
                   "region": f"one launch of {K} steps (one CUDA graph replay), repeated {len(times)} times "
                             f"(at least {MIN_REPEATS}, at least {MIN_TIMED_MS:.0f} ms of timed launches in "
                             f"all), median launch; each repeat continues the integration",
                   "launch_ms": {"median": med_ms, "min": min(times), "max": max(times)},
                   "lanes_per_system": {str(k): v for k, v in sorted(lanes.items())},
                   "mapping": "autotuned" if not args.no_autotune else "smallest group"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d / K, "d2h_bytes_per_step": d2h / K,
                "note": f"one C-ABI call chain: upload {h2d} B, {K} steps, download {d2h} B; wall clock, median of "
                        f"{len(e2e_times)} repeats"},
        "autotune": tuning,
        "gpu_launches": int(launches * len(times)),
        "gpu_launches_note": f"{int(launches)} kernel launches per timed launch of {K} steps, {len(times)} timed "
                             "launches",
        "plain_path": plain,
        "batched_over_plain": value / world / plain["value"],
        "clocks": clock_info,
        "systems_frozen": int(np.sum((st & L.SYS_FATAL_MASK) != 0)),
        "midpoint_iterations": {str(k): int(v) for k, v in zip(*np.unique(final["sys_i64"][:, L.SI_LAST_MIDPOINT_ITERS],
                                                                           return_counts=True))},
    }
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        import oracle
        oracle.build()
        cpu = cpu_leg(ens, K, args.cpu_seconds, os.cpu_count() or 1)
        flops = cpu.pop("flops_per_system_step")
        result["cpu_baseline"] = cpu
        # accuracy: relative Newtonian-energy deviation from the oracle's own
        # trajectory on a sample of the benchmarked systems, at the step the
        # bench left them
        sample = list(range(0, batch.n_sys, max(1, batch.n_sys // 8)))[:8]
        sub = {k: (v[sample] if isinstance(v, np.ndarray) and k != "tables" else v) for k, v in ens.items()}
        sub["n_sys"] = len(sample)
        it = int(final["sys_i64"][sample[0], L.SI_ITERATION])
        ref, _, _ = oracle.run(sub, max_steps=it, init_physical=True, nthreads=len(sample))
        errs = [abs(newtonian_energy(final, s) - newtonian_energy(ref, i)) / abs(newtonian_energy(ref, i))
                for i, s in enumerate(sample)]
        result["energy_rel_err_vs_oracle"] = max(errs)
        result["accuracy_note"] = (f"relative deviation of the barycentric Newtonian energy from the oracle's own "
                                   f"trajectory after the {it} steps the bench ran, max over {len(sample)} sampled "
                                   f"systems; energy_at_horizon gives the configured horizon")
        if not args.no_extras and args.workload in ("ensemble8", "uneven"):
            result["energy_at_horizon"] = energy_horizon(args.workload, args.horizon_systems, args.horizon_steps, mode)
            result["adjoint_over_forward"] = adjoint_over_forward(args.adjoint_steps)
        achieved = flops * batch.n_sys * K / (med_ms * 1e-3) / 1e12
        per_sys = DRAM_BYTES_PER_SYSTEM_LAUNCH.get(args.workload)
        # a timed launch of the balanced schedule is several kernel launches,
        # each reading and writing every system's state once
        traffic = None if per_sys is None else per_sys * batch.n_sys * launches
        result["roofline"] = {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                              "frac": achieved / peak, "traffic": traffic,
                              "traffic_note": "DRAM bytes per timed launch: the per-system bytes of one ncu capture "
                                              "of the kernel (profiles/) x systems x kernel launches per timed "
                                              "launch; FP64-bound, the state stays on chip between steps",
                              "flops_per_system_step": flops,
                              "peak_source": "measured in-run: posi_fp64_probe (DFMA chains; MEASURED_PEAKS.json "
                                             "has no FP64 entry)",
                              "note": "algorithmic flops (+ - * / sqrt = 1, counted by the oracle) per launch / "
                                      "CUDA-event launch time"}
    if rank == 0:
        print(json.dumps(result), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
