#!/usr/bin/env python
"""Throughput of the rigid-water MD path on GB300: ns/day of TIP4P water.

Workload (N=1): 4,096 rigid TIP4P waters at 1.0 g/cm^3 (L = 49.655 A), seeded
lattice with random quaternions, pre-equilibrated 2,000 steps (the stored state
tests/golden/tip4p4096_eq.npz), cutoff 9.0 A with a 2 A switch, Nose-Hoover
NVT at 300 K, dt = 2 fs.  One step = one full MD step (Gear predict,
placement, neighbour-list upkeep, force, collect, correct, reductions,
thermostat).  ``value`` is the mixed-precision ns/day; the plain FP64 mode and
the 32,768-molecule TIP4P/TIP5P systems are reported beside it.

Timing: per-step CUDA events on the library's stream, an L2 flush (256 MiB
write) between timed steps, W untimed warm-up steps, barrier + synchronize on
both sides, max over ranks.  ``e2e`` runs the host-buffer entry point
g6_md_step_host (state uploaded from pinned host memory and read back every
step).  ``--impl reference`` times the CPU restatement of the reference on all
host cores.  With --gpus N the ranks form a replica-exchange ensemble: rank r
runs its own TIP4P-4096 replica at 300 K * 1.01^r, and between four chunks of
the timed steps the ranks gather (E, beta, T) over a gloo group and apply the
same exchange decisions (genesis6_gb300.replicas); `value` sums the ranks'
ns/day and the exchange attempts are inside the timed total.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ns/day TIP4P 4k/32k mixed vs FP64, 1 GB300; MC ESS/GPU-s learned vs plain"
DT = 0.002          # ps
RC, SWITCH = 9.0, 2.0
TEMP = 300.0
TAU_NOSE = 0.5      # ps; q = T0 tau^2 / dt in the reference's internal form
N_MAIN = 4096
N_BIG = 32768
EQUIL_STEPS = 2000
FLOPS_PER_PAIR = {"TIP4P": 287, "TIP5P": 441, "ST2": 456}   # algorithmic flops per pair within rc


def ns_per_day(ms_per_step, dt=DT):
    return dt * 1e-3 * 86400.0 / (ms_per_step * 1e-3)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=200)
    p.add_argument("--warmup", type=int, default=10)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--no-32k", action="store_true")
    p.add_argument("--equil", type=int, default=0,
                   help="extra untimed steps after the stored equilibrated state (which already holds %d steps)"
                        % EQUIL_STEPS)
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline (profiling runs)")
    p.add_argument("--no-extra", action="store_true", help="skip the replica-exchange and Monte Carlo legs")
    p.add_argument("--n", type=int, default=N_MAIN, help="molecules of the 'md' profiling case")
    p.add_argument("--prec", choices=["mixed", "fp64"], default="mixed", help="precision of the 'md' profiling case")
    p.add_argument("--shape", default=None,
                   help="'md' profiling case: lanes,step_lanes,molecules_per_warp,skin[,half (1: half list, the "
                        "default; 0: full list)] instead of running the tuner "
                        "(keeps the tuner's many launches out of a profiler capture)")
    p.add_argument("--profile", choices=["md", "e2e", "mc", "mc-learned", "rdf"], default=None,
                   help="run a short untimed case for a profiler capture and exit: 'md' = --steps MD steps of "
                        "--n TIP4P molecules (--prec, Nose 300 K, one g6_md_run after a 20-step start); 'mc' = two runs of --steps trials on "
                        "32 chains x 1,024 ST2 (fixed widths) from a short MD start; 'mc-learned' = the same "
                        "with the network trained on 32,768 records first, then learned widths; 'rdf' = --steps "
                        "g6_rdf calls on TIP4P-32768")
    return p.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def config_block(args, world, precision="mixed (fp32 site math, fp64 sums)",
                 l2="flushed between timed steps (256 MiB write)"):
    return {"workload": "TIP4P-4096 rigid water, NVT Nose-Hoover 300 K, dt 2 fs, rc 9.0 A (2 A switch)",
            "molecules": N_MAIN, "box_A": round((N_MAIN / 0.033456) ** (1 / 3), 3), "cutoff_A": RC,
            "start": "tests/golden/tip4p4096_eq.npz (lattice + 2,000 FP64 Nose-Hoover steps at 300 K)",
            "parallelism": "replica-exchange ensemble, one replica per rank" if world > 1 else "single",
            "l2": l2, "precision": precision}


START = os.path.join(ROOT, "tests", "golden", "tip4p4096_eq.npz")
REFERENCE_UNAVAILABLE = ("Genesis6's Fortran cannot be built: no Fortran compiler on the GPU box "
                         "(gfortran, flang, ifort, ifx, nvfortran, lfortran, f95 probed: all absent)")


def equilibrated_start():
    """The stored equilibrated TIP4P-4096 state that both arms start from."""
    from genesis6_gb300 import config
    return config.load_start(START, DT)


# ---------------------------------------------------------------------------
# CPU side (reference arm and cpu_baseline): oracle restatement, all host cores.
# Nothing here loads libg6gpu.so: model tables come from the oracle.
# ---------------------------------------------------------------------------
def nose_thermo_cpu():
    q = TEMP * TAU_NOSE ** 2 / DT
    return np.array([1, q, 0.0, TEMP, 0, 0, 0, 0, 0, 0], float)


def cpu_md_run(steps, warmup, threads=None):
    """`warmup` untimed and `steps` timed MD steps of the oracle (FP64, OpenMP
    force and pair search) from the stored equilibrated state.  Returns
    (ms per step, threads, Epot of the first step)."""
    import oracle
    oracle.build()
    b = equilibrated_start()
    threads = threads or os.cpu_count() or 1
    th = nose_thermo_cpu()
    rec = b["rec"]
    rec, th, log = oracle.md_run_threaded("TIP4P", rec, b["L"], [RC] * 3, RC - SWITCH, RC, DT, max(1, warmup), th,
                                          threads)
    first_epot = float(log[0, 0])
    t0 = time.perf_counter()
    oracle.md_run_threaded("TIP4P", rec, b["L"], [RC] * 3, RC - SWITCH, RC, DT, steps, th, threads)
    wall = time.perf_counter() - t0
    return 1e3 * wall / steps, threads, first_epot


def cpu_md_rate(steps=200, warmup=3):
    ms, threads, e0 = cpu_md_run(steps, warmup)
    return {"value": ns_per_day(ms), "unit": "ns/day", "cores": threads, "kind": "port",
            "sample": "%d MD steps of TIP4P-4096 from the stored equilibrated state (oracle restatement of the "
                      "reference, FP64, OpenMP force and pair search, %d threads, g++ -O2)" % (steps, threads),
            "ms_per_step": ms, "first_step_epot": e0}


def run_reference(args, rank, world):
    """The reference's CPU path on the host cores: the FP64 restatement of
    Genesis6's MD step (the Fortran itself has no compiler here or on the GPU
    box), from the same stored state as the GPU arm, >= 200 timed steps."""
    if rank != 0:
        return
    steps = min(max(args.steps, 200), 2000)
    ms, threads, e0 = cpu_md_run(steps, max(args.warmup, 3))
    v = ns_per_day(ms)
    line = {"metric": METRIC, "value": v, "unit": "ns/day", "impl": "reference", "n_gpus": world,
            "steps": steps, "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_block(args, world, precision="fp64 (the reference's arithmetic)",
                                   l2="host cores (no GPU)"),
            "first_step_epot": e0,
            "cpu_baseline": {"value": v, "unit": "ns/day", "cores": threads, "kind": "port",
                             "sample": "%d MD steps of TIP4P-4096 on %d host threads; %s, so the CPU restatement "
                                       "of its MD step is timed" % (steps, threads, REFERENCE_UNAVAILABLE)},
            "e2e": {"value": v, "unit": "ns/day", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# GPU side
# ---------------------------------------------------------------------------
class Clocks:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc:
            time.sleep(0.3)
            self.proc.terminate()
            out, _ = self.proc.communicate(timeout=10)
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0])); mx.append(float(f[1]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[4 + k].lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def fp32_peak_tflops(torch):
    """FP32 CUDA-core throughput of cuBLAS SGEMM with TF32 off (the roofline denominator)."""
    torch.backends.cuda.matmul.allow_tf32 = False
    n = 8192
    a = torch.randn(n, n, device="cuda", dtype=torch.float32)
    b = torch.randn(n, n, device="cuda", dtype=torch.float32)
    for _ in range(2):
        torch.mm(a, b)
    torch.cuda.synchronize()
    best = 1e9
    for _ in range(5):
        e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
        e0.record(); torch.mm(a, b); e1.record(); e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


def make_system(model, n, prec, L, rec):
    import genesis6_gb300 as g6
    s = g6.RigidWater(model, n, L, path="custom", precision=prec, rc=RC, switch=SWITCH)
    s.upload_state(rec)
    return s


def thermo_for(s, n=1, temp=TEMP):
    q = temp * TAU_NOSE ** 2 / DT
    return s.thermostats(n, "nose", temp=temp, q=q, dump=0.0)


def timed_md(torch, s, steps, warmup, flush, kernel_steps=50, temp=TEMP, exchange=None, chunks=1):
    """`steps` MD steps, each a one-step CUDA graph that records events around
    the whole step, with a 256 MiB L2 flush on the same stream before every
    step.  The pair kernel is timed on `kernel_steps` further steps with events
    around the kernel as well (event nodes between the kernels add latency of
    their own, so they stay out of the step timing).  With `exchange` (a
    callable taking the chunk index and the thermostats, returning its wall
    time in ms) the timed steps run in `chunks` runs with a replica-exchange
    attempt after each; step_ms then includes those attempts."""
    from genesis6_gb300 import _capi
    L = s.L
    th = thermo_for(s, temp=temp)
    shape = _capi.Shape()
    s._check(L.g6_tune_shape(s.ctx, _capi.TUNE_SKIN, ctypes.byref(shape)))
    if warmup:
        s.md_run(DT, warmup, th, log=False)
    sp = ctypes.c_void_p()
    s._check(L.g6_stream(s.ctx, ctypes.byref(sp)))
    stream = torch.cuda.ExternalStream(sp.value)
    a, b = ctypes.c_double(), ctypes.c_double()

    def run(mode, nst):
        log = np.zeros((nst, 1, 10))
        step_ms, kms = np.zeros(nst), np.zeros(nst)
        s._check(L.g6_set_step_timing(s.ctx, mode))
        torch.cuda.synchronize()
        s._check(L.g6_md_begin(s.ctx, DT, nst, th, 1))
        for k in range(nst):
            with torch.cuda.stream(stream):
                flush.add_(1.0)
            s._check(L.g6_md_advance(s.ctx, 1))
            s._check(L.g6_step_times(s.ctx, ctypes.byref(a), ctypes.byref(b)))
            step_ms[k], kms[k] = a.value, b.value
        s._check(L.g6_md_end(s.ctx, th, log.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        s._check(L.g6_set_step_timing(s.ctx, 0))
        torch.cuda.synchronize()
        return step_ms, kms, log
    if exchange is None or chunks <= 1:
        step_ms, _, log = run(1, steps)
    else:
        parts, logs = [], []
        bounds = np.linspace(0, steps, chunks + 1).astype(int)
        for c in range(chunks):
            st, _, lg = run(1, int(bounds[c + 1] - bounds[c]))
            st[-1] += exchange(c, th)
            parts.append(st); logs.append(lg)
        step_ms, log = np.concatenate(parts), np.concatenate(logs)
    _, kms, _ = run(2, max(1, min(kernel_steps, steps)))
    return step_ms, kms, log, shape.as_dict()


def e2e_md(torch, s, rec, steps):
    """g6_md_step_host with pinned host state: H2D + step + D2H every step, wall clock."""
    n = rec.shape[0]
    host = torch.empty((n, 53), dtype=torch.float64, pin_memory=True)
    host.copy_(torch.from_numpy(rec))
    hv = host.numpy()
    th = thermo_for(s)
    lg = np.zeros(10)
    s.md_step_host(DT, hv, th, lg)     # warm
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        s.md_step_host(DT, hv, th, lg)
    wall = time.perf_counter() - t0
    rec_b = n * 53 * 8
    # records in, and the run's control block (thermostat, factors, control words
    # and counters: 256 bytes for one replica) that the records-in kernel reads
    h2d = rec_b + 256
    # records out, and the thermostat (112 bytes), the 5 step sums, the control
    # words, the overflow flag and the log row the records-out kernel writes
    d2h = rec_b + 112 + 5 * 8 + 32 + 4 + 80
    return 1e3 * wall / steps, h2d, d2h


def ess_geyer(x):
    """Effective sample size by Geyer's initial positive sequence on autocovariances."""
    x = np.asarray(x, float)
    n = len(x)
    if n < 4 or np.var(x) == 0:
        return float(n)
    xc = x - x.mean()
    f = np.fft.rfft(xc, 2 * n)
    acov = np.fft.irfft(f * np.conj(f))[:n] / n
    rho = acov / acov[0]
    s = 0.0
    for k in range(0, n - 1, 2):
        g = rho[k] + rho[k + 1]
        if g <= 0:
            break
        s += g
    tau = max(1.0, 2.0 * s - 1.0)
    return n / tau


def bench_replicas(torch, steps=50000, every=500, loop_steps=200, seed=20261203):
    """64 TIP4P replicas (216-2,048 molecules, log-uniform), 220-360 K geometric,
    stochastic-collision thermostat, rc 8.5 A, dt 2 fs, neighbour swaps every
    500 steps over 50,000 steps (the temperature slots alternate parity; FP64
    acceptance): all replicas in one context (CUDA-graph steps) vs one context
    per replica run one after the other.  Aggregate ns/day, and the acceptance
    of every neighbouring pair of temperature slots."""
    import genesis6_gb300 as g6
    from genesis6_gb300 import config
    R = 64
    sizes = config.replica_sizes(R, 216, 2048, seed)
    temps = 220.0 * (360.0 / 220.0) ** (np.arange(R) / (R - 1))
    boxes, recs = [], []
    for r in range(R):
        b = config.water_box("TIP4P", int(sizes[r]), seed + 100 + r, temp=float(temps[r]), dt=DT)
        boxes.append(b["L"]); recs.append(b["rec"])
    rate = 1.0   # collisions per molecule per ps

    def thermo(s, tr):
        return s.thermostats(len(tr), "andersen", temp=tr, rate=rate, seed=seed)
    # batched
    s = g6.RigidWater("TIP4P", sizes, np.array(boxes), path="custom", precision="mixed", rc=8.5)
    s.upload_state(np.concatenate(recs))
    th = thermo(s, temps)
    s.md_run(DT, 500, th, log=False)   # warm-up (graph capture, list builds, the lattice start relaxes)
    beta = 1.0 / np.array([th[r].temp for r in range(R)])
    pair_att = np.zeros(R - 1, int)
    pair_acc = np.zeros(R - 1, int)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    done = 0
    swap = 0
    while done < steps:
        k = min(every, steps - done)
        s.md_run(DT, k, th, log=False)
        done += k
        if done % every == 0:
            slots = np.array(sorted(range(R), key=lambda r: (-beta[r], r)))   # temperature slots before the attempt
            beta, a = s.replica_exchange(swap & 1, seed, swap, beta, th)
            for j in range(swap & 1, R - 1, 2):
                pair_att[j] += 1
                pair_acc[j] += int(a[slots[j]])
            swap += 1
    torch.cuda.synchronize()
    t_batched = time.perf_counter() - t0
    agg_batched = R * steps * DT * 1e-3 * 86400.0 / t_batched
    s.close()
    # one replica after another
    ctxs = []
    for r in range(R):
        c = g6.RigidWater("TIP4P", int(sizes[r]), boxes[r], path="custom", precision="mixed", rc=8.5)
        c.upload_state(recs[r])
        tc = thermo(c, [temps[r]])
        c.md_run(DT, 20, tc, log=False)
        ctxs.append((c, tc))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for c, tc in ctxs:
        c.md_run(DT, loop_steps, tc, log=False)
    torch.cuda.synchronize()
    t_loop = time.perf_counter() - t0
    agg_loop = R * loop_steps * DT * 1e-3 * 86400.0 / t_loop
    for c, _ in ctxs:
        c.close()
    rates = pair_acc / np.maximum(pair_att, 1)
    return {"replicas": R, "molecules": int(sizes.sum()), "min_size": int(sizes.min()), "max_size": int(sizes.max()),
            "batched_ns_per_day_aggregate": agg_batched, "loop_ns_per_day_aggregate": agg_loop,
            "batched_over_loop": agg_batched / agg_loop, "batched_steps": steps, "batched_seconds": t_batched,
            "loop_steps": loop_steps, "swap_every": every, "swap_attempts": int(pair_att.sum()),
            "accepted_swaps": int(pair_acc.sum()),
            "acceptance_per_slot_pair": [round(float(x), 3) for x in rates],
            "acceptance_slot_pairs_K": [[round(float(temps[j]), 1), round(float(temps[j + 1]), 1)] for j in range(R - 1)],
            "thermostat": "stochastic collisions, 1 per molecule per ps", "precision": "mixed",
            "structure": "all 64 replicas in every kernel of a step (head, pair kernel, integrator kernel), "
                         "16-step CUDA graphs; a swap attempt between graph launches"}


def mc_chains(C=32, N=1024, T=260.0, rc=9.0, seed=20261203, melt_steps=5000, md_steps=30000):
    """32 chains x 1,024 ST2 at 1.0 g/cm^3: seeded lattices melted by MD at 400 K,
    then MD at T (stochastic-collision thermostat, rc 9 A with a 2 A switch, dt
    2 fs), all chains in one replica context.  Returns boxes and records."""
    import genesis6_gb300 as g6
    from genesis6_gb300 import config
    boxes, recs = [], []
    for c in range(C):
        b = config.water_box("ST2", N, seed + 500 + c, temp=400.0)
        boxes.append(b["L"]); recs.append(b["rec"])
    s = g6.RigidWater("ST2", [N] * C, np.array(boxes), path="custom", precision="mixed", rc=rc, switch=2.0, skin=1.0)
    s.upload_state(np.concatenate(recs))
    s.md_run(DT, melt_steps, s.thermostats(C, "andersen", temp=400.0, rate=5.0, seed=seed), log=False)
    log = s.md_run(DT, md_steps, s.thermostats(C, "andersen", temp=T, rate=5.0, seed=seed + 1))
    rec = s.download_state()
    s.close()
    q = max(md_steps // 4, 1)
    return np.array(boxes), rec, {"md_U_last_quarters": [float(log[k * q:(k + 1) * q, :, 0].mean()) for k in range(4)],
                                  "md_T_last_quarter": float(log[3 * q:, :, 3].mean())}


def mc_compare(torch, s, rec_state, beta, seed, sweeps, records, w_move, w_energy):
    """One learned-vs-fixed comparison from rec_state with its own draws:
    training records from the fixed sampler, training, then `sweeps` sweeps of
    each sampler.  Returns the two samplers' numbers and the learned widths."""
    from genesis6_gb300 import _capi
    C, N = s.nrep, s.nmol[0]
    NF, NREC = _capi.MLP_NFEAT, _capi.MLP_RECORD
    s.upload_state(rec_state)
    ntr = records // C
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s.mc_run(ntr, seed, 10 ** 8, beta, 0.15, 0.15, mode="collect")       # training records
    loss = np.zeros(8)
    s._check(s.L.g6_mlp_objective(s.ctx, w_move, w_energy))
    s._check(s.L.g6_mlp_train(s.ctx, 8, 1024, 2e-3, seed, 0.15, 0.15, _capi.dptr(loss)))
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    # widths the trained network gives on the collected (plain-sampler) configurations
    nrec = min(200_000, ntr * C)
    rec = np.zeros((nrec, NREC), np.float32)
    cnt = ctypes.c_int64()
    s._check(s.L.g6_mlp_records(s.ctx, _capi.fptr(rec), nrec, ctypes.byref(cnt)))
    feat = np.ascontiguousarray(rec[:, :NF])
    wt = np.zeros(nrec); wr = np.zeros(nrec)
    s._check(s.L.g6_mlp_widths(s.ctx, _capi.fptr(feat), nrec, _capi.dptr(wt), _capi.dptr(wr)))
    out = {"training_records": ntr * C, "training_loss_first_last": [float(loss[0]), float(loss[-1])],
           "collect_and_train_seconds": t_train,
           "learned_widths_on_records": {"sigma_t_mean": float(wt.mean()), "sigma_r_mean": float(wr.mean()),
                                         "sigma_t_p10_p90": [float(np.percentile(wt, 10)), float(np.percentile(wt, 90))],
                                         "sigma_r_p10_p90": [float(np.percentile(wr, 10)), float(np.percentile(wr, 90))]}}
    for name in ("plain", "learned"):
        s.upload_state(rec_state)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = s.mc_run(sweeps * N, seed, 3 * 10 ** 8, beta, 0.15, 0.15, mode=name, sample_every=N)
        torch.cuda.synchronize()
        gpu_s = time.perf_counter() - t0
        samples = r["samples"]
        F, tau, ep, vir = s.force()
        ess = np.array([ess_geyer(samples[c]) for c in range(C)])
        u = samples.mean(1)
        var_mean = np.array([np.var(samples[c]) / max(ess[c], 1.0) for c in range(C)])
        out["fixed" if name == "plain" else name] = {
            "ess_total": float(ess.sum()), "gpu_seconds": gpu_s, "ess_per_gpu_s": float(ess.sum() / gpu_s),
            "us_per_trial": gpu_s / (sweeps * N) * 1e6,
            "mean_U_internal": float(u.mean()), "stderr_U": float(np.sqrt(var_mean.sum()) / C),
            "acceptance": float(r["accepted"].sum() / r["trials"].sum()), "sweeps": sweeps,
            "running_minus_full_energy_rel": float(np.abs(r["energy"] - ep).max() / np.abs(ep).max())}
    f, l = out["fixed"], out["learned"]
    out["ess_per_gpu_s_learned_over_fixed"] = l["ess_per_gpu_s"] / f["ess_per_gpu_s"]
    out["with_collect_and_train_charged"] = (l["ess_total"] / (l["gpu_seconds"] + t_train)) / f["ess_per_gpu_s"]
    out["ess_per_trial_learned_over_fixed"] = l["ess_total"] / f["ess_total"]
    sig = np.hypot(l["stderr_U"], f["stderr_U"])
    out["mean_U_difference_in_sigma"] = float(abs(l["mean_U_internal"] - f["mean_U_internal"]) / sig) if sig > 0 else None
    return out


def bench_umbrella(torch, s, rec_state, beta, seed, sweeps=20):
    """Umbrella chains (g6_mc_run_umbrella, mc2.F90:684-830) on the same 32 x 1,024 ST2
    state: fixed widths 0.15 A / 0.15 rad, an umbrella centred at each chain's current order
    parameter, `sweeps` sweeps per kind.  Wall time per trial (all chains in parallel) next to
    the plain chain's, and the incremental order parameter against a fresh evaluation."""
    N = s.nmol[0]
    ntr = sweeps * N
    ref = np.ones(21)
    coeff = {"ep": 1.0e-3, "q6": 1.0e5, "triangle": 1.0e3}
    out = {"sweeps": sweeps, "triangle_reference": "flat (21 bins)"}
    s.upload_state(rec_state)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s.mc_run(ntr, seed + 5, 10 ** 9, beta, 0.15, 0.15)
    torch.cuda.synchronize()
    plain = time.perf_counter() - t0
    out["plain_us_per_trial"] = plain / ntr * 1e6
    for kind in ("ep", "q6", "triangle"):
        s.upload_state(rec_state)
        op0 = s.order_parameter(kind, refhist=ref)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = s.mc_run_umbrella(ntr, seed + 5, 10 ** 9, beta, kind, op0, coeff[kind], refhist=ref)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        fresh = s.order_parameter(kind, refhist=ref)
        out[kind] = {"us_per_trial": wall / ntr * 1e6, "over_plain": wall / plain, "coeff": coeff[kind],
                     "acceptance": float(r["accepted"].sum() / r["trials"].sum()),
                     "op_start_mean": float(np.mean(op0)), "op_end_mean": float(np.mean(r["op"])),
                     "incremental_minus_fresh_max_rel": float(np.abs(r["op"] - fresh).max() / np.abs(fresh).max())}
    return out


def bench_mc(torch, seed=20261203, seeds=3, sweeps=3000, records=1_000_000, equil_sweeps=1000, w_move=0.0,
             w_energy=1.0, T=260.0, rc=9.0, md_steps=30000):
    """32 chains x 1,024 ST2 (custom path, Coulomb taper), T = 260 K, rc 9 A with
    a 2 A switch.  Chains start from MD-equilibrated liquid (melt at 400 K, then
    MD at T) and are equilibrated further by the fixed-width sampler; then, for
    each of `seeds` independent draw streams, the MLP is trained on `records`
    plain-sampler moves and both samplers run `sweeps` sweeps from the same
    state: fixed widths (0.15 A, 0.15 rad) vs the learned widths.  ESS of U per
    GPU-second (U sampled every sweep of 1,024 trials), <U> agreement per seed,
    and the ratio with the collect + train time charged to the learned sampler."""
    import genesis6_gb300 as g6
    C, N = 32, 1024
    t0 = time.perf_counter()
    boxes, rec0, md = mc_chains(C, N, T, rc, seed, md_steps=md_steps)
    t_md = time.perf_counter() - t0
    s = g6.RigidWater("ST2", [N] * C, boxes, path="custom", precision="mixed", rc=rc, switch=2.0, skin=0.0)
    s.upload_state(rec0)
    beta = 1.0 / T
    t0 = time.perf_counter()
    eq = s.mc_run(equil_sweeps * N, seed, 0, beta, 0.15, 0.15, sample_every=N)["samples"]
    torch.cuda.synchronize()
    t_equil = time.perf_counter() - t0
    rec_state = s.download_state()
    runs = [mc_compare(torch, s, rec_state, beta, seed + 17 * k, sweeps, records, w_move, w_energy)
            for k in range(seeds)]
    umbrella = bench_umbrella(torch, s, rec_state, beta, seed)
    s.close()
    ratios = [r["ess_per_gpu_s_learned_over_fixed"] for r in runs]
    charged = [r["with_collect_and_train_charged"] for r in runs]
    # <U> over the seeds: each seed's mean is one independent estimate, so the
    # scatter between seeds gives a standard error that does not rest on one
    # run's ESS estimate
    uf = np.array([r["fixed"]["mean_U_internal"] for r in runs])
    ul = np.array([r["learned"]["mean_U_internal"] for r in runs])
    pooled = None
    if len(runs) > 1:
        se = np.sqrt(uf.var(ddof=1) / len(uf) + ul.var(ddof=1) / len(ul))
        pooled = {"fixed": float(uf.mean()), "learned": float(ul.mean()),
                  "stderr_between_seeds": float(se),
                  "difference_in_sigma": float((ul.mean() - uf.mean()) / se) if se > 0 else 0.0,
                  "per_seed_stderr_over_between_seed_scatter_fixed":
                      float(np.mean([r["fixed"]["stderr_U"] for r in runs]) / uf.std(ddof=1)) if uf.std(ddof=1) > 0
                      else None}
    q = max(equil_sweeps // 4, 1)
    return {"chains": C, "molecules_per_chain": N, "model": "ST2 (custom path, Coulomb taper)", "T_K": T,
            "rc_A": rc, "start": "lattice, MD melt 5,000 steps at 400 K, MD %d steps at %g K (%.1f s)" % (md_steps, T, t_md),
            "md": md, "equilibration_sweeps": equil_sweeps, "equilibration_seconds": t_equil,
            "equilibration_U_quarters": [float(eq[:, k * q:(k + 1) * q].mean()) for k in range(4)],
            "objective": {"w_move": w_move, "w_energy": w_energy}, "seeds": seeds, "sweeps_per_sampler": sweeps,
            "ess_per_gpu_s_learned_over_fixed": float(np.median(ratios)),
            "ess_per_gpu_s_learned_over_fixed_per_seed": ratios,
            "with_collect_and_train_charged_per_seed": charged,
            "mean_U_difference_in_sigma_per_seed": [r["mean_U_difference_in_sigma"] for r in runs],
            "mean_U_over_seeds": pooled,
            "runs": runs, "umbrella": umbrella, "U_unit": "10 J/mol per chain (internal)"}


def bench_rdf(torch, n=N_BIG, rc=9.0, nbin=200, width=0.05, reps=5, seed=20261207):
    """Site-site distance histogram of a 32,768-molecule TIP4P configuration
    (g6_rdf: pair search, FP64 site positions, shared-memory histogram, read
    back) against the oracle's numpy counting of the same configuration on one
    host core; the two histograms must be equal."""
    import genesis6_gb300 as g6
    from genesis6_gb300 import config
    from oracle import analysis as orc_analysis
    b = config.water_box("TIP4P", n, seed, temp=TEMP, dt=DT)
    s = make_system("TIP4P", n, "mixed", b["L"], b["rec"])
    s.md_run(DT, 200, thermo_for(s), log=False)
    rec = s.download_state()
    s.rdf_counts(nbin, width)                      # warm-up (allocations, first launch)
    t0 = time.perf_counter()
    for _ in range(reps):
        h = s.rdf_counts(nbin, width)
    gpu_ms = (time.perf_counter() - t0) / reps * 1e3
    npair = ctypes.c_int64()
    s._check(s.L.g6_pairsearch(s.ctx, ctypes.byref(npair)))
    s.hbonds()
    t0 = time.perf_counter()
    for _ in range(reps):
        hb = s.hbonds()
    hb_ms = (time.perf_counter() - t0) / reps * 1e3
    s.close()
    com, quat = rec[:, 0:3], rec[:, 33:37]
    t0 = time.perf_counter()
    ho = orc_analysis.rdf_counts("TIP4P", com, quat, np.asarray(b["L"], float), rc, nbin, width)
    cpu_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    hbo = orc_analysis.hbonds("TIP4P", com, quat, np.asarray(b["L"], float), rc)
    hb_cpu_s = time.perf_counter() - t0
    hb_equal = set(map(tuple, hb.tolist())) == set(map(tuple, hbo.tolist()))
    return {"molecules": n, "pairs_within_rc": int(npair.value), "site_pairs_per_pair": 25, "nbin": nbin,
            "binwidth_A": width, "gpu_ms_per_call": gpu_ms,
            "cpu_baseline": {"s_per_call": cpu_s, "kind": "port", "cores": 1,
                             "sample": "the same configuration, oracle pair search + numpy counting"},
            "equal_to_cpu": bool(np.array_equal(h[0], ho)),
            "timing": "wall clock per g6_rdf call (pair search + positions + histogram + read-back)",
            "hbonds": {"bonds": int(len(hb)), "gpu_ms_per_call": hb_ms, "cpu_baseline_s_per_call": hb_cpu_s,
                       "equal_to_cpu": bool(hb_equal),
                       "timing": "wall clock per RigidWater.hbonds call (pair search, positions, "
                                 "O-H test, compaction, read-back of the bonds)"}}


def bench_rms(torch, rec_eq, L, snapshots=100, every=20):
    """Relative RMS force and torque error of the mixed path on `snapshots`
    configurations of a TIP4P-4096 Nose-Hoover trajectory (one every `every`
    steps), against the FP64 path (which follows the FP64 oracle to 1e-12)."""
    sm = make_system("TIP4P", N_MAIN, "mixed", L, rec_eq)
    s64 = make_system("TIP4P", N_MAIN, "fp64", L, rec_eq)
    th = thermo_for(sm)
    num_f = den_f = num_t = den_t = num_fs = num_ts = 0.0
    worst = 0.0
    for k in range(snapshots):
        sm.md_run(DT, every, th, log=False)
        rec = sm.download_state()
        s64.upload_state(rec)
        Fm, tm, _, _ = sm.force()
        Fs, ts, _ = sm.step_forces()
        F6, t6, _, _ = s64.force()
        num_f += float(np.sum((Fm - F6) ** 2)); den_f += float(np.sum(F6 ** 2))
        num_t += float(np.sum((tm - t6) ** 2)); den_t += float(np.sum(t6 ** 2))
        num_fs += float(np.sum((Fs - F6) ** 2)); num_ts += float(np.sum((ts - t6) ** 2))
        worst = max(worst, float(np.sqrt(np.sum((Fm - F6) ** 2) / np.sum(F6 ** 2))))
    sm.close(); s64.close()
    return {"snapshots": snapshots, "every_steps": every, "rms_force_rel": float(np.sqrt(num_f / den_f)),
            "rms_torque_rel": float(np.sqrt(num_t / den_t)), "worst_snapshot_force_rel": worst,
            "md_step_rms_force_rel": float(np.sqrt(num_fs / den_f)),
            "md_step_rms_torque_rel": float(np.sqrt(num_ts / den_t)),
            "against": "the FP64 path on the same configurations; rms_*: the force-only call (full list, lanes "
                       "combined in FP64), md_step_*: the MD step's pair kernel (g6_step_forces: its list form, "
                       "float-pair lanes, partner shares by float atomics)"}


def c3_state(model, seed, melt=2000, equil=2000, dt=0.001):
    """32,768 molecules of `model` at 1.0 g/cm^3 (L = 99.309 A), rc 9 A with the
    2 A switch, dt 1 fs: the seeded random-quaternion lattice melted for `melt`
    steps at 400 K, then `equil` steps at 300 K (both with the stochastic-collision
    thermostat, 5 collisions per molecule per ps), in mixed precision.  The 300 K
    stage makes the NVE run that follows start in equilibrium at 300 K.
    Returns (box, records)."""
    from genesis6_gb300 import config
    b = config.water_box(model, N_BIG, seed, temp=400.0, dt=dt)
    s = make_system(model, N_BIG, "mixed", b["L"], b["rec"])
    s.md_run(dt, melt, s.thermostats(1, "andersen", temp=400.0, rate=5.0, seed=seed), log=False)
    s.md_run(dt, equil, s.thermostats(1, "andersen", temp=300.0, rate=5.0, seed=seed + 1), log=False)
    rec = s.download_state()
    s.close()
    return b["L"], rec


def drift(log, n, dt):
    """Least-squares slope of H per molecule (kJ/mol) against time (ns)."""
    H = log[:, 0, 5] * 1e-3 / n
    tns = np.arange(len(H)) * dt * 1e-3
    return float(np.polyfit(tns, H, 1)[0])


def bench_c3(torch, flush, model="TIP4P", seed=20261205, steps=5000, snapshots=20, every=100, timed_steps=100):
    """The 32,768-molecule configuration: `model` at 1.0 g/cm^3, rc 9 A, dt 1 fs,
    lattice melted 2,000 steps at 400 K and equilibrated 2,000 steps at 300 K.
    Reported: device-timed ns/day of the mixed and FP64 steps (per-step CUDA
    events, L2 flushed, NVE); NVE energy drift over `steps` steps of each from
    the same start (wall clock gives their ns/day of a production run); and the
    relative RMS force and torque error of the mixed path against the FP64 path
    on `snapshots` configurations of the mixed NVE trajectory (one every `every`
    steps)."""
    dt = 0.001
    n = N_BIG
    L, start = c3_state(model, seed)
    out = {"model": model, "molecules": n, "dt_fs": 1.0,
           "start": "lattice, 2,000 steps at 400 K, 2,000 steps at 300 K (stochastic collisions)", "nve_steps": steps}
    sm = make_system(model, n, "mixed", L, start)
    s64 = make_system(model, n, "fp64", L, start)
    # RMS force/torque error on snapshots of the mixed trajectory
    num_f = den_f = num_t = den_t = num_fs = num_ts = 0.0
    for k in range(snapshots):
        sm.md_run(dt, every, sm.thermostats(1, "nve"), log=False)
        rec = sm.download_state()
        s64.upload_state(rec)
        Fm, tm, _, _ = sm.force()
        Fs, ts, _ = sm.step_forces()
        F6, t6, _, _ = s64.force()
        num_f += float(np.sum((Fm - F6) ** 2)); den_f += float(np.sum(F6 ** 2))
        num_t += float(np.sum((tm - t6) ** 2)); den_t += float(np.sum(t6 ** 2))
        num_fs += float(np.sum((Fs - F6) ** 2)); num_ts += float(np.sum((ts - t6) ** 2))
    out["rms_force_rel"] = float(np.sqrt(num_f / den_f))
    out["rms_torque_rel"] = float(np.sqrt(num_t / den_t))
    out["md_step_rms_force_rel"] = float(np.sqrt(num_fs / den_f))     # the MD step's own pair-kernel forces
    out["md_step_rms_torque_rel"] = float(np.sqrt(num_ts / den_t))
    out["rms_snapshots"] = {"count": snapshots, "every_steps": every, "against": "the FP64 path (oracle-pinned to 1e-12)"}
    # device-timed steps (NVE, one-step graphs with events, L2 flushed between steps)
    nve = lambda s: s.thermostats(1, "nve")
    for prec, s, k in (("mixed", sm, timed_steps), ("fp64", s64, max(5, timed_steps // 10))):
        s.upload_state(start)
        from genesis6_gb300 import _capi
        shape = _capi.Shape()
        s._check(s.L.g6_tune_shape(s.ctx, _capi.TUNE_SKIN, ctypes.byref(shape)))
        st, km, lg = timed_nve(torch, s, dt, k, 3, flush)
        out[prec + "_ms_per_step"] = float(st.mean())
        out[prec + "_ns_per_day"] = ns_per_day(float(st.mean()), dt)
        if prec == "mixed":
            pairs = float(lg[:, 0, 6].mean())
            out["pairs_within_rc"] = pairs
            out["force_kernel_ms"] = float(km.mean())
            out["force_tflops"] = FLOPS_PER_PAIR[model] * pairs / (float(km.mean()) * 1e-3) / 1e12
            out["shape"] = shape.as_dict()
        else:
            out["fp64_shape"] = shape.as_dict()
    out["mixed_over_fp64"] = out["fp64_ms_per_step"] / out["mixed_ms_per_step"]
    # NVE drift from the same start
    for prec, s in (("mixed", sm), ("fp64", s64)):
        s.upload_state(start)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        log = s.md_run(dt, steps, nve(s))
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        out[prec + "_nve"] = {"drift_kJ_per_mol_per_ns": drift(log, n, dt), "T_mean_K": float(log[:, 0, 3].mean()),
                              "ns_per_day_wall": ns_per_day(1e3 * wall / steps, dt)}
    sm.close(); s64.close()
    out["timing"] = ("ns_per_day: per-step CUDA events, L2 flushed between steps; ns_per_day_wall: wall clock of "
                     "the 5,000-step NVE run (16-step CUDA graphs, no flush)")
    return out


def timed_nve(torch, s, dt, steps, warmup, flush):
    """Like timed_md for an NVE run at time step dt."""
    L = s.L
    th = s.thermostats(1, "nve")
    s.md_run(dt, warmup, th, log=False)
    sp = ctypes.c_void_p()
    s._check(L.g6_stream(s.ctx, ctypes.byref(sp)))
    stream = torch.cuda.ExternalStream(sp.value)
    a, b = ctypes.c_double(), ctypes.c_double()
    log = np.zeros((steps, 1, 10))
    step_ms, kms = np.zeros(steps), np.zeros(steps)
    s._check(L.g6_set_step_timing(s.ctx, 2))
    torch.cuda.synchronize()
    s._check(L.g6_md_begin(s.ctx, dt, steps, th, 1))
    for k in range(steps):
        with torch.cuda.stream(stream):
            flush.add_(1.0)
        s._check(L.g6_md_advance(s.ctx, 1))
        s._check(L.g6_step_times(s.ctx, ctypes.byref(a), ctypes.byref(b)))
        step_ms[k], kms[k] = a.value, b.value
    s._check(L.g6_md_end(s.ctx, th, log.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
    s._check(L.g6_set_step_timing(s.ctx, 0))
    torch.cuda.synchronize()
    return step_ms, kms, log


def nve_drift_4096(torch, steps=5000, dt=0.001):
    """NVE energy drift of TIP4P-4096 from the stored equilibrated state, dt 1 fs,
    `steps` steps: the GPU's mixed and FP64 paths and, as the CPU baseline of the
    drift, the oracle's FP64 restatement of the reference MD step (StdForce
    arithmetic, all host cores) from the same start."""
    import oracle
    from genesis6_gb300 import config
    b = config.load_start(START, dt)
    n = N_MAIN
    out = {"molecules": n, "dt_fs": 1.0, "steps": steps, "start": "tests/golden/tip4p4096_eq.npz"}
    for prec in ("mixed", "fp64"):
        s = make_system("TIP4P", n, prec, b["L"], b["rec"])
        log = s.md_run(dt, steps, s.thermostats(1, "nve"))
        out[prec] = {"drift_kJ_per_mol_per_ns": drift(log, n, dt), "T_mean_K": float(log[:, 0, 3].mean())}
        s.close()
    oracle.build()
    th = np.zeros(10)
    t0 = time.perf_counter()
    _, _, lo = oracle.md_run_threaded("TIP4P", b["rec"], b["L"], [RC] * 3, RC - SWITCH, RC, dt, steps, th,
                                      os.cpu_count() or 1)
    wall = time.perf_counter() - t0
    out["cpu_baseline_oracle"] = {"drift_kJ_per_mol_per_ns": drift(lo[:, None, :], n, dt),
                                  "T_mean_K": float(lo[:, 3].mean()), "seconds": wall,
                                  "kind": "port", "cores": os.cpu_count() or 1}
    return out


def run_gpu(args, rank, world, local):
    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import genesis6_gb300 as g6
    from genesis6_gb300 import config
    g6.lib()
    b = equilibrated_start()
    L = b["L"]
    s = make_system("TIP4P", N_MAIN, "mixed", L, b["rec"])
    # the first step from the stored state, for comparison with the reference arm's
    first_epot = float(s.md_run(DT, 1, thermo_for(s))[0, 0, 0])
    s.upload_state(b["rec"])
    if args.equil:   # optional extra untimed steps
        s.md_run(DT, args.equil, thermo_for(s), log=False)
    rec_eq = s.download_state()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")   # 256 MiB > 129 MB L2

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    s.upload_state(rec_eq)
    # N > 1: a replica-exchange ensemble sharded over the ranks -- rank r runs its
    # own TIP4P-4096 system at T_r = 300 K * 1.01^r and the ranks attempt
    # neighbour exchanges (gathered over a gloo group) between chunks of steps
    exchange, temp_r = None, TEMP
    if world > 1:
        from genesis6_gb300 import replicas
        temp_r = TEMP * 1.01 ** rank
        host_group = dist.new_group(backend="gloo")
        shard = replicas.ShardedExchange(1, group=host_group)
        beta_r = [1.0 / temp_r]
        accepted = []

        def exchange(c, th):
            t0 = time.perf_counter()
            res = shard.attempt(c & 1, 20261203, c, s.last_epot(), beta_r, [th[0].temp])
            replicas.apply_exchange(s, th, res)
            beta_r[0] = float(res["beta"][0])
            accepted.append(int(res["accepted_global"].sum()))
            return 1e3 * (time.perf_counter() - t0)
    barrier()
    with Clocks(local) as clk:
        step_ms, kms, log, shape = timed_md(torch, s, args.steps, args.warmup, flush, temp=temp_r, exchange=exchange,
                                            chunks=4 if exchange else 1)
        barrier()
    total_ms = float(step_ms.sum())
    if dist:
        t = torch.tensor([total_ms], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    ms = total_ms / args.steps
    value = world * ns_per_day(ms)

    # plain FP64 mode, same state
    s64 = make_system("TIP4P", N_MAIN, "fp64", L, rec_eq)
    k64 = max(5, min(args.steps, 60))
    step64, kms64, log64, shape64 = timed_md(torch, s64, k64, min(args.warmup, 5), flush)
    ms64 = float(step64.mean())

    # e2e through the host-buffer entry point
    s.upload_state(rec_eq)
    e2e_steps = max(10, min(args.steps, 200))
    e2e_ms, h2d, d2h = e2e_md(torch, s, rec_eq, e2e_steps)

    big = None if args.no_32k else bench_c3(torch, flush, "TIP4P")

    if rank != 0:
        return
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except Exception:
        pass
    fp32_peak = fp32_peak_tflops(torch)
    pairs = float(log[:, 0, 6].mean())
    kmean = float(kms.mean())
    achieved = FLOPS_PER_PAIR["TIP4P"] * pairs / (kmean * 1e-3) / 1e12
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "k_pairs_tip4p4096_step.txt")
    if os.path.exists(tpath):
        for l in open(tpath):
            if l.startswith("traffic_bytes_per_launch:"):
                traffic = float(l.split(":")[1])
    cpu = None if args.no_cpu else cpu_md_rate()
    rex = None if args.no_extra else bench_replicas(torch)
    mcb = None if args.no_extra else bench_mc(torch)
    rms = None if args.no_extra else bench_rms(torch, rec_eq, L)
    t5p = None if (args.no_extra or args.no_32k) else bench_c3(torch, flush, "TIP5P", seed=20261206)
    drift4k = None if (args.no_extra or args.no_cpu) else nve_drift_4096(torch)
    rdf = None if (args.no_extra or args.no_32k) else bench_rdf(torch)
    line = {
        "metric": METRIC, "value": value, "unit": "ns/day", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 site math / f64 accumulation", "data": "synthetic (seeded lattice, random quaternions, "
        "Maxwell-Boltzmann 300 K, then 2,000 FP64 Nose-Hoover steps: the stored state both arms start from)", "config": config_block(args, world),
        "fp64_ns_per_day": world * ns_per_day(ms64), "fp64_ms_per_step": ms64, "mixed_over_fp64": ms64 / ms,
        "fp64_shape": shape64,
        "first_step_epot": first_epot,
        "fp64_gpu_over_fp64_cpu": None if cpu is None else ns_per_day(ms64) / cpu["value"],
        "tip4p_32k": big,
        "tip5p_32k": t5p,
        "nve_drift_4096": drift4k,
        "mixed_rms_error_4096": rms,
        "replica_exchange": rex,
        "mc_learned_vs_fixed": mcb,
        "rdf_32k": rdf,
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved / fp32_peak, "traffic": traffic,
                     "kernel": ("k_pairs<TIP4P, mixed, MD step, %s> (in-range compaction of the Verlet rows + "
                                "FP32 site loops%s; the Gear corrector runs in k_integrate_mixed)"
                                % (("half list", ", each pair once, the partner's share by vector atomics")
                                   if shape.get("step_half") else ("full list", ", each pair from both sides"))),
                     "flops_per_pair": FLOPS_PER_PAIR["TIP4P"],
                     "pairs_per_launch": pairs, "kernel_ms": kmean, "shape": shape,
                     "peak_source": "cuBLAS SGEMM 8192^3 with TF32 off, measured in this run (FP32 CUDA-core "
                                    "pipe; the kernel uses no tensor cores and moves a few MB per launch)",
                     "hbm_peak_gbs": peaks.get("hbm_gbs")},
        "cpu_baseline": None if cpu is None else {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "e2e": {"value": world * ns_per_day(e2e_ms), "unit": "ns/day", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms, "entry": "g6_md_step_host"},
        "gpu_launches": 3 * args.steps,
        "clocks": clk.summary(),
    }
    print(json.dumps(line))


def run_profile(args):
    """Workloads for ncu captures: nothing is timed and no JSON line is printed."""
    import genesis6_gb300 as g6
    from genesis6_gb300 import config
    if args.profile == "rdf":   # --steps calls of g6_rdf on 32,768 TIP4P (lattice start)
        b = config.water_box("TIP4P", N_BIG, 20261207, temp=TEMP, dt=DT)
        s = make_system("TIP4P", N_BIG, "mixed", b["L"], b["rec"])
        for _ in range(args.steps):
            h = s.rdf_counts(200, 0.05)
        print("rdf ok: %d counts" % int(h.sum()))
    elif args.profile == "e2e":   # --steps host-buffer steps (g6_md_step_host, pinned record) of TIP4P-4096
        import torch
        b = equilibrated_start()
        s = make_system("TIP4P", N_MAIN, "mixed", b["L"], b["rec"])
        ms, _, _ = e2e_md(torch, s, b["rec"], args.steps)
        print("e2e ok: %.1f us per host-buffer step" % (1e3 * ms))
    elif args.profile == "md":
        if args.n == N_MAIN:
            b = equilibrated_start()
        else:
            b = config.water_box("TIP4P", args.n, 20261203, temp=TEMP, dt=DT)
        s = make_system("TIP4P", args.n, args.prec, b["L"], b["rec"])
        s.md_run(DT, 20, thermo_for(s), log=False)
        from genesis6_gb300 import _capi
        shape = _capi.Shape()
        if args.shape:
            f = args.shape.split(",")
            lp, slp, mpw, sk = f[:4]
            half = int(f[4]) if len(f) > 4 else 1
            shape = _capi.Shape(lpi=int(lp), step_lpi=int(slp), step_mpw=int(mpw), skin=float(sk), cap=0, step_ms=0.0,
                                step_half=half)
            s._check(s.L.g6_set_shape(s.ctx, ctypes.byref(shape)))
        else:
            s._check(s.L.g6_tune_shape(s.ctx, _capi.TUNE_SKIN, ctypes.byref(shape)))
        print("shape:", shape.as_dict())
        log = s.md_run(DT, args.steps, thermo_for(s))
        print("md ok: %d steps, last T %.1f K" % (args.steps, float(log[-1, 0, 3])))
    else:
        C, N, seed = 32, 1024, 20261203
        boxes, rec0, _ = mc_chains(C, N, 260.0, 9.0, seed, melt_steps=1000, md_steps=2000)
        s = g6.RigidWater("ST2", [N] * C, boxes, path="custom", precision="mixed", rc=9.0, switch=2.0, skin=0.0)
        s.upload_state(rec0)
        mode = "plain"
        if args.profile == "mc-learned":
            s.mc_run(1024, seed, 10 ** 8, 1.0 / 260.0, mode="collect")
            s._check(s.L.g6_mlp_objective(s.ctx, 0.0, 1.0))
            s._check(s.L.g6_mlp_train(s.ctx, 1, 1024, 2e-3, seed, 0.15, 0.15, None))
            mode = "learned"
        for k in range(2):
            r = s.mc_run(args.steps, seed, k * args.steps, 1.0 / 260.0, mode=mode)
        print("mc ok (%s): acceptance %.3f" % (mode, r["accepted"].sum() / r["trials"].sum()))
    s.close()


def main():
    args = parse()
    rank, world, local = dist_info()
    if args.profile:
        run_profile(args)
        return
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    run_gpu(args, rank, world, local)


if __name__ == "__main__":
    main()
