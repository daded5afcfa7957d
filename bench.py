#!/usr/bin/env python
"""Benchmark: learned-proposal vs plain Metropolis chains of the N=100 complex RBM.

Workload (the configuration the headline metric is quoted on): complex RBM with
N=100 visible and M=400 hidden units, parameters complex Normal(0, 0.1^2) drawn from
PCG64(104); periodic 1D transverse-field Ising chain with h=1.0 (200 Pauli strings);
16384 walkers per GPU.  Two chains run on the same GPU:

* plain: single-spin-flip Metropolis (the reference's method); one step = one row =
  `--sweeps-per-row` sweeps of N proposals per walker, then the local energy of every
  walker;
* learned: after the same thermalisation and `--train-steps` steps of online training
  (cross-entropy to the locally balanced proposal + Adam on the first `--train-walkers`
  walkers), the frozen proposal network's cluster-flip Metropolis-Hastings steps; one
  row = `--learned-steps-per-row` steps (a row of about the plain row's duration), then
  the local energy of every walker.

The headline metric is effective samples per second of the learned chain: walkers x
rows / tau_int(E_loc) per second of its timed rows, tau_int (in rows) from Sokal's
automatic windowing (c = 5) of the walkers' E_loc series; the plain chain's figures sit
beside it ("plain"), with E_loc/s, the energy standard error per spin, and a flag where
the window did not converge (tau_int is then a lower bound).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--workload serving|s_matrix]

`--workload serving` times the batched serving of 64 uneven RBMs instead (one line of
its own); `--workload s_matrix` times get_S_matrix of the N=64, M=128 RBM over 16384
Monte Carlo samples (P = 8448).

For N > 1 run under torchrun: every rank samples its own replica of the walker sets
(Philox keys offset by rank), no data-path collective; value = all ranks' effective
samples / max over ranks of the timed region.
"""
import argparse
import json
import multiprocessing as mp
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

N_SPINS, M_HIDDEN, SIGMA, PARAM_SEED, FIELD, WALKERS = 100, 400, 0.1, 104, 1.0, 16384
# single-flip sweeps from random +-1 starts before either chain is measured: the plain
# chain's E_loc per spin relaxes for about 6000 sweeps on this glassy target (sigma 0.1) and
# then stays level; both chains start from these equilibrated configurations
THERM_SWEEPS = 8000
METRIC = "effective samples/s (ESS of E_loc) at N=100: learned-proposal MCMC (plain single-flip beside)"
UNIT = "samples/s"
L2_FLUSH_BYTES = 256 << 20
# DRAM bytes of one sampler launch: dram__bytes_read.sum + dram__bytes_write.sum of an ncu
# capture of rbm_mc_kernel<13,2> on these 16384 walkers
SAMPLER_DRAM_BYTES = 1.059e6

# algorithmic FP32 flops of the sampler, from the operation list of
# rbmongpu_gb300/csrc/device_math.cuh and rbm_impl.cuh (FMA = 2, mul/add/div = 1)
FLOPS_LC_RE = 37          # Re f(theta), Metropolis test
FLOPS_LC_C = 44           # complex f(theta), measurement
FLOPS_PROPOSAL_ANGLE = FLOPS_LC_RE + 4 + 2     # theta update (2 FMA) + difference and sum
FLOPS_ELOC_ANGLE = FLOPS_LC_C + 4 + 4          # theta'' update + complex difference and sum


def workload():
    rng = np.random.Generator(np.random.PCG64(PARAM_SEED))
    b = rng.normal(0, SIGMA, M_HIDDEN) + 1j * rng.normal(0, SIGMA, M_HIDDEN)
    W = rng.normal(0, SIGMA, (N_SPINS, M_HIDDEN)) + 1j * rng.normal(0, SIGMA, (N_SPINS, M_HIDDEN))
    return b, W


def flops_per_sweep(N=N_SPINS, M=M_HIDDEN):
    """FP32 flops of one sweep of one walker: N proposals + the angle refresh."""
    return N * M * FLOPS_PROPOSAL_ANGLE + 2 * N * M + FLOPS_LC_RE * M


def flops_per_eloc(N=N_SPINS, M=M_HIDDEN, n_offdiag=N_SPINS):
    return 2 * N * M + FLOPS_LC_C * M + n_offdiag * M * FLOPS_ELOC_ANGLE


def tau_int(series, c=5.0):
    """Integrated autocorrelation time (in rows) of E_loc, Sokal's automatic windowing:
    tau(W) = 1 + 2 sum_{t=1}^{W} rho(t), smallest W with W >= c tau(W); rho averaged over
    walkers, each series centred on the all-walker mean.  series: [K, walkers].
    Returns (tau, window, converged); not converged means no window W < K satisfied the
    rule, and tau is then a lower bound."""
    x = np.asarray(series.real, np.float64)
    x = x - x.mean()
    K = x.shape[0]
    f = np.fft.rfft(x, n=2 * K, axis=0)
    ac = np.fft.irfft(f * np.conj(f), n=2 * K, axis=0)[:K].mean(axis=1) / np.arange(K, 0, -1)
    if ac[0] <= 0:
        return 1.0, 1, True
    rho = ac / ac[0]
    tau, window = 1.0, 1
    for window in range(1, K):
        tau = 1.0 + 2.0 * rho[1:window + 1].sum()
        if window >= c * tau:
            return max(tau, 1.0), window, True
    return max(tau, 1.0), window, False


def series_stats(series, seconds, N=N_SPINS):
    """ESS figures of an E_loc series [rows, walkers] measured over `seconds`."""
    x = np.asarray(series.real, np.float64)
    rows, B = x.shape
    tau, window, ok = tau_int(series)
    se = x.std() * np.sqrt(tau / x.size)
    wm = x.mean(axis=0)
    se_walkers = wm.std(ddof=1) / np.sqrt(B)
    # stationarity: second-half minus first-half mean, in standard errors of the walker means
    h = rows // 2
    m1, m2 = x[:h].mean(axis=0), x[h:].mean(axis=0)
    drift = (m2.mean() - m1.mean()) / np.sqrt((m1.var(ddof=1) + m2.var(ddof=1)) / B) if h > 0 else None
    return {"ess": x.size / tau, "ess_per_s": x.size / tau / seconds, "tau_int_rows": tau, "tau_window": window,
            "tau_converged": ok, "rows": rows, "seconds": seconds, "eloc_per_s": x.size / seconds,
            "energy_per_spin": x.mean() / N, "se_per_spin": se / N, "se_per_spin_walker_means": se_walkers / N,
            "ess_walker_means": x.var() / se_walkers ** 2 if se_walkers > 0 else None,
            "half_drift_in_se": float(drift) if drift is not None else None}


# --------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([v.strip() for v in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        sm = [float(r[0]) for r in self.rows if len(r) >= 8 and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) >= 8 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows if len(r) >= 8 for k in range(4) if r[4 + k] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


# --------------------------------------------------------------------- CPU chains
def _cpu_worker(args):
    """One CPU chain of the same workload with the CPU restatement (FP64, the reference's
    arithmetic), persistent across calls; returns (seconds, E_loc series)."""
    chain, sweeps, state_path = args
    from oracle import pyoracle as po
    b, W = workload()
    psi = po.RBM(b, W)
    from rbmongpu_gb300.operators import tfim_chain
    op = po.Op(*tfim_chain(N_SPINS, 1.0, FIELD))
    if os.path.exists(state_path):
        st = np.load(state_path)
        state = (st["spins"].copy(), st["rng"].copy(), [1])
    else:
        state = (np.zeros((1, po.nwords(N_SPINS)), np.uint64), np.zeros(1, np.uint64), [0])
    therm = 0 if state[2][0] else 2
    t0 = time.perf_counter()
    _, _, el, _, _ = po.mc_run(psi, op, 1, sweeps, 1, therm, rng=po.OR_RNG_PHILOX, seed=7000, prec=po.OR_PREC_REF64,
                               chain_begin=chain, total_chains=4096, state=state)
    dt = time.perf_counter() - t0
    np.savez(state_path, spins=state[0], rng=state[1])
    return dt, el[:, 0]


def cpu_chains(steps, seconds_per_step, workers, tmpdir):
    """Runs `workers` persistent CPU chains for `steps` steps of about seconds_per_step."""
    ctx = mp.get_context("spawn")
    with ctx.Pool(workers) as pool:
        dt, _ = pool.map(_cpu_worker, [(w, 1, os.path.join(tmpdir, f"calib{w}.npz")) for w in range(workers)])[0]
        sweeps = max(1, int(seconds_per_step / max(dt, 1e-3)))
        series, wall = [], 0.0
        for k in range(steps):
            t0 = time.perf_counter()
            out = pool.map(_cpu_worker, [(w, sweeps, os.path.join(tmpdir, f"s{w}.npz")) for w in range(workers)])
            wall += time.perf_counter() - t0
            series.append(np.stack([o[1] for o in out], axis=1))
    return np.concatenate(series, axis=0), wall, sweeps


# --------------------------------------------------------------------- ranks
def combine_ranks(tot, tmax, device):
    """Whole-job figures of independent replicas: sums of `tot` (effective samples,
    samples) and maxima of `tmax` (seconds) over the ranks of the default process group."""
    import torch
    t1 = torch.tensor(np.asarray(tot, np.float64), device=device)
    t2 = torch.tensor(np.asarray(tmax, np.float64), device=device)
    torch.distributed.all_reduce(t1, op=torch.distributed.ReduceOp.SUM)
    torch.distributed.all_reduce(t2, op=torch.distributed.ReduceOp.MAX)
    return t1.cpu().numpy(), t2.cpu().numpy()


def learned_slices(args, walkers):
    """walker slices of a frozen learned row (Chain.set_learned_streams; 0 = automatic:
    two from 8192 walkers)"""
    return args.learned_streams or (2 if walkers >= 8192 else 1)


def replica_seeds(rank):
    """Philox keys of the rank's plain chain, learned chain and proposal network: every rank
    samples its own replica of the walker sets."""
    return 1000 + rank, 3000 + rank, 2000 + rank


# --------------------------------------------------------------------- GPU arms
def run_gpu(args, rank, world, local_rank):
    import torch
    import rbmongpu_gb300 as rg

    torch.cuda.set_device(local_rank)
    rg.setDevice(local_rank)
    b, W = workload()
    psi = rg.Psi(np.zeros(N_SPINS), np.zeros(N_SPINS), b, W, 1.0, False, True)
    op = rg.Operator(*rg.operators.tfim_chain(N_SPINS, 1.0, FIELD))
    B, K, Wm = args.walkers, args.steps, args.warmup
    S, L = args.sweeps_per_row, args.learned_steps_per_row
    sp = rg.library_stream()
    stream = torch.cuda.ExternalStream(sp)
    eloc = torch.empty((K, B, 2), dtype=torch.float64, device="cuda")
    scratch = torch.empty((B, 2), dtype=torch.float64, device="cuda")
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    def sync():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def timed_rows(n, row):
        """per-row milliseconds (CUDA events on the library stream), L2 flushed between rows"""
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(n)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(n)]
        with torch.cuda.stream(stream):
            for k in range(n):
                flush.fill_(k & 0xFF)
                starts[k].record(stream)
                row(k)
                ends[k].record(stream)
        torch.cuda.synchronize()
        return np.array([a.elapsed_time(e) for a, e in zip(starts, ends)])

    def series_of(n):
        return eloc[:n].cpu().numpy().view(np.complex128)[..., 0]

    clocks = ClockSampler(local_rank)
    # ---- plain single-flip chain
    seed_plain, seed_learned, seed_net = replica_seeds(rank)
    plain = rg.Chain(psi, B, seed=seed_plain)
    with torch.cuda.stream(stream):
        plain.sweep_async(psi, None, THERM_SWEEPS, 1, 0, sp)
    sync()
    start = plain.checkpoint()["spins"]   # the learned chain starts here too
    with torch.cuda.stream(stream):
        for _ in range(Wm):
            plain.sweep_async(psi, op, S, S, scratch.data_ptr(), sp)
    sync()
    clocks.start()
    _, a0, p0 = plain.state()
    plain_ms = timed_rows(K, lambda k: plain.sweep_async(psi, op, S, S, eloc[k].data_ptr(), sp))
    _, a1, p1 = plain.state()
    plain_series = series_of(K)
    # the sampler kernel alone (one launch of S sweeps), for its roofline
    kernel_ms = timed_rows(max(3, K // 20), lambda k: plain.sweep_async(psi, None, S, 1, 0, sp))
    plain_accept = (a1 - a0) / max(p1 - p0, 1)

    # ---- learned-proposal chain
    prop = rg.Proposal(N_SPINS, seed=seed_net, lr=1e-3)
    lc = rg.Chain(psi, B, seed=seed_learned)
    lc.set_learned_streams(args.learned_streams)
    zero = np.zeros(B, np.uint64)
    lc.restore(dict(spins=start, rng_index=zero, accepts=zero, proposals=zero))
    sync()
    t0 = time.perf_counter()
    with torch.cuda.stream(stream):
        lc.learned_async(psi, None, prop, args.train_steps, args.train_walkers, 1, 0, sp)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    with torch.cuda.stream(stream):
        for _ in range(Wm):
            lc.learned_async(psi, op, prop, L, 0, L, scratch.data_ptr(), sp)
    sync()
    _, a0, p0 = lc.state()
    learned_ms = timed_rows(K, lambda k: lc.learned_async(psi, op, prop, L, 0, L, eloc[k].data_ptr(), sp))
    _, a1, p1 = lc.state()
    clk = clocks.stop()
    learned_series = series_of(K)
    learned_accept = (a1 - a0) / max(p1 - p0, 1)

    plain_stats = series_stats(plain_series, float(plain_ms.sum()) / 1e3)
    learned_stats = series_stats(learned_series, float(learned_ms.sum()) / 1e3)

    # end to end through the public API with host buffers: per row the RBM parameters go
    # host -> device (psi.params) and the row's local energies device -> host (pinned)
    e2e_K = max(4, K // 10)
    p_host = psi.params
    pinned = torch.empty((B, 2), dtype=torch.float64, pin_memory=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(e2e_K):
        psi.params = p_host
        with torch.cuda.stream(stream):
            lc.learned_async(psi, op, prop, L, 0, L, scratch.data_ptr(), sp)
            pinned.copy_(scratch, non_blocking=True)
        stream.synchronize()
        _ = pinned.numpy().view(np.complex128)[:, 0].mean()
    e2e_s = time.perf_counter() - t0
    h2d = (N_SPINS + 1) * ((M_HIDDEN + 31) // 32 * 32) * 8     # complex64 W and b, padded rows
    d2h = B * 16

    fp32_peak = None
    if rank == 0:
        import ctypes
        from rbmongpu_gb300._lib import call
        v = ctypes.c_double()
        call("rbmg_probe_fp32_tflops", 20000, ctypes.byref(v))
        fp32_peak = v.value

    # whole-job sums over ranks (walker sets are independent replicas); times are maxima
    tot = np.array([learned_stats["ess"], plain_stats["ess"], B * e2e_K / learned_stats["tau_int_rows"],
                    learned_series.size, plain_series.size], np.float64)
    tmax = np.array([learned_stats["seconds"], plain_stats["seconds"], e2e_s], np.float64)
    if world > 1:
        tot, tmax = combine_ranks(tot, tmax, "cuda")
    return dict(tot=tot, tmax=tmax, plain=plain_stats, learned=learned_stats, plain_ms=plain_ms,
                learned_ms=learned_ms, kernel_ms=kernel_ms, plain_accept=plain_accept, learned_accept=learned_accept,
                train_s=train_s, e2e_K=e2e_K, h2d=h2d, d2h=d2h, clocks=clk, fp32_peak=fp32_peak)


# --------------------------------------------------------------------- serving workload
def serving_instances(rg):
    """64 complex RBMs: N uniform in {16, 24, ..., 144}, alpha in {1, 2, 4}, parameters complex
    Normal(0, 0.05^2) from PCG64(105000 + i), periodic TFIM with h uniform in [0.5, 2],
    256 N / 16 walkers each (PCG64(105) draws the shapes)."""
    rng = np.random.Generator(np.random.PCG64(105))
    inst = []
    for i in range(64):
        N = int(rng.choice(np.arange(16, 145, 8)))
        alpha = int(rng.choice([1, 2, 4]))
        h = float(rng.uniform(0.5, 2.0))
        pr = np.random.Generator(np.random.PCG64(105_000 + i))
        M = alpha * N
        b = pr.normal(0, 0.05, M) + 1j * pr.normal(0, 0.05, M)
        W = pr.normal(0, 0.05, (N, M)) + 1j * pr.normal(0, 0.05, (N, M))
        psi = rg.Psi(np.zeros(N), np.zeros(N), b, W, 1.0, False, True)
        inst.append((psi, rg.Operator(*rg.operators.tfim_chain(N, 1.0, h)), 256 * N // 16, 5000 + i))
    return inst


def run_serving(args):
    """One step = one replay of the batch graph: a sweep of every walker of the 64 networks,
    their local energies and every network's O_k sums."""
    import torch
    import rbmongpu_gb300 as rg
    torch.cuda.set_device(0)
    inst = serving_instances(rg)
    batch = rg.Batch(inst)
    batch.run(100, 1)
    tune = batch.autotune(sweeps=1, reps=3)
    sp = rg.library_stream()
    stream = torch.cuda.ExternalStream(sp)
    for _ in range(args.warmup):
        batch.run(0, 1)
    K = args.steps
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    clocks = ClockSampler(0)
    clocks.start()
    for k in range(K):
        with torch.cuda.stream(stream):
            flush.fill_(k & 0xFF)
            starts[k].record(stream)
        batch.run(0, 1)
        with torch.cuda.stream(stream):
            ends[k].record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = np.array([a.elapsed_time(e) for a, e in zip(starts, ends)])
    walkers = sum(w for _, _, w, _ in inst)
    # end to end: the replay plus every network's energy and gradient back on the host
    e2e_K = max(3, K // 5)
    t0 = time.perf_counter()
    d2h = 0
    for _ in range(e2e_K):
        batch.run(0, 1)
        for q in range(len(inst)):
            E, g, _ = batch.result(q)
            d2h += 16 * inst[q][2] + 2 * 8 * (inst[q][0].N + 1) * ((inst[q][0].M + 31) // 32 * 32)
    e2e_s = time.perf_counter() - t0
    flops = 0
    for psi, _, w, _ in inst:
        N, M = psi.N, psi.M
        flops += w * (flops_per_sweep(N, M) + flops_per_eloc(N, M, N) + 8 * (N + 1) * M)
    peak = None
    import ctypes
    from rbmongpu_gb300._lib import call
    v = ctypes.c_double()
    call("rbmg_probe_fp32_tflops", 20000, ctypes.byref(v))
    peak = v.value
    sec = float(ms.mean()) / 1e3
    w_shape, rows, blocks = batch.shape
    line = {
        "metric": "serving: walker-sweeps/s with E_loc and O_k sums, 64 uneven RBMs in one persistent launch",
        "value": walkers / sec, "unit": "walker-sweeps/s", "n_gpus": 1, "steps": K, "warmup": args.warmup,
        "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (complex64)", "data": "synthetic (seeded PCG64 parameters)",
        "config": {"workload": "serving_64_rbm_n16_144_alpha124_tfim", "instances": len(inst), "walkers": walkers,
                   "step": "1 sweep + E_loc of every walker + O_k sums (one CUDA-graph replay)",
                   "shape": {"warps_per_block": w_shape, "tile_rows": rows, "blocks": blocks,
                             "register_cap": batch.register_cap},
                   "autotune_ms": {f"r{c}_{a}x{b}": t for (c, a, b), t in tune.items()},
                   "l2": "flushed between timed steps"},
        "eloc_per_s": walkers / sec,
        "e2e": {"value": walkers * e2e_K / e2e_s, "unit": "walker-sweeps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": int(d2h / e2e_K)},
        "gpu_launches": K,
        "roofline": {"bound": "fp32", "achieved": flops / sec / 1e12, "peak": peak, "unit": "TFLOP/s",
                     "frac": flops / sec / 1e12 / peak, "traffic": None,
                     "peak_source": "measured in this run by the library's FP32 FMA probe kernel",
                     "kernel": "serve_kernel (persistent)", "flops_per_launch": flops},
        "cpu_baseline": None,
        "clocks": clk,
    }
    print(json.dumps(line))


# --------------------------------------------------------------------- S-matrix workload
def measured_peak(key):
    """A roofline denominator from MEASURED_PEAKS.json beside this file (None if absent)."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)[key])
    except (OSError, KeyError, ValueError):
        return None


SM_N, SM_M, SM_CHAINS, SM_PER_CHAIN = 64, 128, 4096, 4
SM_TC_DRAM_BYTES = 6.279e9 + 2.571e9   # ncu, one sm_tc_kernel launch of this workload


def sm_workload(N=SM_N, M=SM_M):
    """The N=64, M=128 complex RBM (sigma 0.05, PCG64(102)) sampled by 4096 chains."""
    rng = np.random.Generator(np.random.PCG64(102))
    b = rng.normal(0, 0.05, M) + 1j * rng.normal(0, 0.05, M)
    W = rng.normal(0, 0.05, (N, M)) + 1j * rng.normal(0, 0.05, (N, M))
    return b, W


def sm_cpu_baseline(b, W, samples, workers):
    """The oracle's FP64 O_k rows of `samples` configurations and the rank-n update with
    numpy's BLAS on the host cores -> samples/s."""
    from oracle import pyoracle as po
    opsi = po.RBM(b, W, 1.0)
    rng = np.random.default_rng(5)
    sp = rng.integers(0, 2 ** 63, (samples, 1), dtype=np.uint64)
    t0 = time.perf_counter()
    O = np.array([po.O_k(opsi, s) for s in sp])
    S = O.T @ O.conj() / samples
    dt = time.perf_counter() - t0
    assert S.shape[0] == O.shape[1]
    return samples / dt


def run_smatrix(args):
    """One step = one get_S_matrix call (the reference's get_S_matrix,
    source/network_functions/S_matrix.cu) over a MonteCarloLoop pass of 16384 samples:
    sampling, tanh rows, the Hermitian rank-16384 update of the 8320 x 8320 block and the
    P x P result copied to the host."""
    import torch
    import ctypes
    import rbmongpu_gb300 as rg
    from rbmongpu_gb300._lib import call
    torch.cuda.set_device(0)
    Ns, Ms = args.sm_n, args.sm_m
    b, W = sm_workload(Ns, Ms)
    psi = rg.Psi(np.zeros(Ns), np.zeros(Ns), b, W, 1.0, False, True)
    n = SM_CHAINS * SM_PER_CHAIN
    mc = rg.MonteCarloLoop(n, 1, 20, SM_CHAINS, True, seed=11)
    L = Ms + Ns * Ms
    simt = bool(args.sm_simt)
    for _ in range(args.warmup):
        rg.get_S_matrix(psi, mc, simt=simt)
    ms_acc, walls = [], []
    ms = ctypes.c_double()
    launches = ctypes.c_int()
    clocks = ClockSampler(0)
    clocks.start()
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        S = rg.get_S_matrix(psi, mc, simt=simt)
        walls.append(time.perf_counter() - t0)
        call("rbmg_s_matrix_timing", ctypes.byref(ms), ctypes.byref(launches))
        ms_acc.append(ms.value)
    clk = clocks.stop()
    assert np.isfinite(S[2 * Ns:, 2 * Ns:]).all()
    wall = float(np.mean(walls))
    acc_s = float(np.mean(ms_acc)) / 1e3
    flops = 8.0 * L * (L + 1) / 2 * n          # 4 FMA per upper-triangle entry and sample
    if simt:
        v = ctypes.c_double()
        call("rbmg_probe_fp32_tflops", 20000, ctypes.byref(v))
        roof = {"bound": "fp32", "achieved": flops / acc_s / 1e12, "peak": v.value, "unit": "TFLOP/s",
                "frac": flops / acc_s / 1e12 / v.value, "traffic": None,
                "peak_source": "measured in this run by the library's FP32 FMA probe kernel",
                "kernel": "sm_herk_kernel"}
    else:
        # six BF16 part products for each of the four real products of a complex one
        tflops = 6.0 * flops / acc_s / 1e12
        peak = measured_peak("bf16_tflops")
        roof = {"bound": "tensor", "achieved": tflops, "peak": peak, "unit": "TFLOP/s",
                "frac": tflops / peak if peak else None, "traffic": None,
                "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst), of measured",
                "kernel": "sm_tc_kernel (+ sm_tc_prep_kernel, in the timed launches)",
                "fp32_equivalent_tflops": flops / acc_s / 1e12,
                "algorithmic": "48 BF16 flops per upper-triangle entry and sample (6 part pairs x 4 real "
                               "products x 2)"}
    if simt:
        roof["flops_per_launch"] = flops / max(1, launches.value)
    else:
        # per launch of sm_tc_kernel (one per 4096-sample chunk; a prep launch precedes each)
        chunks = max(1, launches.value // 2)
        roof["flops_per_launch"] = 6.0 * flops / chunks
        if (Ns, Ms) == (SM_N, SM_M):
            roof["traffic"] = SM_TC_DRAM_BYTES
            roof["traffic_source"] = ("dram__bytes_read.sum + dram__bytes_write.sum of one sm_tc_kernel launch "
                                      "(4096 samples, this workload) from ncu; algorithmic: the FP64 tile "
                                      "read and written once per 1024-sample window (4.5 GB) + the planes")
    P = 2 * Ns + L
    cpu = None
    if args.cpu_seconds > 0:
        cs = 512
        cpu = {"value": sm_cpu_baseline(b, W, cs, os.cpu_count() or 1), "unit": "samples/s",
               "cores": os.cpu_count() or 1, "kind": "port",
               "sample": f"{cs} random configurations: oracle FP64 O_k rows + numpy BLAS rank-{cs} update"}
    line = {
        "metric": "S matrix (get_S_matrix): MC samples folded into the P x P O_k covariance per second",
        "value": n / acc_s, "unit": "samples/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": acc_s * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": ("f32 products (complex64 rows), f64 accumulation" if simt else
                  "bf16 x3 split products of complex64 rows, f32 sums of <= 1024 samples, f64 accumulation"),
        "data": "synthetic (seeded PCG64 parameters)",
        "config": {"workload": f"s_matrix_rbm_n{Ns}_m{Ms}_mc{n}", "N": Ns, "M": Ms, "P": P,
                   "samples": n, "chains": SM_CHAINS, "products": "fp32 cuda cores" if simt else "tensor cores",
                   "l2": f"the {16 * L * L / 1e9:.2f} GB FP64 matrix, read and written every 1024 samples, "
                         "exceeds L2 at N=64"},
        "e2e": {"value": n / wall, "unit": "samples/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 16 * P * P},
        "gpu_launches": int(launches.value) * args.steps,
        "roofline": roof,
        "cpu_baseline": cpu,
        "clocks": clk,
    }
    print(json.dumps(line))


# --------------------------------------------------------------------- deep-net adjoint workload
DEEP_N, DEEP_SIZES, DEEP_WALKERS, DEEP_SEED = 100, (200, 100, 50), 8192, 107


def deep_workload():
    """Dense complex PsiDeep N=100 -> 200 -> 100 -> 50: weights and biases complex
    Normal(0, 0.1 / fan_in) (variance, split over the real and imaginary parts), final
    weights 1, PCG64(107)."""
    rng = np.random.Generator(np.random.PCG64(DEEP_SEED))
    b, conn, W = [], [], []
    fan = DEEP_N
    for m in DEEP_SIZES:
        sd = np.sqrt(0.1 / fan / 2)
        b.append(rng.normal(0, sd, m) + 1j * rng.normal(0, sd, m))
        conn.append(np.array([[c] * m for c in range(fan)]))
        W.append(rng.normal(0, sd, (fan, m)) + 1j * rng.normal(0, sd, (fan, m)))
        fan = m
    return b, conn, W, np.ones(DEEP_SIZES[-1])


def deep_flops():
    """FP32 flops (a complex MAC = 8, the activation ~50 per unit) of: one full forward pass;
    one single-flip proposal of the sampler (layer 0's pre-activations moved by the flipped
    spin's row, the activations and the later layers evaluated); and the adjoint per
    sample: one full forward pass of the sample, then for its N flipped neighbours
    (layer 0 moved like a proposal's) and itself (layer 0 kept) a stored forward pass,
    a reverse pass (2 x the MACs) and the outer products of the parameter gradient
    (1 x)."""
    s0, s1, s2 = DEEP_SIZES
    macs = DEEP_N * s0 + s0 * s1 + s1 * s2
    fwd = 8 * macs + 50 * sum(DEEP_SIZES)
    proposal = 8 * s0 + 8 * (s0 * s1 + s1 * s2) + 50 * sum(DEEP_SIZES)
    adj = fwd + DEEP_N * proposal + (proposal - 8 * s0) + (DEEP_N + 1) * 3 * 8 * macs
    return fwd, proposal, adj


def run_deep(args):
    """One step = the gradient of <H> of the deep net through the adjoint kernels
    (ExpectationValue.eloc_gradient, score=True; the autograd Function's backward) over a
    MonteCarloLoop pass of 8192 walkers (3 thermalisation sweeps, then one sample each)."""
    import torch
    import rbmongpu_gb300 as rg
    from rbmongpu_gb300.autograd import energy
    torch.cuda.set_device(0)
    b, conn, W, fw = deep_workload()
    N = DEEP_N
    psi = rg.PsiDeep(np.zeros(N), np.zeros(N), b, conn, W, fw, 1.0, False, True)
    H = rg.Operator(*rg.operators.tfim_chain(N, 1.0, 1.0))
    therm = 3
    mk = lambda: rg.MonteCarloLoop(DEEP_WALKERS, 1, therm, DEEP_WALKERS, True, seed=21)   # noqa: E731
    ev = rg.ExpectationValue()
    for _ in range(args.warmup):
        ev.eloc_gradient(psi, H, mk(), score=True)
    sp = rg.library_stream()
    stream = torch.cuda.ExternalStream(sp)
    K = args.steps
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    clocks = ClockSampler(0)
    clocks.start()
    for k in range(K):
        torch.cuda.synchronize()
        starts[k].record(stream)
        g, E = ev.eloc_gradient(psi, H, mk(), score=True)
        ends[k].record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = np.array([a.elapsed_time(e) for a, e in zip(starts, ends)])
    assert np.isfinite(E) and np.all(np.isfinite(g))
    sec = float(ms.mean()) / 1e3
    # end to end through the autograd Function: parameters from a host tensor, the
    # gradient back in it
    params = torch.tensor(psi.params, requires_grad=True)
    t0 = time.perf_counter()
    for _ in range(K):
        params.grad = None
        loss = energy(params, psi, H, mk())
        loss.backward()
    e2e_s = (time.perf_counter() - t0) / K
    fwd, proposal, adj = deep_flops()
    # per sweep: layer 0 and log psi from the spins (one full pass), then N proposals
    flops = DEEP_WALKERS * ((therm + 1) * (fwd + N * proposal) + adj)
    v = ctypes_probe_fp32()
    cpu = None
    if args.cpu_seconds > 0:
        from oracle import pyoracle as po
        opsi = po.Deep(N, b, conn, W, fw, 1.0)
        rng = np.random.default_rng(5)
        spins = rng.integers(0, 2 ** 63, (4, 2), dtype=np.uint64)
        spins[:, 1] &= (1 << (N - 64)) - 1
        t0 = time.perf_counter()
        po.samples_gradient(opsi, po.Op(*rg.operators.tfim_chain(N, 1.0, 1.0)), spins)
        dt = time.perf_counter() - t0
        cpu = {"value": len(spins) / dt, "unit": "samples/s", "cores": 1, "kind": "port",
               "sample": "4 configurations: the reference's O_k gradient estimator (E_k term included) in FP64 "
                         "by the CPU restatement, one core"}
    P = psi.num_params
    line = {
        "metric": "deep-net gradient of <H> (adjoint kernels): MC samples per second",
        "value": DEEP_WALKERS / sec, "unit": "samples/s", "n_gpus": 1, "steps": K, "warmup": args.warmup,
        "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (complex64 net), f64 gradient sums", "data": "synthetic (seeded PCG64 parameters)",
        "config": {"workload": "psideep_100_200_100_50_tfim_adjoint", "N": N, "layers": list(DEEP_SIZES),
                   "walkers": DEEP_WALKERS, "therm_sweeps": therm,
                   "step": "MonteCarloLoop pass (3 thermalisation sweeps, 1 sample per walker) + adjoint gradient"},
        "eloc_per_s": DEEP_WALKERS / sec,
        "e2e": {"value": DEEP_WALKERS / e2e_s, "unit": "samples/s", "h2d_bytes_per_step": 16 * P,
                "d2h_bytes_per_step": 16 * P},
        # per gradient call of this workload (its launch list): the sampler, 6 adjoint chunks,
        # 84 outer-product reductions, 84 split sums and the 2 weighted-mean launches
        "gpu_launches": 177 * K,
        "roofline": {"bound": "fp32", "achieved": flops / sec / 1e12, "peak": v, "unit": "TFLOP/s",
                     "frac": flops / sec / 1e12 / v if v else None, "traffic": None,
                     "peak_source": "measured in this run by the library's FP32 FMA probe kernel",
                     "kernel": "deep_mc_multi_kernel + deep_adjoint_multi_kernel + adj_cgemm_kernel (the whole step)",
                     "flops_per_step": flops},
        "cpu_baseline": cpu,
        "clocks": clk,
    }
    print(json.dumps(line))


def ctypes_probe_fp32():
    import ctypes
    from rbmongpu_gb300._lib import call
    v = ctypes.c_double()
    call("rbmg_probe_fp32_tflops", 20000, ctypes.byref(v))
    return v.value


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400, help="timed rows of each chain")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--walkers", type=int, default=WALKERS)
    ap.add_argument("--sweeps-per-row", type=int, default=10)
    ap.add_argument("--learned-steps-per-row", type=int, default=150,
                    help="learned steps per row; 150 makes a learned row last about as long as a plain row")
    ap.add_argument("--learned-streams", type=int, default=0,
                    help="streams of the frozen learned steps (0: automatic, 2 slices from 8192 walkers)")
    ap.add_argument("--train-steps", type=int, default=2000)
    ap.add_argument("--train-walkers", type=int, default=4096)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=16.0, help="budget of the CPU baseline leg")
    ap.add_argument("--sm-n", type=int, default=SM_N, help="s_matrix workload: visible units")
    ap.add_argument("--sm-m", type=int, default=SM_M, help="s_matrix workload: hidden units")
    ap.add_argument("--sm-simt", type=int, default=0, help="s_matrix workload: 1 = FP32 CUDA-core products")
    ap.add_argument("--workload", default="learned", choices=["learned", "serving", "s_matrix", "deep"],
                    help="learned: the N=100 learned-vs-plain chains (headline); serving: 64 uneven RBMs; "
                         "s_matrix: get_S_matrix of the N=64, M=128 RBM over 16384 MC samples; "
                         "deep: the PsiDeep 100-200-100-50 gradient through the adjoint kernels")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    workers = max(1, min(os.cpu_count() or 1, 64))
    import tempfile

    if args.workload == "serving" and args.impl == "ours":
        if rank == 0:
            run_serving(args)
        return
    if args.workload == "s_matrix" and args.impl == "ours":
        if rank == 0:
            run_smatrix(args)
        return
    if args.workload == "deep" and args.impl == "ours":
        if rank == 0:
            run_deep(args)
        return

    if args.impl == "reference":
        # the reference cannot run N=100 (MAX_SPINS=64 in its include/types.h); its CPU
        # algorithm (single-flip Metropolis in FP64) is timed through the restatement
        if rank != 0:
            return
        with tempfile.TemporaryDirectory() as td:
            series, wall, sweeps = cpu_chains(args.warmup + args.steps, 1.0, workers, td)
        series = series[args.warmup * sweeps:]
        tau, _, ok = tau_int(series)
        n = series.size
        timed = wall * args.steps / (args.warmup + args.steps)
        value = n / tau / timed
        line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * timed / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded PCG64 parameters)",
                "config": {"workload": "rbm_n100_m400_tfim_chain", "method": "plain single-flip Metropolis",
                           "walkers": workers, "sweeps_per_step": sweeps},
                "cpu_baseline": {"value": value, "unit": UNIT, "cores": workers, "kind": "port",
                                 "sample": f"{workers} FP64 chains x {args.steps * sweeps} sweeps with E_loc each"},
                "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "eloc_per_s": n / timed, "tau_int_sweeps": tau, "tau_converged": ok}
        print(json.dumps(line))
        return

    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    r = run_gpu(args, rank, world, local_rank)
    if rank != 0:
        if world > 1:
            import torch
            torch.distributed.destroy_process_group()
        return
    S, L, B = args.sweeps_per_row, args.learned_steps_per_row, args.walkers
    ess_l, ess_p, ess_e2e, n_l, n_p = r["tot"]
    sec_l, sec_p, sec_e2e = r["tmax"]
    fl = flops_per_sweep() * S * B
    avg_launch = float(np.mean(r["kernel_ms"])) / 1e3
    achieved = fl / avg_launch / 1e12
    peak = r["fp32_peak"]
    pl, le = r["plain"], r["learned"]
    # CPU baseline on the host cores: the plain method, FP64 restatement, bounded sample
    cpu = None
    if args.cpu_seconds > 0:
        with tempfile.TemporaryDirectory() as td:
            cs, cwall, csweeps = cpu_chains(max(1, int(args.cpu_seconds)), 1.0, workers, td)
        cpu_eloc_s = cs.size / cwall
        tau_sweeps = pl["tau_int_rows"] * S
        cpu = {"value": cpu_eloc_s / tau_sweeps, "unit": UNIT, "cores": workers, "kind": "port",
               "sample": f"{workers} FP64 restatement chains x {cs.shape[0]} sweeps with E_loc each; ESS/s "
                         f"divides their E_loc/s by the GPU plain chain's tau_int in sweeps",
               "eloc_per_s": cpu_eloc_s}
    gap = (le["energy_per_spin"] - pl["energy_per_spin"]) / np.hypot(le["se_per_spin"], pl["se_per_spin"])
    line = {
        "metric": METRIC, "value": ess_l / sec_l, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.mean(r["learned_ms"])),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (complex64 RBM), bf16 MLP with f32 accumulation",
        "data": f"synthetic (seeded PCG64 parameters; random +-1 starts, {THERM_SWEEPS} single-flip sweeps "
                "shared by both chains)",
        "config": {"workload": "rbm_n100_m400_tfim_chain_learned_vs_plain", "N": N_SPINS, "M": M_HIDDEN,
                   "walkers_per_gpu": B, "sigma": SIGMA, "h": FIELD, "therm_sweeps": THERM_SWEEPS,
                   "step": f"learned: {L} frozen MH steps + E_loc; plain: {S} sweeps + E_loc",
                   "train_steps": args.train_steps, "train_walkers": args.train_walkers,
                   "learned_streams": learned_slices(args, B),
                   "l2": "flushed between timed rows"},
        "learned": dict(le, ess_per_s=ess_l / sec_l, acceptance=r["learned_accept"], train_seconds=r["train_s"],
                        ms_per_row=float(np.mean(r["learned_ms"]))),
        "plain": dict(pl, ess_per_s=ess_p / sec_p, acceptance=r["plain_accept"],
                      ms_per_row=float(np.mean(r["plain_ms"]))),
        "learned_over_plain_ess_per_s": (ess_l / sec_l) / (ess_p / sec_p),
        "note": "both chains start from the same equilibrated configurations; where tau_converged is false "
                "the window reached the series length, tau_int is a lower bound and ESS/s an upper bound; "
                "half_drift_in_se compares the series' two halves (stationarity)",
        "energy_gap_in_se": gap,
        "eloc_per_s": n_l / sec_l,
        "e2e": {"value": ess_e2e / sec_e2e, "unit": UNIT, "h2d_bytes_per_step": int(r["h2d"]),
                "d2h_bytes_per_step": int(r["d2h"])},
        # per learned row and walker slice: the first step's draw, then L x (tensor-core
        # network on the proposed states, accept + next draw); per row: the angles from
        # scratch, the current states' network pass and the local-energy pass
        "gpu_launches": args.steps * (learned_slices(args, B) * (2 * L + 1) + 3),
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak if peak else None, "traffic": SAMPLER_DRAM_BYTES,
                     "traffic_source": "ncu dram__bytes_read + write of one launch (W and walker state are "
                                       "read once per launch whatever its sweep count)",
                     "peak_source": "measured in this run by the library's FP32 FMA probe kernel",
                     "kernel": f"rbm_mc_kernel<13,2> (plain sampler, {S} sweeps per launch)",
                     "flops_per_launch": fl, "ms_per_launch": avg_launch * 1e3},
        "cpu_baseline": cpu,
        "clocks": r["clocks"],
    }
    print(json.dumps(line))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
