#!/usr/bin/env python
"""Benchmark: learned-proposal vs plain Metropolis chains of the N=100 complex RBM.

Workload: complex RBM with N=100 visible and M=400 hidden units, parameters complex
Normal(0, sigma^2) drawn from PCG64(104); periodic 1D transverse-field Ising chain with
h=1.0 (200 Pauli strings); 16384 walkers per GPU.  Two chains run on the same GPU from the
same equilibrated configurations:

* plain: single-spin-flip Metropolis (the reference's method); one step = one row =
  `--sweeps-per-row` sweeps of N proposals per walker, then the local energy of every
  walker;
* learned: after `--train-steps` steps of online training (cross-entropy to the locally
  balanced proposal + Adam on the first `--train-walkers` walkers), the frozen proposal
  network's cluster-flip Metropolis-Hastings steps; one row = `--learned-steps-per-row`
  steps, then the local energy of every walker.

Each chain's row length is the one that maximises its own ESS/s (measured on GB300: the
learned chain 323k / 569k / 672k / 685k / 647k / 549k samples/s at 10 / 30 / 60 / 100 /
150 / 250 steps per row, the plain chain 1.44M / 1.68M / 1.54M / 1.13M at 1 / 2 / 4 / 8
sweeps per row): 100 learned steps, 2 sweeps.

The headline is effective samples per second of the learned chain: walkers /
tau_int(E_loc) per second of a timed row, tau_int (in rows) from Sokal's automatic
windowing (c = 5) of the E_loc series formed by the K timed rows and the `--tau-rows`
rows that follow them, so that the measurement does not depend on K.  At sigma = 0.1
the RBM's |psi|^2 is a spin glass: neither chain equilibrates within 2e5 sweeps (the
E_loc autocorrelation decays logarithmically), so tau_int has no finite estimate there.
The headline therefore runs the same network at sigma = 0.05 (`--mix-sigma`), where both
chains mix and tau_int converges, and reports the sigma = 0.1 rows beside it
("glass_sigma0.1", tau_int lower bounds, energy drift by quarter of the series).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--workload serving|s_matrix|deep]

`--workload serving` times the batched serving of 64 uneven RBMs instead (one line of
its own); `--workload s_matrix` times get_S_matrix of the N=64, M=128 RBM over 16384
Monte Carlo samples (P = 8448); `--workload deep` the PsiDeep 100-200-100-50 gradient.

For N > 1 run under torchrun: every rank samples its own replica of the walker sets
(Philox keys offset by rank), no data-path collective; value = the sum over ranks of
walkers / tau_int over the maximum over ranks of the seconds per row.
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
# capture of rbm_mc_smem_kernel<13,2> on these 16384 walkers
SAMPLER_DRAM_BYTES = 1.059e6
# DRAM bytes of one learned_accept_kernel<13,2> launch of 16384 walkers (ncu, sigma 0.05, mean
# of three launches: 100.3 MB read, 4.1 MB written -- accepted angles stay in L2 within a launch)
ACCEPT_DRAM_BYTES = 104.4e6
# rows of the sigma 0.1 measurement: 10 sweeps, or 150 learned steps (about as long)
GLASS_SWEEPS_PER_ROW, GLASS_STEPS_PER_ROW = 10, 150

# algorithmic FP32 flops of the sampler, from the operation list of
# rbmongpu_gb300/csrc/device_math.cuh and rbm_impl.cuh (FMA = 2, mul/add/div = 1)
FLOPS_LC_RE = 37          # Re f(theta), Metropolis test
FLOPS_LC_C = 44           # complex f(theta), measurement
FLOPS_PROPOSAL_ANGLE = FLOPS_LC_RE + 4 + 2     # theta update (2 FMA) + difference and sum
FLOPS_ELOC_ANGLE = FLOPS_LC_C + 4 + 4          # theta'' update + complex difference and sum


def workload(sigma=SIGMA):
    """The N=100, M=400 complex RBM: b and W complex Normal(0, sigma^2) from PCG64(104)."""
    rng = np.random.Generator(np.random.PCG64(PARAM_SEED))
    b = rng.normal(0, sigma, M_HIDDEN) + 1j * rng.normal(0, sigma, M_HIDDEN)
    W = rng.normal(0, sigma, (N_SPINS, M_HIDDEN)) + 1j * rng.normal(0, sigma, (N_SPINS, M_HIDDEN))
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
    x = np.asarray(series.real)
    mean = float(x.mean(dtype=np.float64))
    K, B = x.shape
    ac = np.zeros(K)
    for j in range(0, B, 1024):           # walkers in blocks (bounded memory)
        y = x[:, j:j + 1024].astype(np.float64) - mean
        f = np.fft.rfft(y, n=2 * K, axis=0)
        ac += np.fft.irfft(f * np.conj(f), n=2 * K, axis=0)[:K].sum(axis=1)
    ac /= B * np.arange(K, 0, -1)
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
    chain, sweeps, state_path, sigma = args
    from oracle import pyoracle as po
    b, W = workload(sigma)
    psi = po.RBM(b, W)
    from rbmongpu_gb300.operators import tfim_chain
    op = po.Op(*tfim_chain(N_SPINS, 1.0, FIELD))
    if os.path.exists(state_path):
        st = np.load(state_path)
        state = (st["spins"].copy(), st["rng"].copy(), [1])
    else:
        state = (np.zeros((1, po.nwords(N_SPINS)), np.uint64), np.zeros(1, np.uint64), [0])
    therm = 0 if state[2][0] else 50
    t0 = time.perf_counter()
    _, _, el, _, _ = po.mc_run(psi, op, 1, sweeps, 1, therm, rng=po.OR_RNG_PHILOX, seed=7000, prec=po.OR_PREC_REF64,
                               chain_begin=chain, total_chains=4096, state=state)
    dt = time.perf_counter() - t0
    np.savez(state_path, spins=state[0], rng=state[1])
    return dt, el[:, 0]


def cpu_chains(steps, seconds_per_step, workers, tmpdir, sigma):
    """Runs `workers` persistent CPU chains for `steps` steps of about seconds_per_step."""
    ctx = mp.get_context("spawn")
    with ctx.Pool(workers) as pool:
        dt, _ = pool.map(_cpu_worker, [(w, 1, os.path.join(tmpdir, f"calib{w}.npz"), sigma)
                                       for w in range(workers)])[0]
        sweeps = max(1, int(seconds_per_step / max(dt, 1e-3)))
        series, wall = [], 0.0
        for k in range(steps):
            t0 = time.perf_counter()
            out = pool.map(_cpu_worker, [(w, sweeps, os.path.join(tmpdir, f"s{w}.npz"), sigma)
                                         for w in range(workers)])
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
class GpuChains:
    """The plain and learned chains of one RBM on this GPU, with the row runners the
    benchmark times.  A plain row is `sweeps` single-flip sweeps, a learned row `steps`
    frozen learned Metropolis-Hastings steps; both end with the local energy of every
    walker, written to an E_loc row on the device."""

    def __init__(self, rg, torch, psi, op, B, seeds, chunk_rows=250):
        self.rg, self.torch, self.psi, self.op, self.B = rg, torch, psi, op, B
        self.sp = rg.library_stream()
        self.stream = torch.cuda.ExternalStream(self.sp)
        self.seed_plain, self.seed_learned, self.seed_net = seeds
        self.plain = rg.Chain(psi, B, seed=self.seed_plain)
        self.learned = None
        self.prop = None
        self.chunk = chunk_rows
        self.eloc = torch.empty((chunk_rows, B, 2), dtype=torch.float64, device="cuda")
        self.scratch = torch.empty((B, 2), dtype=torch.float64, device="cuda")
        self.flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
        self.train_s = 0.0

    def equilibrate(self, sweeps):
        with self.torch.cuda.stream(self.stream):
            self.plain.sweep_async(self.psi, None, sweeps, 1, 0, self.sp)
        self.torch.cuda.synchronize()

    def start_learned(self, args, train_steps):
        """The learned chain starts from the plain chain's configurations (its own Philox
        streams); its network is trained online from there, then frozen."""
        rg = self.rg
        objective = rg.Proposal.REINFORCE if args.objective == "reinforce" else rg.Proposal.LOCALLY_BALANCED
        self.prop = rg.Proposal(self.psi.N, seed=self.seed_net, lr=1e-3, objective=objective)
        self.learned = rg.Chain(self.psi, self.B, seed=self.seed_learned)
        self.learned.set_learned_streams(args.learned_streams)
        zero = np.zeros(self.B, np.uint64)
        self.learned.restore(dict(spins=self.plain.checkpoint()["spins"], rng_index=zero, accepts=zero,
                                  proposals=zero))
        self.torch.cuda.synchronize()
        t0 = time.perf_counter()
        with self.torch.cuda.stream(self.stream):
            self.learned.learned_async(self.psi, None, self.prop, train_steps, args.train_walkers, 1, 0, self.sp)
        self.torch.cuda.synchronize()
        self.train_s = time.perf_counter() - t0

    def row_fn(self, kind, per_row):
        if kind == "plain":
            return lambda ptr: self.plain.sweep_async(self.psi, self.op, per_row, per_row, ptr, self.sp)
        return lambda ptr: self.learned.learned_async(self.psi, self.op, self.prop, per_row, 0, per_row, ptr, self.sp)

    def warm(self, kind, per_row, n):
        row = self.row_fn(kind, per_row)
        with self.torch.cuda.stream(self.stream):
            for _ in range(n):
                row(self.scratch.data_ptr())
        self.torch.cuda.synchronize()

    def timed_rows(self, kind, per_row, n, sync):
        """n rows, each timed by CUDA events on the library stream with L2 flushed in
        between (outside the events); returns (ms per row [n], E_loc real parts [n, B])."""
        torch = self.torch
        row = self.row_fn(kind, per_row)
        ms, series = [], []
        for c0 in range(0, n, self.chunk):
            m = min(self.chunk, n - c0)
            starts = [torch.cuda.Event(enable_timing=True) for _ in range(m)]
            ends = [torch.cuda.Event(enable_timing=True) for _ in range(m)]
            sync()
            with torch.cuda.stream(self.stream):
                for k in range(m):
                    self.flush.fill_(k & 0xFF)
                    starts[k].record(self.stream)
                    row(self.eloc[k].data_ptr())
                    ends[k].record(self.stream)
            sync()
            ms += [a.elapsed_time(e) for a, e in zip(starts, ends)]
            series.append(self.eloc[:m, :, 0].float().cpu().numpy())
        return np.array(ms), np.concatenate(series, axis=0)

    def more_rows(self, kind, per_row, n):
        """n further rows, untimed (the series that fixes tau_int)."""
        row = self.row_fn(kind, per_row)
        out = []
        for c0 in range(0, n, self.chunk):
            m = min(self.chunk, n - c0)
            with self.torch.cuda.stream(self.stream):
                for k in range(m):
                    row(self.eloc[k].data_ptr())
            self.torch.cuda.synchronize()
            out.append(self.eloc[:m, :, 0].float().cpu().numpy())
        return np.concatenate(out, axis=0) if out else np.zeros((0, self.B), np.float32)

    def acceptance(self, chain):
        _, a, p = chain.state()
        return a, p


def acf_lags(series, lags):
    """Walker-averaged normalised autocorrelation of E_loc at the given lags (rows)."""
    x = np.asarray(series, np.float64)
    x = x - x.mean()
    v = (x * x).mean()
    return {int(t): float((x[t:] * x[:len(x) - t]).mean() / v) for t in lags if t < len(x)}


def chain_stats(series, timed_ms, B, N=N_SPINS, train_s=0.0):
    """ESS figures of one chain: tau_int (rows) from the whole series (timed rows and the
    rows that follow them), the rate from the timed rows alone."""
    x = np.asarray(series, np.float64)
    tau, window, ok = tau_int(x)
    row_s = float(np.mean(timed_ms)) / 1e3
    sigma = x.std()
    ess_per_s = B / tau / row_s
    se = sigma * np.sqrt(tau / x.size)
    h = len(x) // 2
    m1, m2 = x[:h].mean(axis=0), x[h:].mean(axis=0)
    drift = (m2.mean() - m1.mean()) / np.sqrt((m1.var(ddof=1) + m2.var(ddof=1)) / B)
    # rows to a standard error of 1e-4 per spin: sigma^2 tau / (B rows) = (1e-4 N)^2
    rows_needed = (sigma / (1e-4 * N)) ** 2 * tau / B
    return {"tau_int_rows": tau, "tau_window": window, "tau_converged": ok, "series_rows": len(x),
            "series_over_tau": len(x) / tau, "timed_rows": len(timed_ms), "ms_per_row": row_s * 1e3,
            "ess_per_s": ess_per_s, "eloc_per_s": B / row_s, "energy_per_spin": x.mean() / N,
            "sigma_eloc": sigma, "se_per_spin": se / N, "half_drift_in_se": float(drift),
            "seconds_to_se_1e-4_per_spin": rows_needed * row_s + train_s,
            "acf": acf_lags(x, (1, 2, 5, 10, 20, 50, 100, 200, 400))}


def run_gpu(args, rank, world, local_rank):
    """The learned-vs-plain comparison on this rank (see the module docstring)."""
    import torch
    import rbmongpu_gb300 as rg

    torch.cuda.set_device(local_rank)
    rg.setDevice(local_rank)
    B, K, Wm = args.walkers, args.steps, args.warmup
    op = rg.Operator(*rg.operators.tfim_chain(N_SPINS, 1.0, FIELD))

    def sync():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    clocks = ClockSampler(local_rank)
    out = {}
    # ---------------------------------------------------------------- headline: sigma 0.05
    b, W = workload(args.mix_sigma)
    psi = rg.Psi(np.zeros(N_SPINS), np.zeros(N_SPINS), b, W, 1.0, False, True)
    g = GpuChains(rg, torch, psi, op, B, replica_seeds(rank))
    S, L = args.sweeps_per_row, args.learned_steps_per_row
    g.equilibrate(args.therm_sweeps)
    g.start_learned(args, args.train_steps)
    g.warm("plain", S, Wm)
    g.warm("learned", L, Wm)
    clocks.start()
    a0 = g.acceptance(g.plain)
    plain_ms, plain_timed = g.timed_rows("plain", S, K, sync)
    a1 = g.acceptance(g.plain)
    l0 = g.acceptance(g.learned)
    learned_ms, learned_timed = g.timed_rows("learned", L, K, sync)
    l1 = g.acceptance(g.learned)
    # the sampler kernel alone (one launch of 10 sweeps, no local energies), its roofline
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
    with torch.cuda.stream(g.stream):
        for k in range(5):
            g.flush.fill_(k)
            starts[k].record(g.stream)
            g.plain.sweep_async(psi, None, 10, 1, 0, g.sp)
            ends[k].record(g.stream)
    torch.cuda.synchronize()
    kernel_ms = np.array([a.elapsed_time(e) for a, e in zip(starts, ends)])
    # per-kernel durations of a learned step (network pass, accept pass), one stream
    ms_net, ms_acc = g.learned.learned_kernel_times(psi, g.prop, 20)
    clk = clocks.stop()
    # the series that fixes tau_int: the timed rows and the rows after them
    plain_series = np.concatenate([plain_timed, g.more_rows("plain", S, args.tau_rows)])
    learned_series = np.concatenate([learned_timed, g.more_rows("learned", L, args.tau_rows)])
    out["plain"] = dict(chain_stats(plain_series, plain_ms, B), acceptance=(a1[0] - a0[0]) / max(a1[1] - a0[1], 1))
    out["learned"] = dict(chain_stats(learned_series, learned_ms, B, train_s=g.train_s),
                          acceptance=(l1[0] - l0[0]) / max(l1[1] - l0[1], 1), train_seconds=g.train_s)
    out.update(plain_ms=plain_ms, learned_ms=learned_ms, kernel_ms=kernel_ms, ms_net=ms_net, ms_acc=ms_acc,
               clocks=clk, learned_accept=out["learned"]["acceptance"])

    # end to end through the public API with host buffers: per row the RBM parameters go
    # host -> device (psi.params) and the row's local energies device -> host (pinned)
    e2e_K = max(4, K // 4)
    p_host = psi.params
    pinned = torch.empty((B, 2), dtype=torch.float64, pin_memory=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(e2e_K):
        psi.params = p_host
        with torch.cuda.stream(g.stream):
            g.learned.learned_async(psi, op, g.prop, L, 0, L, g.scratch.data_ptr(), g.sp)
            pinned.copy_(g.scratch, non_blocking=True)
        g.stream.synchronize()
        _ = pinned.numpy().view(np.complex128)[:, 0].mean()
    out["e2e_s"] = (time.perf_counter() - t0) / e2e_K
    out["h2d"] = (N_SPINS + 1) * ((M_HIDDEN + 31) // 32 * 32) * 8     # complex64 W and b, padded rows
    out["d2h"] = B * 16
    del g

    # ---------------------------------------------------------------- the glassy target (sigma 0.1)
    if args.glass_rows > 0:
        b, W = workload(SIGMA)
        psi = rg.Psi(np.zeros(N_SPINS), np.zeros(N_SPINS), b, W, 1.0, False, True)
        g = GpuChains(rg, torch, psi, op, B, replica_seeds(rank))
        g.equilibrate(THERM_SWEEPS)
        g.start_learned(args, args.train_steps)
        gl = {}
        for kind, per in (("plain", GLASS_SWEEPS_PER_ROW), ("learned", GLASS_STEPS_PER_ROW)):
            ms, x0 = g.timed_rows(kind, per, min(K, args.glass_rows), sync)
            x = np.concatenate([x0, g.more_rows(kind, per, args.glass_rows - len(x0))])
            st = chain_stats(x, ms, B)
            rm = x.mean(axis=1) / N_SPINS
            q = max(1, len(rm) // 4)
            st["energy_per_spin_by_quarter"] = [float(rm[i * q:(i + 1) * q].mean()) for i in range(4)]
            st["walker_mean_spread_per_spin"] = float(x.mean(axis=0).std() / N_SPINS)
            gl[kind] = st
        out["glass"] = gl
        del g

    fp32_peak = None
    if rank == 0:
        fp32_peak = max(ctypes_probe_fp32(), ctypes_probe_fp32(pairs=True))
    out["fp32_peak"] = fp32_peak
    # whole-job sums over ranks (walker sets are independent replicas); times are maxima
    pl, le = out["plain"], out["learned"]
    tot = np.array([B / le["tau_int_rows"], B / pl["tau_int_rows"], learned_series.size, plain_series.size],
                   np.float64)
    tmax = np.array([le["ms_per_row"] / 1e3, pl["ms_per_row"] / 1e3, out["e2e_s"]], np.float64)
    if world > 1:
        tot, tmax = combine_ranks(tot, tmax, "cuda")
    out.update(tot=tot, tmax=tmax)
    return out


# --------------------------------------------------------------------- long-chain autocorrelation
def run_autocorrelation(args):
    """Both chains of the N=100, M=400 RBM at weight scale --ac-sigma for --ac-rows rows
    (plain: 10 sweeps, learned: 150 steps per row) after the shared equilibration: the
    walker-averaged E_loc autocorrelation at lags up to 8000 rows, the mean energy by
    twentieth of the series (drift) and the spread of the walkers' time averages -- the
    evidence of whether tau_int can be measured at that weight scale."""
    import torch
    import rbmongpu_gb300 as rg
    torch.cuda.set_device(0)
    b, W = workload(args.ac_sigma)
    psi = rg.Psi(np.zeros(N_SPINS), np.zeros(N_SPINS), b, W, 1.0, False, True)
    op = rg.Operator(*rg.operators.tfim_chain(N_SPINS, 1.0, FIELD))
    B, R = args.walkers, args.ac_rows
    g = GpuChains(rg, torch, psi, op, B, replica_seeds(0), chunk_rows=200)
    g.equilibrate(THERM_SWEEPS)
    g.start_learned(args, args.train_steps)
    out = {"workload": f"rbm_n100_m400_tfim_chain_sigma{args.ac_sigma:g}", "walkers": B, "rows": R,
           "therm_sweeps": THERM_SWEEPS, "row": "plain 10 sweeps / learned 150 frozen steps, + E_loc"}
    lags = [t for t in (1, 2, 5, 10, 20, 50, 100, 200, 500, 1000, 2000, 4000, 8000) if t < R]
    for kind, per in (("plain", 10), ("learned", 150)):
        t0 = time.perf_counter()
        x = g.more_rows(kind, per, R)
        sec = time.perf_counter() - t0
        tau, window, ok = tau_int(x)
        rm = x.mean(axis=1, dtype=np.float64) / N_SPINS
        q = max(1, R // 20)
        wm = x.mean(axis=0, dtype=np.float64) / N_SPINS
        out[kind] = {"seconds": sec, "tau_int_rows": tau, "tau_window": window, "tau_converged": ok,
                     "acf": acf_lags(x, lags), "energy_per_spin_by_twentieth":
                     [round(float(rm[i * q:(i + 1) * q].mean()), 5) for i in range(20)],
                     "walker_mean_per_spin_percentiles": [round(float(v), 4) for v in
                                                          np.percentile(wm, [1, 10, 50, 90, 99])]}
    print(json.dumps(out))


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
    # algorithmic flops per walker: the sweep, E_loc, and the reference estimator's E_k term
    # at its minimum -- tanh(theta'') of every off-diagonal string from the denominator its
    # f(theta'') already formed (44 flops), U_j += e_n tanh (8), and per (row, unit) of the
    # sums V = e_n tanh (6) and the three centred accumulations (16); the tiles' recomputation
    # of tanh(theta'') (stored nowhere, to keep O(N^2 M) bytes per walker off HBM) is not counted
    flops = 0
    for psi, _, w, _ in inst:
        N, M = psi.N, psi.M
        flops += w * (flops_per_sweep(N, M) + flops_per_eloc(N, M, N) + N * M * (44 + 8) + (N + 1) * M * (6 + 16))
    peak = max(ctypes_probe_fp32(), ctypes_probe_fp32(pairs=True))
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
                     "peak_source": "measured in this run: the larger of the library's scalar and packed-pair FP32 FMA probes",
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
        peak = max(ctypes_probe_fp32(), ctypes_probe_fp32(pairs=True))
        roof = {"bound": "fp32", "achieved": flops / acc_s / 1e12, "peak": peak, "unit": "TFLOP/s",
                "frac": flops / acc_s / 1e12 / peak, "traffic": None,
                "peak_source": "measured in this run: the larger of the library's scalar and packed-pair FP32 FMA probes",
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
    v = max(ctypes_probe_fp32(), ctypes_probe_fp32(pairs=True))
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
                     "peak_source": "measured in this run: the larger of the library's scalar and packed-pair FP32 FMA probes",
                     "kernel": "deep_mc_multi_kernel + deep_adjoint_multi_kernel + adj_cgemm_kernel (the whole step)",
                     "flops_per_step": flops},
        "cpu_baseline": cpu,
        "clocks": clk,
    }
    print(json.dumps(line))


def run_plain(args):
    """One step = one 10-sweep launch of the plain single-flip sampler on the N=100, M=400
    RBM (sigma --mix-sigma), all walkers, the L2 flushed before each launch: the sampler
    kernel alone, for its roofline and for profiling (no other kernel of the library runs)."""
    import torch
    import rbmongpu_gb300 as rg
    torch.cuda.set_device(0)
    b, W = workload(args.mix_sigma)
    N = N_SPINS
    psi = rg.Psi(np.zeros(N), np.zeros(N), b, W, 1.0, False, True)
    sp = rg.library_stream()
    stream = torch.cuda.ExternalStream(sp)
    B = args.walkers
    ch = rg.Chain(psi, B, seed=1000)
    ch.sweep_async(psi, None, 200, 1, 0, sp)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    sweeps = 10
    for k in range(args.warmup):
        ch.sweep_async(psi, None, sweeps, 1, 0, sp)
    torch.cuda.synchronize()
    K = args.steps
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    clocks = ClockSampler(0)
    clocks.start()
    with torch.cuda.stream(stream):
        for k in range(K):
            flush.fill_(k & 255)
            starts[k].record(stream)
            ch.sweep_async(psi, None, sweeps, 1, 0, sp)
            ends[k].record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = np.array([a.elapsed_time(e) for a, e in zip(starts, ends)])
    sec = float(ms.mean()) / 1e3
    _, acc, props = ch.state()
    flops = flops_per_sweep() * sweeps * B
    peak = max(ctypes_probe_fp32(), ctypes_probe_fp32(pairs=True))
    line = {
        "metric": "plain single-flip sampler: walker-sweeps/s at N=100, M=400",
        "value": B * sweeps / sec, "unit": "walker-sweeps/s", "n_gpus": 1, "steps": K, "warmup": args.warmup,
        "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (complex64)", "data": "synthetic (seeded PCG64 parameters)",
        "config": {"workload": "rbm_n100_m400_plain_sampler_sigma%g" % args.mix_sigma, "N": N, "M": M_HIDDEN,
                   "walkers": B, "sweeps_per_step": sweeps, "l2": "flushed before each launch"},
        "acceptance": float(acc) / float(props) if props else None,
        "gpu_launches": K,
        "roofline": {"bound": "fp32", "achieved": flops / sec / 1e12, "peak": peak, "unit": "TFLOP/s",
                     "frac": flops / sec / 1e12 / peak, "traffic": SAMPLER_DRAM_BYTES,
                     "peak_source": "measured in this run: the larger of the library's scalar and packed-pair FP32 "
                                    "FMA probes",
                     "kernel": "rbm_mc_smem_kernel<13,2>", "flops_per_launch": flops},
        "clocks": clk,
    }
    print(json.dumps(line))


MCG_CHAINS, MCG_SWEEPS, MCG_THERM = 4096, 1000, 200


def run_mc_gradient(args):
    """One step = ExpectationValue.gradient over a MonteCarloLoop pass of the plain
    Metropolis configuration: 4096 walkers of the N=64, M=128 complex RBM (sigma 0.05,
    PCG64(102)) on the periodic 8x8 transverse-field Ising model (J = 1, h = 3), random
    +-1 starts, 200 thermalisation sweeps, then 1000 sweeps of 64 single-flip proposals
    with E_loc and O_k of every walker after every sweep: <E> and the reference gradient
    <E O_k*> + conj<E_k> - 2 <E><O_k*> over 4 096 000 samples (the call a user makes; its
    results come back to the host)."""
    import torch
    import rbmongpu_gb300 as rg
    torch.cuda.set_device(0)
    b, W = sm_workload()
    N, M = SM_N, SM_M
    psi = rg.Psi(np.zeros(N), np.zeros(N), b, W, 1.0, False, True)
    op_t = rg.operators.tfim_square(8, 1.0, 3.0)
    op = rg.Operator(*op_t)
    ev = rg.ExpectationValue()
    mk = lambda k: rg.MonteCarloLoop(MCG_CHAINS * MCG_SWEEPS, 1, MCG_THERM, MCG_CHAINS, seed=2024 + k)   # noqa: E731
    for k in range(args.warmup):
        ev.gradient(psi, op, mk(k))
    sp = rg.library_stream()
    stream = torch.cuda.ExternalStream(sp)
    K = args.steps
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    walls = []
    clocks = ClockSampler(0)
    clocks.start()
    for k in range(K):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        starts[k].record(stream)
        g, E = ev.gradient(psi, op, mk(100 + k))
        ends[k].record(stream)
        walls.append(time.perf_counter() - t0)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = np.array([a.elapsed_time(e) for a, e in zip(starts, ends)])
    assert np.isfinite(E) and np.all(np.isfinite(g))
    samples = MCG_CHAINS * MCG_SWEEPS
    sec = float(ms.mean()) / 1e3
    e2e_s = float(np.mean(walls))
    n_off = N   # one X string per site
    per_sample = (flops_per_sweep(N, M) + flops_per_eloc(N, M, n_off) + n_off * M * (44 + 8) + (N + 1) * M * (6 + 16))
    flops = MCG_CHAINS * (MCG_THERM + MCG_SWEEPS) * flops_per_sweep(N, M) + samples * (per_sample - flops_per_sweep(N, M))
    peak = max(ctypes_probe_fp32(), ctypes_probe_fp32(pairs=True))
    cpu = None
    if args.cpu_seconds > 0:
        # the reference's arithmetic (FP64) of the same method: 4 chains, 5 thermalisation
        # sweeps, then sweeps with E_loc, and the gradient estimator on their samples
        from oracle import pyoracle as po
        opsi, oop = po.RBM(b, W, 1.0), po.Op(*op_t)
        n_s = 48
        t0 = time.perf_counter()
        ospins, _, _, _, _ = po.mc_run(opsi, oop, 4, n_s, 1, 5, seed=5, prec=po.OR_PREC_REF64, want_eloc=True)
        po.samples_gradient(opsi, oop, ospins.reshape(-1, ospins.shape[-1]))
        dt = time.perf_counter() - t0
        cpu = {"value": 4 * n_s / dt, "unit": "samples/s", "cores": 1, "kind": "port",
               "sample": "4 chains x (5 thermalisation + 48 measured sweeps) with E_loc, then the O_k gradient "
                         "estimator (E_k term included) on their 192 samples, FP64 restatement, one core"}
    P = psi.num_params
    line = {
        "metric": "plain MCMC with E_loc and the O_k gradient every sweep: samples/s (N=64, M=128, 8x8 TFIM)",
        "value": samples / sec, "unit": "samples/s", "n_gpus": 1, "steps": K, "warmup": args.warmup,
        "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (complex64), f64 sums", "data": "synthetic (seeded PCG64 parameters)",
        "config": {"workload": "rbm_n64_m128_tfim8x8_h3_mc_gradient", "N": N, "M": M, "walkers": MCG_CHAINS,
                   "therm_sweeps": MCG_THERM, "measured_sweeps": MCG_SWEEPS,
                   "step": "MonteCarloLoop pass + E_loc + O_k gradient sums of every sample (one gradient call)",
                   "l2": "inputs larger than L2 are not involved: the pass reads W (64 KB) and writes sums"},
        "eloc_per_s": samples / sec,
        "e2e": {"value": samples / e2e_s, "unit": "samples/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 16 * P + 16},
        "roofline": {"bound": "fp32", "achieved": flops / sec / 1e12, "peak": peak, "unit": "TFLOP/s",
                     "frac": flops / sec / 1e12 / peak, "traffic": None,
                     "peak_source": "measured in this run: the larger of the library's scalar and packed-pair FP32 "
                                    "FMA probes",
                     "kernel": "the whole call (sampler sweeps, local energies, estimator sums)",
                     "flops_per_step": flops},
        "cpu_baseline": cpu,
        "clocks": clk,
    }
    print(json.dumps(line))


def ctypes_probe_fp32(pairs=False):
    """FP32 FMA rate of this GPU from the library's probe kernel (scalar or packed pairs)."""
    import ctypes
    from rbmongpu_gb300._lib import call
    v = ctypes.c_double()
    call("rbmg_probe_fp32x2_tflops" if pairs else "rbmg_probe_fp32_tflops", 20000, ctypes.byref(v))
    return v.value


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400, help="timed rows of each chain")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--walkers", type=int, default=WALKERS)
    ap.add_argument("--sweeps-per-row", type=int, default=2)
    ap.add_argument("--learned-steps-per-row", type=int, default=100,
                    help="learned steps per row (100: the learned chain's largest ESS/s)")
    ap.add_argument("--tau-rows", type=int, default=3000,
                    help="rows of each chain after the timed ones: the series tau_int is taken from")
    ap.add_argument("--therm-sweeps", type=int, default=2000, help="shared equilibration sweeps (headline)")
    ap.add_argument("--mix-sigma", type=float, default=0.05,
                    help="weight scale of the headline's RBM (both chains mix at 0.05; not at 0.07 or 0.1)")
    ap.add_argument("--glass-rows", type=int, default=300,
                    help="rows of each chain on the sigma 0.1 RBM (0: skip that part)")
    ap.add_argument("--learned-streams", type=int, default=0,
                    help="streams of the frozen learned steps (0: automatic, 2 slices from 8192 walkers)")
    ap.add_argument("--train-steps", type=int, default=2000)
    ap.add_argument("--train-walkers", type=int, default=4096)
    ap.add_argument("--objective", default="balanced", choices=["balanced", "reinforce"],
                    help="training objective of the proposal: cross-entropy to the locally balanced proposal, or "
                         "REINFORCE on the acceptance (the accept-rate objective)")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=16.0, help="budget of the CPU baseline leg")
    ap.add_argument("--sm-n", type=int, default=SM_N, help="s_matrix workload: visible units")
    ap.add_argument("--sm-m", type=int, default=SM_M, help="s_matrix workload: hidden units")
    ap.add_argument("--sm-simt", type=int, default=0, help="s_matrix workload: 1 = FP32 CUDA-core products")
    ap.add_argument("--ac-sigma", type=float, default=SIGMA, help="autocorrelation workload: weight scale")
    ap.add_argument("--ac-rows", type=int, default=20000, help="autocorrelation workload: rows of each chain")
    ap.add_argument("--workload", default="learned",
                    choices=["learned", "serving", "s_matrix", "deep", "autocorrelation", "plain", "mc_gradient"],
                    help="learned: the N=100 learned-vs-plain chains (headline); serving: 64 uneven RBMs; "
                         "s_matrix: get_S_matrix of the N=64, M=128 RBM over 16384 MC samples; "
                         "deep: the PsiDeep 100-200-100-50 gradient through the adjoint kernels; "
                         "plain: 10-sweep launches of the plain sampler alone (its roofline, profiling); "
                         "mc_gradient: the N=64, M=128 8x8-TFIM gradient over 4096 walkers x 1000 sweeps")
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
    if args.workload == "plain" and args.impl == "ours":
        if rank == 0:
            run_plain(args)
        return
    if args.workload == "mc_gradient" and args.impl == "ours":
        if rank == 0:
            run_mc_gradient(args)
        return
    if args.workload == "autocorrelation":
        if rank == 0 and args.impl == "ours":
            run_autocorrelation(args)
        return

    if args.impl == "reference":
        # the reference cannot run N=100 (MAX_SPINS=64 in its include/types.h); its CPU
        # algorithm (single-flip Metropolis in FP64) is timed through the restatement
        if rank != 0:
            return
        with tempfile.TemporaryDirectory() as td:
            series, wall, sweeps = cpu_chains(args.warmup + args.steps, 1.0, workers, td, args.mix_sigma)
        series = series[args.warmup * sweeps:]
        tau, window, ok = tau_int(series)
        n = series.size
        timed = wall * args.steps / (args.warmup + args.steps)
        value = n / tau / timed
        line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * timed / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded PCG64 parameters)",
                "config": {"workload": f"rbm_n100_m400_tfim_chain_sigma{args.mix_sigma:g}",
                           "method": "plain single-flip Metropolis", "walkers": workers, "sweeps_per_step": sweeps},
                "cpu_baseline": {"value": value, "unit": UNIT, "cores": workers, "kind": "port",
                                 "sample": f"{workers} FP64 chains x {args.steps * sweeps} sweeps with E_loc each"},
                "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "eloc_per_s": n / timed, "tau_int_sweeps": tau, "tau_window": window, "tau_converged": ok,
                "series_over_tau": series.shape[0] / tau}
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
    inv_tau_l, inv_tau_p, n_l, n_p = r["tot"]
    sec_l, sec_p, sec_e2e = r["tmax"]
    ess_l, ess_p = inv_tau_l / sec_l, inv_tau_p / sec_p
    pl, le = r["plain"], r["learned"]
    # the dominant kernel of a learned row: the accept pass (HBM), one launch of all walkers
    KP = ((M_HIDDEN + 31) // 32 + 1) // 2
    O = N_SPINS + 8
    state_b = KP * 32 * (16 + 8)             # angles (paired float4) and Re f (paired float2)
    acc = le["acceptance"]
    accept_bytes = B * (state_b + 4 * O + 52 + 40 + acc * (state_b + 4 * O + 16))
    hbm = measured_peak("hbm_gbs")
    accept_gbs = accept_bytes / (r["ms_acc"] / 1e3) / 1e9
    mlp_flops = B * 2.0 * (N_SPINS * 256 + 256 * 256 + 256 * O)
    bf16 = measured_peak("bf16_tflops")
    mlp_tfs = mlp_flops / (r["ms_net"] / 1e3) / 1e12
    fl = flops_per_sweep() * 10 * B
    avg_launch = float(np.mean(r["kernel_ms"])) / 1e3
    peak = r["fp32_peak"]
    # CPU baseline on the host cores: the plain method, FP64 restatement, bounded sample
    cpu = None
    if args.cpu_seconds > 0:
        with tempfile.TemporaryDirectory() as td:
            cs, cwall, csweeps = cpu_chains(max(3, int(args.cpu_seconds)), 1.0, workers, td, args.mix_sigma)
        n_cpu = cs.shape[0]
        cs = cs[2 * csweeps:]
        cwall = cwall * cs.shape[0] / n_cpu
        ctau, _, cok = tau_int(cs)
        cpu = {"value": cs.size / ctau / cwall, "unit": UNIT, "cores": workers, "kind": "port",
               "sample": f"{workers} FP64 restatement chains (sigma {args.mix_sigma:g}) x {cs.shape[0]} sweeps with "
                         f"E_loc each; ESS/s from their own tau_int", "tau_int_sweeps": ctau, "tau_converged": cok,
               "eloc_per_s": cs.size / cwall}
    gap = (le["energy_per_spin"] - pl["energy_per_spin"]) / np.hypot(le["se_per_spin"], pl["se_per_spin"])
    line = {
        "metric": METRIC, "value": ess_l, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.mean(r["learned_ms"])),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (complex64 RBM), bf16 MLP with f32 accumulation",
        "data": f"synthetic (seeded PCG64 parameters; random +-1 starts, {args.therm_sweeps} single-flip sweeps "
                "shared by both chains)",
        "config": {"workload": f"rbm_n100_m400_tfim_chain_sigma{args.mix_sigma:g}_learned_vs_plain", "N": N_SPINS,
                   "M": M_HIDDEN, "walkers_per_gpu": B, "sigma": args.mix_sigma, "h": FIELD,
                   "therm_sweeps": args.therm_sweeps,
                   "step": f"one row: learned {L} frozen MH steps + E_loc; plain {S} sweeps + E_loc",
                   "tau_series_rows": args.steps + args.tau_rows, "train_steps": args.train_steps,
                   "train_walkers": args.train_walkers, "objective": args.objective,
                   "learned_streams": learned_slices(args, B),
                   "l2": "flushed between timed rows"},
        "learned": le,
        "plain": pl,
        "learned_over_plain_ess_per_s": ess_l / ess_p,
        "energy_gap_in_se": gap,
        "note": ("ESS/s = walkers / tau_int(E_loc, rows) / seconds per timed row; tau_int by Sokal's windowing "
                 "(c = 5) of the timed rows and the tau_rows that follow them; seconds_to_se_1e-4_per_spin = "
                 "rows needed at that tau x seconds per row (+ the online training for the learned chain). "
                 "The headline runs the configuration's network at sigma 0.05, where both chains mix; "
                 "glass_sigma0.1 holds the same measurement at sigma 0.1, where neither chain equilibrates "
                 "within the run (tau_int lower bounds)"),
        "eloc_per_s": B * world / sec_l,
        "e2e": {"value": inv_tau_l / sec_e2e, "unit": UNIT, "h2d_bytes_per_step": int(r["h2d"]),
                "d2h_bytes_per_step": int(r["d2h"])},
        # per learned row and walker slice: the first step's draw, then L x (tensor-core
        # network on the proposed states, accept + next draw); per row: the angles from
        # scratch, the current states' network pass and the local-energy pass
        "gpu_launches": args.steps * (learned_slices(args, B) * (2 * L + 1) + 3),
        "roofline": {"bound": "hbm", "achieved": accept_gbs, "peak": hbm, "unit": "GB/s",
                     "frac": accept_gbs / hbm if hbm else None, "traffic": ACCEPT_DRAM_BYTES,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one learned_accept_kernel "
                                       "launch of 16384 walkers",
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs, of measured",
                     "kernel": "learned_accept_kernel<13,2> (accept + next draw; one launch of all walkers, one stream)",
                     "bytes_per_launch": accept_bytes, "ms_per_launch": r["ms_acc"],
                     "algorithmic": "per walker: angles and Re f read (24 B per hidden unit pair slot), the proposed "
                                    "logits row, move and stream words; the same written back on accept"},
        "network_roofline": {"bound": "tensor", "achieved": mlp_tfs, "peak": bf16, "unit": "TFLOP/s",
                             "frac": mlp_tfs / bf16 if bf16 else None,
                             "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst), of measured",
                             "kernel": "mlp_tc_kernel (tcgen05, the proposed states' logits)",
                             "flops_per_launch": mlp_flops, "ms_per_launch": r["ms_net"]},
        "plain_sampler_roofline": {"bound": "fp32", "achieved": fl / avg_launch / 1e12, "peak": peak,
                                   "unit": "TFLOP/s", "frac": fl / avg_launch / 1e12 / peak if peak else None,
                                   "traffic": SAMPLER_DRAM_BYTES,
                                   "peak_source": "measured in this run: the larger of the library's scalar and "
                                                  "packed-pair FP32 FMA probes",
                                   "kernel": "rbm_mc_smem_kernel<13,2> (plain sampler, 10 sweeps per launch, sigma 0.05)",
                                   "flops_per_launch": fl, "ms_per_launch": avg_launch * 1e3},
        "glass_sigma0.1": r.get("glass"),
        "cpu_baseline": cpu,
        "clocks": r["clocks"],
    }
    print(json.dumps(line))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
