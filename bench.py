#!/usr/bin/env python
"""Benchmark of the plain Metropolis chain of the N=100 complex RBM.

Workload (the configuration the headline metric is quoted on): complex RBM with
N=100 visible and M=400 hidden units, parameters complex Normal(0, 0.1^2) drawn from
PCG64(104); periodic 1D transverse-field Ising chain with h=1.0 (200 Pauli
strings); 16384 walkers.  One step = one sweep (N single-spin Metropolis proposals
per walker) followed by the local energy of every walker.  The headline metric is
effective samples per second: walkers x steps / tau_int(E_loc) per second, with
tau_int from Sokal's automatic windowing (c = 5) of the walkers' E_loc series;
E_loc/s is reported beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

For N > 1 run under torchrun: every rank samples its own replica of the walker set
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
THERM_SWEEPS = 1000          # several tau_int of the plain chain (~130 sweeps)
METRIC = "effective samples/s (ESS of E_loc), plain single-flip Metropolis, N=100 RBM"
UNIT = "samples/s"
L2_FLUSH_BYTES = 256 << 20

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


def flops_per_walker_step(N=N_SPINS, M=M_HIDDEN, n_offdiag=N_SPINS):
    sweep = N * M * FLOPS_PROPOSAL_ANGLE + 2 * N * M + FLOPS_LC_RE * M     # proposals + angle refresh
    measure = 2 * N * M + FLOPS_LC_C * M + n_offdiag * M * FLOPS_ELOC_ANGLE
    return sweep + measure


def tau_int(series, c=5.0):
    """Integrated autocorrelation time (in steps) of E_loc, Sokal's automatic windowing:
    tau(W) = 1 + 2 sum_{t=1}^{W} rho(t), smallest W with W >= c tau(W); rho averaged over
    walkers, each series centred on the all-walker mean.  series: [K, walkers]."""
    x = np.asarray(series.real, np.float64)
    x = x - x.mean()
    K = x.shape[0]
    f = np.fft.rfft(x, n=2 * K, axis=0)
    ac = np.fft.irfft(f * np.conj(f), n=2 * K, axis=0)[:K].mean(axis=1) / np.arange(K, 0, -1)
    if ac[0] <= 0:
        return 1.0, 1
    rho = ac / ac[0]
    tau, window = 1.0, 1
    for window in range(1, K):
        tau = 1.0 + 2.0 * rho[1:window + 1].sum()
        if window >= c * tau:
            break
    return max(tau, 1.0), window


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


# --------------------------------------------------------------------- GPU arm
def run_gpu(args, rank, world, local_rank):
    import torch
    import rbmongpu_gb300 as rg

    torch.cuda.set_device(local_rank)
    rg.setDevice(local_rank)
    b, W = workload()
    psi = rg.Psi(np.zeros(N_SPINS), np.zeros(N_SPINS), b, W, 1.0, False, True)
    op_t = rg.operators.tfim_chain(N_SPINS, 1.0, FIELD)
    op = rg.Operator(*op_t)
    B = args.walkers
    chain = rg.Chain(psi, B, seed=1000 + rank)
    sp = rg.library_stream()
    stream = torch.cuda.ExternalStream(sp)
    K, Wm = args.steps, args.warmup
    eloc = torch.empty((K, B, 2), dtype=torch.float64, device="cuda")
    scratch = torch.empty((max(Wm, 1), B, 2), dtype=torch.float64, device="cuda")
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    with torch.cuda.stream(stream):
        chain.sweep_async(psi, None, THERM_SWEEPS, 1, 0, sp)
        for w in range(Wm):
            chain.sweep_async(psi, op, 1, 1, scratch[w].data_ptr(), sp)
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(K)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local_rank)
    clocks.start()
    with torch.cuda.stream(stream):
        for k in range(K):
            flush.fill_(k & 0xFF)                 # L2 flush between timed steps (not timed)
            starts[k].record(stream)
            chain.sweep_async(psi, op, 1, 1, eloc[k].data_ptr(), sp)
            ends[k].record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    if world > 1:
        torch.distributed.barrier()
    step_ms = np.array([s.elapsed_time(e) for s, e in zip(starts, ends)])
    total_s = float(step_ms.sum()) / 1e3
    series = eloc.cpu().numpy().view(np.complex128)[..., 0]
    tau, window = tau_int(series)
    _, acc, props = chain.state()

    # end to end through the public API with host buffers: per step the parameters go
    # host -> device (psi.params) and the walkers' local energies device -> host
    e2e_K = max(4, K // 10)
    p_host = psi.params
    host_eloc = np.empty((e2e_K, B), np.complex128)
    pinned = torch.empty((B, 2), dtype=torch.float64, pin_memory=True)
    dbuf = torch.empty((B, 2), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(e2e_K):
        psi.params = p_host
        with torch.cuda.stream(stream):
            chain.sweep_async(psi, op, 1, 1, dbuf.data_ptr(), sp)
            pinned.copy_(dbuf, non_blocking=True)
        stream.synchronize()
        host_eloc[k] = pinned.numpy().view(np.complex128)[:, 0]
    e2e_s = time.perf_counter() - t0
    # the short e2e series cannot resolve tau_int; it shares the device-timed chains' tau
    h2d = (N_SPINS + 1) * ((M_HIDDEN + 31) // 32 * 32) * 8     # complex64 W and b, padded rows
    d2h = B * 16

    fp32_peak = None
    if rank == 0:
        import ctypes
        from rbmongpu_gb300._lib import call
        v = ctypes.c_double()
        call("rbmg_probe_fp32_tflops", 20000, ctypes.byref(v))
        fp32_peak = v.value

    stats = np.array([total_s, B * K / tau, B * K, e2e_s, B * e2e_K / tau], np.float64)
    if world > 1:
        t = torch.tensor(stats, device="cuda")
        mx = t.clone()
        torch.distributed.all_reduce(mx, op=torch.distributed.ReduceOp.MAX)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.SUM)
        stats = t.cpu().numpy()
        stats[0], stats[3] = mx[0].item(), mx[3].item()
    return dict(step_ms=step_ms, total_s=stats[0], ess=stats[1], samples=stats[2], tau=tau, window=window,
                e2e_s=stats[3], e2e_ess=stats[4], h2d=h2d, d2h=d2h, clocks=clk, accept=acc / max(props, 1),
                fp32_peak=fp32_peak, E_mean=complex(series.mean()))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--walkers", type=int, default=WALKERS)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=16.0, help="budget of the CPU baseline leg")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    workers = max(1, min(os.cpu_count() or 1, 64))
    import tempfile

    if args.impl == "reference":
        # the reference cannot run N=100 (MAX_SPINS=64 in its include/types.h); its CPU
        # algorithm is timed through the FP64 restatement on the host cores
        if rank != 0:
            return
        with tempfile.TemporaryDirectory() as td:
            series, wall, sweeps = cpu_chains(args.warmup + args.steps, 1.0, workers, td)
        series = series[args.warmup * sweeps:]
        tau, _ = tau_int(series)
        n = series.size
        timed = wall * args.steps / (args.warmup + args.steps)
        value = n / tau / timed
        line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * timed / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded PCG64 parameters)",
                "config": {"workload": "rbm_n100_m400_tfim_chain_plain_metropolis", "walkers": workers,
                           "sweeps_per_step": sweeps},
                "cpu_baseline": {"value": value, "unit": UNIT, "cores": workers, "kind": "port",
                                 "sample": f"{workers} chains x {args.steps * sweeps} sweeps with E_loc each"},
                "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "eloc_per_s": n / timed, "tau_int_sweeps": tau}
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
    fl = flops_per_walker_step() * args.walkers
    avg_launch = float(np.mean(r["step_ms"])) / 1e3
    achieved = fl / avg_launch / 1e12
    peak = r["fp32_peak"]
    # CPU baseline on the host cores: same chains, FP64 restatement, bounded sample
    cpu = None
    if args.cpu_seconds > 0:
        with tempfile.TemporaryDirectory() as td:
            cs, cwall, csweeps = cpu_chains(max(1, int(args.cpu_seconds)), 1.0, workers, td)
        cpu_eloc_s = cs.size / cwall
        cpu = {"value": cpu_eloc_s / r["tau"], "unit": UNIT, "cores": workers, "kind": "port",
               "sample": f"{workers} FP64 restatement chains x {cs.shape[0]} sweeps with E_loc; "
                         f"ESS/s uses the GPU chains' tau_int", "eloc_per_s": cpu_eloc_s}
    line = {
        "metric": METRIC, "value": r["ess"] / r["total_s"], "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * r["total_s"] / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 (complex64), FP64 sums",
        "data": "synthetic (seeded PCG64 parameters, random +-1 starts)",
        "config": {"workload": "rbm_n100_m400_tfim_chain_plain_metropolis", "N": N_SPINS, "M": M_HIDDEN,
                   "walkers_per_gpu": args.walkers, "sigma": SIGMA, "h": FIELD,
                   "step": "1 sweep (N proposals) + E_loc per walker", "l2": "flushed between timed steps"},
        "eloc_per_s": r["samples"] / r["total_s"],
        "proposals_per_s": r["samples"] * N_SPINS / r["total_s"],
        "tau_int_sweeps": r["tau"], "tau_window": r["window"], "acceptance": r["accept"],
        "mean_energy": r["E_mean"].real,
        "e2e": {"value": r["e2e_ess"] / r["e2e_s"], "unit": UNIT, "h2d_bytes_per_step": int(r["h2d"]),
                "d2h_bytes_per_step": int(r["d2h"])},
        "gpu_launches": 2 * args.steps,     # per step: the sampler and the local-energy pass
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak if peak else None, "traffic": None,
                     "peak_source": "measured in this run by the library's FP32 FMA probe kernel",
                     "kernel": "rbm_mc_kernel<13,2> + rbm_eloc_kernel<13,2> (one step)",
                     "flops_per_launch": fl},
        "cpu_baseline": cpu,
        "clocks": r["clocks"],
    }
    print(json.dumps(line))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
