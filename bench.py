"""Throughput benchmark of the GB300 link engine (one JSON line on stdout).

Workload: 4x4 MIMO spatial multiplexing, 1024-point FFT with 600 used
subcarriers, CP 72, 14 words, 64-QAM, 30.72 MHz sampling, 23-tap Rayleigh
channel (delays k*50 ns, power -0.4k dB, 20 sinusoids, Doppler 500 Hz),
ideal CSI with per-subcarrier 4x4 LMMSE detection, SNR uniform in [0, 30] dB
per drop, 4096 drops per step, complex64 samples. Synthetic data: every bit,
channel draw and noise sample comes from the engine's Philox streams.

One step = one batch of 4096 whole drops: realize -> transmit -> propagate +
AWGN -> demodulate -> ideal CSI + LMMSE + demap + bit-error count. ``value``
is simulated bits/s with the per-drop noise powers already in HBM; ``e2e`` is
the same through the public ``LinkEngine.simulate`` call with host buffers
(noise powers copied in, error counts copied out, inside the timed region).

``--impl reference`` times the CPU restatement of the reference's drop (float64
numpy, one process per host core) on a bounded sample of the same workload.
"""

from __future__ import annotations

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

FS = 30.72e6
N, U, CP, WORDS, ORDER = 1024, 600, 72, 14, 64
NTX = NRX = 4
DROPS = 4096
BITS_PER_DROP = WORDS * U * 6 * NTX  # 201 600
METRIC = "simulated bits/sec on 1 GB300, learned vs LMMSE estimator at equal BER; NMSE dB"
CONFIG = {
    "workload": "4x4 MIMO OFDM 1024/600 CP72 14 sym 64-QAM, 23-tap Rayleigh (k*50ns, -0.4k dB, 500 Hz), "
                "ideal CSI + per-subcarrier 4x4 LMMSE, SNR U[0,30] dB",
    "drops_per_step": DROPS,
    "bits_per_drop": BITS_PER_DROP,
    "samples": "complex64",
    "l2": "working set per step ~5.3 GB (tx/rx samples, grids) > 129 MB L2; no flush needed",
}


def oracle_drop(args):
    """One float64 oracle drop (runs in a worker process)."""

    seed, drop, level = args
    from oracle.link import LinkConfig, simulate_drop
    from tests.configs import mimo_channel, mimo_frame

    cfg = LinkConfig(mimo_frame(ORDER), mimo_channel(FS), FS, NTX, NRX, "ideal", "lmmse", "snr")
    return simulate_drop(cfg, seed, drop, level)["errors"]


def cpu_pool():
    import multiprocessing as mp

    for v in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[v] = "1"
    cores = os.cpu_count() or 1
    return mp.get_context("spawn").Pool(cores), cores


def time_cpu(pool, cores, rounds: int, seed: int = 11) -> tuple[float, int, float]:
    """Run `rounds` rounds of `cores` parallel oracle drops; returns (bits/s, drops, seconds)."""

    rng = np.random.default_rng(seed)
    drops = rounds * cores
    work = [(seed, 1_000_000 + i, float(rng.uniform(0, 30))) for i in range(drops)]
    pool.map(oracle_drop, work[:cores])  # warm the workers (imports)
    t0 = time.perf_counter()
    pool.map(oracle_drop, work, chunksize=1)
    dt = time.perf_counter() - t0
    return drops * BITS_PER_DROP / dt, drops, dt


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    pool, cores = cpu_pool()
    for _ in range(args.warmup):
        time_cpu(pool, cores, 1)
    vals, drops, secs = [], 0, 0.0
    for k in range(args.steps):
        v, d, s = time_cpu(pool, cores, 1, seed=100 + k)
        vals.append(v)
        drops += d
        secs += s
    pool.close()
    value = drops * BITS_PER_DROP / secs
    line = {
        "impl": "reference",
        "metric": METRIC, "value": value, "unit": "bits/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (Philox draws)",
        "config": dict(CONFIG, drops_per_step=cores),
        "cpu_baseline": {"value": value, "unit": "bits/s", "cores": cores, "kind": "port",
                         "sample": f"{drops} drops of the workload (float64 numpy restatement of the reference's "
                                   f"drop, one process per core)"},
        "e2e": {"value": value, "unit": "bits/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


class Clocks:
    """nvidia-smi clock / throttle sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int) -> None:
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in getattr(self, "lines", []):
            f = [x.strip() for x in line.split(",")]
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def stage_bytes(T: int, D: int, stride: int) -> dict:
    """Algorithmic HBM bytes per drop of each stage."""

    C = U
    return {
        "fading_realize": stride,
        "ofdm_modulate_bits": 8 * NTX * T,
        "fading_propagate": 8 * (NTX * T + NRX * (T + D)),
        "ofdm_demodulate": 8 * NRX * WORDS * (N + C),
        "detect_ideal_lmmse": 8 * NRX * WORDS * C + 4,
    }


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--drops", type=int, default=DROPS)
    ap.add_argument("--cpu-rounds", type=int, default=4, help="rounds of per-core oracle drops for cpu_baseline")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
        return

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    # the CPU pool starts before the first GPU call (spawned workers never touch CUDA)
    pool, cores = cpu_pool() if rank == 0 else (None, 0)

    import torch

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import hermespy_gb300 as hg
    from hermespy_gb300 import _lib
    from hermespy_gb300.build import build
    from tests.configs import mimo_channel

    build()
    drops = args.drops
    cfg = mimo_channel(FS)
    wf = hg.OFDMWaveform([hg.GridResource(1, prefix_ratio=CP / N, elements=[hg.GridElement(hg.ElementType.DATA, U)])],
                         [hg.SymbolSection(WORDS, [0])], num_subcarriers=N, modulation_order=ORDER)
    seed = 20261203
    ch = hg.MultipathFadingChannel(cfg.delays, cfg.power_profile, cfg.rice_factors, num_sinusoids=20,
                                   doppler_frequency=500.0, seed=seed)
    eng = hg.LinkEngine(wf, ch, NTX, NRX, FS, "ideal", "lmmse", "snr", max_drops=drops, seed=seed)
    fh, fd = eng._fading.handle, wf._frame()
    T, D = wf.samples_per_frame(), eng._fading.max_delay
    stride = eng._fading.state_bytes
    dev = torch.device("cuda", local)
    rng = np.random.default_rng(seed + rank)
    snr_db = rng.uniform(0.0, 30.0, size=drops)
    p_host = eng.noise_power(snr_db).astype(np.float32)
    p_dev = torch.from_numpy(p_host).to(dev)
    state = eng._fading.new_state(drops)
    x = torch.empty((drops, NTX, T), dtype=torch.complex64, device=dev)
    y = torch.empty((drops, NRX, T + D), dtype=torch.complex64, device=dev)
    grid = torch.empty((drops, NRX, WORDS, U), dtype=torch.complex64, device=dev)
    errors = torch.empty(drops, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream
    stages = list(stage_bytes(T, D, stride))

    def step(drop0: int, ev=None):
        calls = [
            ("hpx_fading_realize", fh, seed, drop0, drops, _lib.ptr(state), sp),
            ("hpx_ofdm_modulate_bits", fd, seed, drop0, drops, NTX, _lib.ptr(x), sp),
            ("hpx_fading_propagate", fh, _lib.ptr(state), drops, _lib.ptr(x), T, _lib.ptr(y), _lib.ptr(p_dev), seed,
             drop0, sp),
            ("hpx_ofdm_demodulate", fd, _lib.ptr(y), T + D, drops * NRX, U, _lib.ptr(grid), sp),
            ("hpx_detect_ideal", fh, _lib.ptr(state), fd, _lib.EQ_LMMSE, _lib.ptr(grid), U, _lib.ptr(p_dev), seed,
             drop0, drops, _lib.ptr(errors), sp),
        ]
        for i, c in enumerate(calls):
            if ev is not None:
                ev[i].record(stream)
            _lib.call(*c)
        if ev is not None:
            ev[len(calls)].record(stream)

    drop_base = rank * (1 << 40)
    for w in range(args.warmup):
        step(drop_base + w * drops)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    events = [[torch.cuda.Event(enable_timing=True) for _ in range(len(stages) + 1)] for _ in range(args.steps)]
    with Clocks(local) as clk:
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        t0.record(stream)
        for k in range(args.steps):
            step(drop_base + (args.warmup + k) * drops, events[k])
        t1.record(stream)
        torch.cuda.synchronize()
    total_ms = t0.elapsed_time(t1)
    stage_ms = {s: 0.0 for s in stages}
    for ev in events:
        for i, s in enumerate(stages):
            stage_ms[s] += ev[i].elapsed_time(ev[i + 1])
    # per-drop bit errors of the last step, for a BER sanity value
    ber = float(errors.sum().item()) / (drops * BITS_PER_DROP)

    # end to end: public API, host noise powers in (pinned), host error counts out
    p_pin = torch.from_numpy(p_host).pin_memory()
    out_pin = torch.empty(drops, dtype=torch.int32).pin_memory()

    def e2e_step(drop0: int):
        pd = p_pin.to(dev, non_blocking=True)
        e = eng.run(drop0, pd)
        out_pin.copy_(e, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        return out_pin

    for w in range(2):
        e2e_step(drop_base + (1 << 30) + w * drops)
    e2e_steps = max(3, args.steps // 2)
    torch.cuda.synchronize()
    s0 = time.perf_counter()
    for k in range(e2e_steps):
        e2e_step(drop_base + (1 << 31) + k * drops)
    e2e_s = (time.perf_counter() - s0) / e2e_steps

    if world > 1:
        import torch.distributed as dist

        tt = torch.tensor([total_ms, e2e_s], dtype=torch.float64, device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        total_ms, e2e_s = float(tt[0]), float(tt[1])
    ms_per_step = total_ms / args.steps
    value = world * drops * BITS_PER_DROP / (ms_per_step / 1e3)
    e2e_value = world * drops * BITS_PER_DROP / e2e_s

    if rank == 0:
        import json as _json

        peaks = {"hbm_gbs": 6800.0, "src": "fallback"}
        pp = os.path.join(ROOT, "MEASURED_PEAKS.json")
        if os.path.exists(pp):
            with open(pp) as f:
                m = _json.load(f)
            peaks = {"hbm_gbs": float(m["hbm_gbs"]), "src": "measured"}
        bpd = stage_bytes(T, D, stride)
        stage_info = {}
        for s in stages:
            avg_ms = stage_ms[s] / args.steps
            gbs = bpd[s] * drops / (avg_ms / 1e3) / 1e9 if avg_ms > 0 else 0.0
            stage_info[s] = {"ms": round(avg_ms, 4), "share": round(stage_ms[s] / max(sum(stage_ms.values()), 1e-9), 4),
                             "algorithmic_bytes": bpd[s] * drops, "achieved_gbs": round(gbs, 1),
                             "frac_hbm": round(gbs / peaks["hbm_gbs"], 4)}
        dom = max(stages, key=lambda s: stage_ms[s])
        traffic = None
        tp = os.path.join(ROOT, "profiles", "traffic.json")
        if os.path.exists(tp):
            with open(tp) as f:
                traffic = _json.load(f).get(dom)
        roof = {"kernel": dom, "bound": "hbm", "achieved": stage_info[dom]["achieved_gbs"], "peak": peaks["hbm_gbs"],
                "unit": "GB/s", "frac": stage_info[dom]["frac_hbm"], "traffic": traffic,
                "peak_source": peaks["src"]}
        cpu_value, cpu_drops, cpu_s = time_cpu(pool, cores, args.cpu_rounds)
        pool.close()
        line = {
            "metric": METRIC, "value": value, "unit": "bits/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c64", "data": "synthetic (Philox draws)",
            "config": dict(CONFIG, drops_per_step=drops, parallelism=f"drop-sharded x{world}"),
            "drops_per_s": world * drops / (ms_per_step / 1e3), "ber": ber,
            "e2e": {"value": e2e_value, "unit": "bits/s", "h2d_bytes_per_step": 4 * drops,
                    "d2h_bytes_per_step": 4 * drops},
            "gpu_launches": len(stages) * args.steps,
            "roofline": roof, "stages": stage_info,
            "cpu_baseline": {"value": cpu_value, "unit": "bits/s", "cores": cores, "kind": "port",
                             "sample": f"{cpu_drops} drops of the workload in {cpu_s:.1f} s (float64 numpy "
                                       f"restatement of the reference's drop, one process per core)"},
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
