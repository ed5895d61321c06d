#!/usr/bin/env python
"""Benchmark: SSFM sample-steps/s on the 5-channel WDM precision-study link.

Workload (one bench step = one forward propagation of the whole batch):
  5 x 32 GBaud 16QAM channels on a 50 GHz grid, 2^15 symbols per channel,
  RRC roll-off 0.1, 16 samples/symbol of the total band -> N = 2^19 complex
  samples per realization; 20 x 80 km SSMF (alpha 0.2 dB/km, D 17 ps/nm/km,
  gamma 1.3 /W/km), ADAPTIVE split step (max nonlinear phase 0.005 rad/step,
  max step 1 km), EDFA after every span (gain = span loss, NF 5 dB, seeded
  ASE).  Batch = 7 launch powers (-2..+4 dBm per channel) x 18 ASE seeds = 126
  realizations (528 MB of complex64, 4.1x the 129 MB L2).
  One sample-step = one complex sample advanced by one split step.

Arms:
  default            hand-written sm_103a kernels through libfocss_gpu (C ABI)
  --impl reference   the reference algorithm on the host cores: the FP64 C
                     restatement of src/focss/solver/ssfm.cpp and amplifier.cpp
                     (oracle port), a bounded sample of the same workload per
                     step (ADAPTIVE steps with ASE over the first 2 km of a
                     span, one realization per host thread).

Prints one JSON line on rank 0.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "SSFM Gsample-steps/s (FP32 GPU; FP64 reference on host cores)"
UNIT = "Gsample-steps/s"
W = dict(
    workload="wdm5_16qam_32GBd_n2^19_20x80km_ssmf_adaptive_ase",
    channels=5, symbols_per_channel=2 ** 15, samples_per_symbol=16, spacing_hz=50e9, baud=32e9,
    roll_off=0.1, spans=20, span_m=80e3, alpha_db_per_km=0.2, dispersion_ps_nm_km=17.0, gamma_per_w_km=1.3,
    max_phase_shift=0.005, max_step_m=1000.0, noise_figure_db=5.0,
    powers_dbm=[-2, -1, 0, 1, 2, 3, 4], ase_seeds=18,
)
N = W["symbols_per_channel"] * W["samples_per_symbol"]
DT = 1.0 / (W["baud"] * W["samples_per_symbol"])
F0 = 299792458.0 / 1.55e-6


def fiber_params():
    alpha = W["alpha_db_per_km"] * 1e-3 * np.log(10) / 10
    beta2 = -(1.55e-6 ** 2) * (W["dispersion_ps_nm_km"] * 1e-6) / (2 * np.pi * 299792458.0)
    gamma = W["gamma_per_w_km"] * 1e-3
    return alpha, beta2, gamma


def gray16():
    s = np.sqrt(10.0)
    re = np.array([-3, -1, 3, 1, -3, -1, 3, 1, -3, -1, 3, 1, -3, -1, 3, 1]) / s
    im = np.array([-3, -3, -3, -3, -1, -1, -1, -1, 3, 3, 3, 3, 1, 1, 1, 1]) / s
    return re + 1j * im


def rrc_taps(n_symbols, osf, beta):
    """Full-length RRC pulse normalized to sum|h|^2 = length (src/focss/processing/modulation.cpp:47-74)."""
    t = np.arange(n_symbols * osf) / osf - n_symbols / 2.0
    h = np.empty_like(t)
    z = t == 0
    q = np.abs(np.abs(t) - 1 / (4 * beta)) < 1e-12
    o = ~(z | q)
    h[z] = 1 - beta + 4 * beta / np.pi
    h[q] = beta / np.sqrt(2) * ((1 + 2 / np.pi) * np.sin(np.pi / (4 * beta)) + (1 - 2 / np.pi) * np.cos(np.pi / (4 * beta)))
    to = t[o]
    h[o] = (np.sin(np.pi * to * (1 - beta)) + 4 * beta * to * np.cos(np.pi * to * (1 + beta))) / (
        np.pi * to * (1 - 16 * beta ** 2 * to ** 2))
    return h * (h.size / np.sum(h ** 2))


def synth_wdm(seed=1):
    """Seeded synthetic 5-channel WDM field at 1 W per channel (scaled per power later)."""
    osf, ns = W["samples_per_symbol"], W["symbols_per_channel"]
    H = np.fft.fft(np.fft.ifftshift(rrc_taps(ns, osf, W["roll_off"]))) / N
    t = np.arange(N) * DT
    x = np.zeros(N, complex)
    g = gray16()
    for ch in range(W["channels"]):
        rng = np.random.default_rng(seed + ch)
        up = np.zeros(N, complex)
        up[::osf] = g[rng.integers(0, 16, ns)]
        # rrc_shaping (modulation.cpp:86-90): IFFT(FFT(x)/N * FFT(h)/N) unnormalized, times osf
        sig = np.fft.ifft(np.fft.fft(up) * H) * osf
        x += sig * np.exp(2j * np.pi * (ch - W["channels"] // 2) * W["spacing_hz"] * t)
    return x


def batch_inputs():
    base = synth_wdm()
    out = np.empty((len(W["powers_dbm"]) * W["ase_seeds"], 1, N), np.complex64)
    i = 0
    for p in W["powers_dbm"]:
        s = np.sqrt(1e-3 * 10 ** (p / 10.0))
        for _ in range(W["ase_seeds"]):
            out[i, 0] = base * s
            i += 1
    return out


# ---------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.strip()]
        os.unlink(self.path)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                for k, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(k)
            except (ValueError, IndexError):
                continue
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------- CPU reference / baseline
def bench_config(world):
    """The workload's `config`, identical in both arms."""
    B = len(W["powers_dbm"]) * W["ase_seeds"]
    return dict(W, batch=B, samples=N,
                l2="batch of %d MB complex64, %.1fx the 129 MB L2 (inputs larger than L2 between steps)"
                   % (B * N * 8 >> 20, B * N * 8 / 129e6),
                parallelism="replicas" if world > 1 else "single GPU")


def cpu_sample(threads, segment_m):
    """The workload's algorithm on the host cores, with the FP64 oracle port of
    src/focss/solver/ssfm.cpp and src/focss/module/amplifier.cpp: 4 x
    `threads` realizations of the N = 2^19 WDM field (launch powers cycling
    over the workload's -2..+4 dBm/ch, highest first so the threads finish
    together), each an ADAPTIVE split-step run (0.005 rad, 1 km) over the
    first `segment_m` metres of a span, then the EDFA with ASE (NF 5 dB, the
    GPU's Philox stream).  Returns (sample-steps/s / 1e9, seconds, split steps
    taken)."""
    from oracle import build as obuild
    from oracle import cpu
    obuild.build_oracle()
    alpha, beta2, gamma = fiber_params()
    base = synth_wdm()
    powers = sorted(W["powers_dbm"], reverse=True)
    R = 4 * threads
    a = np.empty((R, 1, N), np.complex128)
    for i in range(R):
        a[i, 0] = base * np.sqrt(1e-3 * 10 ** (powers[(i * len(powers)) // R] / 10.0))
    fib = cpu.Fiber(alpha, beta2, gamma, segment_m, 1.55e-6, 1.0)
    G = 10 ** (W["alpha_db_per_km"] * W["span_m"] / 1e3 / 10)
    NF = 10 ** (W["noise_figure_db"] / 10)
    t0 = time.perf_counter()
    out, steps = cpu.ssfm_batch(a, DT, fib, cpu.ADAPTIVE, 1, W["max_phase_shift"], W["max_step_m"], threads=threads)
    for i in range(R):
        out[i] = cpu.amplify(out[i], DT, F0, G, NF, seed=7, counter=0, realization=i)
    dt = time.perf_counter() - t0
    k = int(np.sum(steps))
    return k * N / dt / 1e9, dt, k


# Metres of the first span per realization in a CPU sample: ~5 s of FP64
# work on 16 host cores per reference-arm step, ~10 s for the baseline.
CPU_REFERENCE_SEGMENT_M = 1000.0
CPU_BASELINE_SEGMENT_M = 2500.0


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_sample(threads, CPU_REFERENCE_SEGMENT_M)
    vals, times, ks = [], [], []
    for _ in range(args.steps):
        v, t, k = cpu_sample(threads, CPU_REFERENCE_SEGMENT_M)
        vals.append(v)
        times.append(t)
        ks.append(k)
    value = float(np.median(vals))
    sample = ("%d realizations (launch powers -2..+4 dBm/ch) x the first %.0f m of a span: ADAPTIVE split "
              "steps (%d in total per sample) and the EDFA with ASE, FP64 oracle port of ssfm.cpp/amplifier.cpp, "
              "%d threads" % (4 * threads, CPU_REFERENCE_SEGMENT_M, int(np.median(ks)), threads))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * float(np.median(times)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(args.gpus),
        "reference_code": "oracle port: the reference's own sources build only where the reference tree exists "
                          "(FFTW/Armadillo stand-ins in oracle/), not on the GPU host",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------- GPU arm
def replica_seed(rank: int, seed: int) -> int:
    """ASE seed of one propagation on `rank`: every replica draws independent
    noise, so N GPUs run N independent batches of realizations (weak scaling,
    no data exchanged between ranks)."""
    return seed + 100003 * rank


def reduce_over_ranks(dist, device, elapsed, work):
    """(max elapsed over ranks, summed work): the whole-job aggregate of the
    replicas, whose throughput is the total work over the slowest rank's
    time.  Single process (dist None): the local values."""
    if dist is None:
        return float(elapsed), float(work)
    import torch
    mx = torch.tensor([float(elapsed)], dtype=torch.float64, device=device)
    tt = torch.tensor([float(work)], dtype=torch.float64, device=device)
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    dist.all_reduce(tt, op=dist.ReduceOp.SUM)
    return float(mx[0]), float(tt[0])


def run_ours(args):
    import focss_gb300 as fg
    if not os.path.exists(fg.LIB_PATH):
        from focss_gb300 import build as gbuild
        gbuild.build()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    import torch

    ctx = fg.Context(local)
    alpha, beta2, gamma = fiber_params()
    fib = fg.Fiber(alpha, beta2, gamma, W["span_m"])
    G = 10 ** (W["alpha_db_per_km"] * W["span_m"] / 1e3 / 10)
    NF = 10 ** (W["noise_figure_db"] / 10)
    ssfm = fg.SSFM(fib)
    ssfm.set_grid(fg.SSFM.ADAPTIVE)
    ssfm.set_maximum_phase_shift(W["max_phase_shift"])
    ssfm.set_maximum_step_size(W["max_step_m"])

    host = batch_inputs()
    B = host.shape[0]
    split = fg.autotune(N, B, ctx=ctx)[0]
    dom = fg.Domain(1, N, DT, F0)
    pristine = fg.Field(dom, data=host, batch=B, ctx=ctx)
    field = fg.Field(dom, batch=B, ctx=ctx)
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))

    def propagate(f, seed):
        # forward_propagation (systems.cpp:39-56): the 20 spans (ADAPTIVE SSFM,
        # then EDFA with ASE) as one graph-captured span loop (focss_span_loop)
        if args.host_loop:
            steps = 0
            amp = fg.Amplifier(G, NF, seed=seed)
            for s in range(W["spans"]):
                steps += int(ssfm.run(f, fg.SSFM.FORWARD).sum())
                amp.amplify(f, counter=s)
            return steps
        st = fg.span_loop([f], fib, ssfm, W["spans"], after=fg.Amplifier.AMPLIFY,
                          amplifier=fg.Amplifier(G, NF, seed=seed))
        return int(st[0].sum())

    def barrier():
        if dist is not None:
            dist.barrier()

    for w in range(args.warmup):
        field.assign(pristine)
        propagate(field, replica_seed(rank, 1000 + w))
    ctx.sync()

    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    torch.cuda.synchronize(local)
    ctx.sync()
    launches0 = fg.launch_count()
    total_ms, total_steps = 0.0, 0
    for k in range(args.steps):
        field.assign(pristine)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        total_steps += propagate(field, replica_seed(rank, 2000 + k))
        e1.record(stream)
        e1.synchronize()
        total_ms += e0.elapsed_time(e1)
    ctx.sync()
    torch.cuda.synchronize(local)
    barrier()
    launches = fg.launch_count() - launches0  # field restores are copies, not kernels
    clk = clocks.stop()
    sample_steps = total_steps * N

    t_max, total_samples = reduce_over_ranks(dist, "cuda", total_ms, sample_steps)
    value = total_samples / (t_max / 1e3) / 1e9

    # ---- roofline probe: the split-step passes alone on the full batch
    # (UNIFORM grid: every pass processes all B realizations).
    probe = fg.SSFM(fib, 40)
    field.assign(pristine)
    probe.run(field)
    ctx.profile_read(reset=True)
    ctx.profile_enable(True)
    field.assign(pristine)
    probe.run(field)
    prof = ctx.profile_read(reset=True)
    ctx.profile_enable(False)
    K = 40
    bytes_per_pass = 16.0 * B * N  # one read + one write of complex64 per sample
    col_bytes = bytes_per_pass * prof["col_launches"]           # FWD, K x KERR, INV: all full
    row_bytes = bytes_per_pass * (prof["row_launches"] - 1)     # trailing pass is a no-op
    col_gbs = col_bytes / (prof["col_ms"] / 1e3) / 1e9
    row_gbs = row_bytes / (prof["row_ms"] / 1e3) / 1e9
    dom_kernel = "col_kernel" if prof["col_ms"] >= prof["row_ms"] else "row_kernel"
    achieved = col_gbs if dom_kernel == "col_kernel" else row_gbs
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        peak, peak_src = float(peaks["hbm_gbs"]), "measured"
    except Exception:
        peak, peak_src = 6800.0, "fallback"
    roofline = {
        "bound": "hbm", "kernel": dom_kernel, "achieved": achieved, "peak": peak, "unit": "GB/s",
        "frac": achieved / peak, "peak_source": peak_src, "traffic": None,
        "algorithmic_bytes_per_launch": bytes_per_pass,
        "per_kernel_gbs": {"col_kernel": col_gbs, "row_kernel": row_gbs},
        "per_kernel_avg_ms": {"col_kernel": prof["col_ms"] / max(1, prof["col_launches"]),
                              "row_kernel": prof["row_ms"] / max(1, prof["row_launches"] - 1)},
        "probe": "UNIFORM %d steps over the full batch, CUDA events around each pass" % K,
    }
    # DRAM bytes per launch of the dominant kernel, from the committed ncu
    # capture (scaled to this batch there).
    traffic_file = os.path.join(ROOT, "profiles", "ssfm_traffic_wdm5_n2e19.txt")
    if os.path.exists(traffic_file):
        for ln in open(traffic_file):
            f = ln.split()
            if len(f) == 2 and f[0] == dom_kernel:
                roofline["traffic"] = int(int(f[1]) * B / 40)
                roofline["traffic_source"] = ("profiles/ssfm_traffic_wdm5_n2e19.txt (ncu, 40 realizations, "
                                              "scaled x %d/40)" % B)

    # ---- end to end through the public API with host buffers (pinned)
    pin_in = torch.from_numpy(host.view(np.float32)).pin_memory()
    pin_out = torch.empty_like(pin_in).pin_memory()
    hin = pin_in.numpy().view(np.complex64)
    hout = pin_out.numpy().view(np.complex64)
    import ctypes as C
    from focss_gb300._lib import check, lib
    e2e_steps, t_e2e = 0, 0.0
    for k in range(max(1, args.steps)):
        ctx.sync()
        t0 = time.perf_counter()
        check(lib().focss_field_upload_c64(field.h, hin.ctypes.data_as(C.c_void_p), hin.size), ctx.h)
        e2e_steps += propagate(field, replica_seed(rank, 3000 + k))
        check(lib().focss_field_download_c64(field.h, hout.ctypes.data_as(C.c_void_p), hout.size), ctx.h)
        t_e2e += time.perf_counter() - t0
    t_e2e_max, e2e_total = reduce_over_ranks(dist, "cuda", t_e2e, e2e_steps * N)
    e2e_val = e2e_total / t_e2e_max / 1e9

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max / max(1, args.steps), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": bench_config(world),
        "fft_split": "%d x %d (autotuned)" % (1 << split, N >> split),
        "sample_steps_per_step": sample_steps / max(1, args.steps),
        "roofline": roofline,
        "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": int(hin.nbytes),
                "d2h_bytes_per_step": int(hout.nbytes)},
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    if not args.no_precision:
        line["precision"] = precision_section(fg, ctx)
    if not args.no_sweep:
        line["sweep"] = sweep_section(fg, ctx, stream)
    if not args.no_ppe:
        line["ppe"] = ppe_section(fg, ctx, stream)
    if not args.no_wdm_ppe:
        line["wdm_ppe"] = wdm_ppe_section(fg, ctx, stream)
    if args.dbp_sweep:
        line["dbp_sweep"] = dbp_sweep_section(fg, ctx)
    if args.single_channel:
        line["single_channel"] = single_channel_section(fg, ctx, stream)
    if world == 1 and rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, t, k = cpu_sample(threads, CPU_BASELINE_SEGMENT_M)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": "%d realizations (launch powers -2..+4 dBm/ch) x the first %.0f m of a "
                                          "span: %d ADAPTIVE split steps in total and the EDFA with ASE, FP64 oracle "
                                          "port of ssfm.cpp/amplifier.cpp, %d threads, %.1f s"
                                          % (4 * threads, CPU_BASELINE_SEGMENT_M, k, threads, t)}
    if not args.no_dbp:
        # last, so the compact learned-vs-plain table ends the line
        line["learned_vs_plain"] = learned_vs_plain_section(fg, ctx)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def precision_section(fg, ctx, spans=None):
    """FP32 against FP64 on the workload's link at its own size, noise off:
    one realization at -2 and one at +4 dBm/ch propagated by the GPU with its
    ADAPTIVE grid recorded (focss_ssfm_run_record), the same grid replayed by
    a complex128 restatement of ssfm.cpp on the GPU (tests/fp64_ssfm.py, test
    infrastructure pinned to the FP64 oracle), field relative L2 after the
    20 spans, and the GPU's step counts against a free-running FP64 run."""
    import math

    import torch
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import fp64_ssfm
    from focss_gb300 import links
    spans = spans or W["spans"]
    link = links.Link(spans=spans)
    fib = link.fiber()
    amp = math.sqrt(link.gain())
    out = {"link": "N=2^19 WDM precision study, 20 x 80 km, ADAPTIVE, noise off, replayed grid"}
    for p in (-2.0, 4.0):
        field, _ = links.wdm_transmitter(link, W["symbols_per_channel"], 1, p, seed=7, ctx=ctx)
        rep = torch.from_numpy(field.numpy()[0]).cuda(ctx.device)
        free = rep.clone()
        s = fg.SSFM(fib)
        s.set_grid(fg.SSFM.ADAPTIVE)
        s.set_maximum_phase_shift(W["max_phase_shift"])
        s.set_maximum_step_size(W["max_step_m"])
        steps, d_steps = 0, 0
        for _ in range(spans):
            st, h = s.run_recorded(field, capacity=1 << 17)
            fg.Amplifier(link.gain()).amplify(field)
            rep = fp64_ssfm.run_steps(rep, field.domain.time_step, fib, h[0]) * amp
            free, taken = fp64_ssfm.run_adaptive(free, field.domain.time_step, fib, W["max_phase_shift"],
                                                 W["max_step_m"])
            free = free * amp
            steps += int(st[0])
            d_steps = max(d_steps, abs(int(st[0]) - len(taken)))
        got, want = field.numpy()[0, 0], rep.cpu().numpy()[0]
        err = float(np.linalg.norm(got - want) / np.linalg.norm(want))
        out["%+d_dbm" % p] = {"steps": steps, "field_rel_l2": err, "per_sqrt_step": err / math.sqrt(steps),
                              "max_step_count_delta_per_span": d_steps}
    return out


LVP = dict(
    wdm_link="5-ch WDM 20 x 80 km ADAPTIVE + ASE, centre channel at 2 sps",
    wdm_powers_dbm=[-2.0, 2.0, 4.0], single_channel="1 channel 4 sps, 20 x 80 km ADAPTIVE + ASE, 3 dBm",
    realizations=16, symbols_per_realization=2 ** 15, steps_per_span=4, iters=300, cnn_iters=1000,
)


def learned_vs_plain_section(fg, ctx):
    """Learned DBP at 4 steps/span against plain DBP at 1 / 4 / 100
    steps/span: Q (dB, mean over 16 test realizations x 2^15 symbols) and DBP
    time (ms) per launch power, on the WDM link's centre channel and on a
    single-channel link (training and test sets generated by the GPU split
    step).  Compact: [q_db, ms] per entry."""
    from focss_gb300 import links
    c = LVP
    out = {"config": c}

    def compact(r):
        return {k: [round(v["q_db"], 3), round(v["ms"], 3)] for k, v in r.items()}

    for p in c["wdm_powers_dbm"]:
        r = links.learned_vs_plain(links.Link(), p, c["symbols_per_realization"], c["realizations"],
                                   seed=int(500 + 10 * p), ctx=ctx, iters=c["iters"], cnn_iters=c["cnn_iters"])
        out["wdm_%+d_dbm" % p] = compact(r)
    single = links.Link(channels=1, osf=4)
    r = links.learned_vs_plain(single, 3.0, c["symbols_per_realization"], c["realizations"], seed=900, ctx=ctx,
                               iters=c["iters"], cnn_iters=c["cnn_iters"])
    out["single_channel_+3_dbm"] = compact(r)
    return out


SWEEP = dict(
    workload="sweep256_16qam_32GBd_2^12-2^16sym_8sps_15x80km_ssmf_ase_dbp_1-16stps",
    realizations=256, log2_symbols=[12, 16], samples_per_symbol=8, dbp_samples_per_symbol=2,
    powers_dbm=[-4.0, 4.0], spans=15, span_m=80e3, noise_figure_db=5.0, roll_off=0.1,
    forward="ADAPTIVE, max 0.005 rad/step, max 1 km", dbp_steps_per_span=[1, 2, 4, 8, 16], seed=3,
)


def _stream_ms(torch, stream, fn):
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    out = fn()
    e1.record(stream)
    e1.synchronize()
    return out, e0.elapsed_time(e1)


SINGLE = dict(
    workload="single_channel_16qam_32GBd_2^14sym_8sps_n2^17_10x80km_uniform_1km_2dBm",
    symbols=2 ** 14, samples_per_symbol=8, roll_off=0.1, spans=10, span_m=80e3, step_m=1000.0,
    power_dbm=2.0, batches=[1, 512], seed=7,
)


def single_channel_section(fg, ctx, stream):
    """Plain single-channel SSFM: 2^14 16QAM symbols at 8 samples/symbol
    (N = 2^17), 10 x 80 km SSMF with fixed 1 km steps and a lossless,
    noise-free EDFA after every span, 2 dBm.  GPU throughput of the span-loop
    graph for one realization (the reference's unit of work) and for 512
    copies (512 MB, 4x the L2); then the whole link, CDC, matched filter,
    phase search, Q and decisions for one realization against the FP64
    oracle, and the oracle's single-thread time for the propagation."""
    import torch
    from focss_gb300 import dsp
    sc = SINGLE
    alpha, beta2, gamma = fiber_params()
    fib = fg.Fiber(alpha, beta2, gamma, sc["span_m"])
    G = 10 ** (W["alpha_db_per_km"] * sc["span_m"] / 1e3 / 10)
    ns, osf = sc["symbols"], sc["samples_per_symbol"]
    n = ns * osf
    steps_per_span = int(round(sc["span_m"] / sc["step_m"]))
    rng = np.random.default_rng(sc["seed"])
    sym = dsp.qam16_map(rng.integers(0, 16, (1, 1, ns)), fg.Domain(1, ns, 1 / 32e9, F0), ctx=ctx)
    dsp.scale_each(sym, np.array([np.sqrt(1e-3 * 10 ** (sc["power_dbm"] / 10))]))
    sig = dsp.rrc_shaping(sym, osf, sc["roll_off"])
    x = sig.numpy()
    ssfm = fg.SSFM(fib, steps_per_span)
    out = {"config": sc, "samples": n, "runs": {}}
    for B in sc["batches"]:
        split = fg.autotune(n, B, ctx=ctx)[0]  # the split the library's autotuner picks for this batch
        f = fg.Field(sig.domain, data=np.broadcast_to(x, (B, 1, n)), batch=B, ctx=ctx)
        amp = fg.Amplifier(G, 0.0)
        fg.span_loop([f], fib, ssfm, sc["spans"], after=fg.Amplifier.AMPLIFY, amplifier=amp)  # warm-up
        ms = []
        for _ in range(3):
            f.upload(np.broadcast_to(x, (B, 1, n)))
            ctx.sync()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fg.span_loop([f], fib, ssfm, sc["spans"], after=fg.Amplifier.AMPLIFY, amplifier=amp)
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        t = statistics.median(ms)
        out["runs"]["batch_%d" % B] = {"ms": t, "gsample_steps_per_s": B * n * steps_per_span * sc["spans"] / t / 1e6,
                                       "log2_n1": split}
    # The whole link once more on one realization, then CDC, matched filter,
    # phase search (3600 angles), Q and decisions, against the FP64 oracle
    # (checker) running the same chain on one host thread.
    from oracle import build as obuild
    from oracle import cpu
    obuild.build_oracle()
    dt, cut = sig.domain.time_step, 100
    g = fg.Field(sig.domain, data=x, ctx=ctx)
    fg.span_loop([g], fib, ssfm, sc["spans"], after=fg.Amplifier.AMPLIFY, amplifier=fg.Amplifier(G, 0.0))
    got = g.numpy()[0, 0]
    fg.cd_compensation(g, fib, sc["spans"])
    y = dsp.PhaseShiftEqualizer(3600).train_equalize(sym, dsp.rrc_sampling(g, osf, sc["roll_off"]))
    q_gpu = float(dsp.q2_factor(sym, y, cut)[0])
    be, se = dsp.error_counts(sym, y, cut)
    codes = dsp.hd_sequence_16qam(y)[0, 0]
    ofib = cpu.Fiber(alpha, beta2, gamma, sc["span_m"], 1.55e-6, 1.0)
    t0 = time.perf_counter()
    xo = x[0, 0].copy()
    for _ in range(sc["spans"]):
        xo, _ = cpu.ssfm_run(xo, dt, ofib, cpu.UNIFORM, steps_per_span)
        xo = cpu.amplify(xo, dt, F0, G, 0.0)
    t_cpu = time.perf_counter() - t0
    field_err = float(np.linalg.norm(got - xo) / np.linalg.norm(xo))
    yo = cpu.rrc_sampling(cpu.cd_compensation(xo, dt, ofib, sc["spans"]), osf, sc["roll_off"])
    tx = sym.numpy()[0, 0]
    yo = cpu.rotate(yo, cpu.pse_estimate(tx, yo, 3600))
    q_o = float(cpu.q2(tx, yo, cut))
    out["link_vs_fp64_oracle"] = {
        "field_rel_l2_after_10_spans": field_err, "q_db_gpu": q_gpu, "q_db_fp64": q_o,
        "q_delta_db": q_gpu - q_o, "bit_errors_gpu": int(be[0]), "bit_errors_fp64": cpu.error_counts(tx, yo, cut)[0],
        "decisions_equal": int(np.sum(codes == cpu.hd_sequence(yo))), "symbols": int(codes.size)}
    out["cpu_oracle_one_thread"] = {"s_10_spans": t_cpu,
                                    "gsample_steps_per_s": n * steps_per_span * sc["spans"] / t_cpu / 1e9}
    return out


def sweep_section(fg, ctx, stream):
    """Batched sweep of independent single-channel realizations of uneven
    lengths: 2^U 16QAM symbols, U uniform in {12..16}, launch powers uniform
    in -4..+4 dBm, 8 samples/symbol, 15 x 80 km SSMF with ASE.  All lengths
    are one span-loop graph launch for the forward propagation and one for
    DBP at 1/2/4/8/16 steps per span (25 fields); the FFT split of every
    length (forward and DBP; -1 = the single-CTA kernel) is picked by the
    autotuner first."""
    import torch
    from focss_gb300 import dsp
    alpha, beta2, gamma = fiber_params()
    sw = SWEEP
    rng = np.random.default_rng(sw["seed"])
    R = sw["realizations"]
    U = rng.integers(sw["log2_symbols"][0], sw["log2_symbols"][1] + 1, R)
    P = rng.uniform(sw["powers_dbm"][0], sw["powers_dbm"][1], R)
    fib = fg.Fiber(alpha, beta2, gamma, sw["span_m"])
    G = 10 ** (W["alpha_db_per_km"] * sw["span_m"] / 1e3 / 10)
    NF = 10 ** (sw["noise_figure_db"] / 10)
    osf, dosf, spans = sw["samples_per_symbol"], sw["dbp_samples_per_symbol"], sw["spans"]
    lengths = sorted(set(int(u) for u in U))
    tx, pristine, pw = [], [], []
    for u in lengths:
        idx = np.nonzero(U == u)[0]
        ns = 1 << u
        codes = rng.integers(0, 16, (len(idx), 1, ns))
        sym = dsp.qam16_map(codes, fg.Domain(1, ns, 1 / 32e9, F0), batch=len(idx), ctx=ctx)
        dsp.scale_each(sym, np.sqrt(1e-3 * 10 ** (P[idx] / 10)))
        tx.append(sym)
        pristine.append(dsp.rrc_shaping(sym, osf, sw["roll_off"]))
        pw.append(P[idx])
    tuned = {}
    for f in pristine:
        tuned[f.domain.samples] = fg.autotune(f.domain.samples, f.batch, ctx=ctx)[0]
    ssfm = fg.SSFM(fib)
    ssfm.set_grid(fg.SSFM.ADAPTIVE)
    ssfm.set_maximum_phase_shift(W["max_phase_shift"])
    ssfm.set_maximum_step_size(W["max_step_m"])
    work = [f.copy() for f in pristine]

    def forward(seed):
        for w, f in zip(work, pristine):
            w.assign(f)
        return fg.span_loop(work, fib, ssfm, spans, after=fg.Amplifier.AMPLIFY,
                            amplifier=fg.Amplifier(G, NF, seed=seed))

    n0 = fg.launch_count()
    forward(300)  # records the graph
    n1 = fg.launch_count()
    steps, fwd_ms = _stream_ms(torch, stream, lambda: forward(301))
    fwd_launches = fg.launch_count() - n1
    fwd_ss = float(sum(int(st.sum()) * f.domain.samples for st, f in zip(steps, work)))

    rx = [dsp.decimate(w, osf // dosf) for w in work]
    for r in rx:  # DBP lengths too (2^12..2^14 may take the single-CTA kernel)
        tuned[r.domain.samples] = fg.autotune(r.domain.samples, r.batch, ctx=ctx)[0]
    ks = sw["dbp_steps_per_span"]
    dbp = [r.copy() for k in ks for r in rx]
    ssfms = [fg.SSFM(fib, k) for k in ks for _ in rx]

    def backward():
        for d, r in zip(dbp, [r for _ in ks for r in rx]):
            d.assign(r)
        return fg.span_loop(dbp, fib, ssfms, spans, direction=fg.SSFM.BACKWARD, amplifier=fg.Amplifier(G),
                            before=fg.Amplifier.DROP_POWER)

    backward()  # records
    n2 = fg.launch_count()
    _, dbp_ms = _stream_ms(torch, stream, backward)
    dbp_launches = fg.launch_count() - n2
    dbp_ss = float(sum(k * spans * r.batch * r.domain.samples for k in ks for r in rx))
    # the same DBP work through the host-driven span loop, for comparison
    host = [r.copy() for k in ks for r in rx]

    def backward_host():
        for d, r, s in zip(host, [r for _ in ks for r in rx], ssfms):
            d.assign(r)
            fg.backward_propagation(d, fib, s, G, spans)

    _, host_ms = _stream_ms(torch, stream, backward_host)
    q = {}
    pse = dsp.PhaseShiftEqualizer(720)
    for i, k in enumerate(ks):
        qs = []
        for j, t in enumerate(tx):
            y = dsp.rrc_sampling(dbp[i * len(rx) + j], dosf, sw["roll_off"])
            qs.append(dsp.q2_factor(t, pse.train_equalize(t, y), 100))
        q["%d_steps_per_span" % k] = float(np.mean(np.concatenate(qs)))
    return {
        "config": sw, "lengths_samples": {str(f.domain.samples): f.batch for f in pristine},
        "autotuned_log2_n1": {str(k): v for k, v in tuned.items()},
        "forward": {"graph_launches": 1, "kernels": int(fwd_launches), "ms": fwd_ms,
                    "sample_steps": fwd_ss, "gsample_steps_per_s": fwd_ss / fwd_ms / 1e6,
                    "first_call_kernels": int(n1 - n0)},
        "dbp": {"graph_launches": 1, "fields": len(dbp), "kernels": int(dbp_launches), "ms": dbp_ms,
                "sample_steps": dbp_ss, "gsample_steps_per_s": dbp_ss / dbp_ms / 1e6,
                "host_driven_ms": host_ms, "q_db_mean": q},
    }


PPE = dict(
    workload="ppe_16qam_32GBd_2^20sym_20x80km_ssmf_3dBm",
    symbols=2 ** 20, realizations=4, samples_per_symbol=4, power_dbm=3.0, spans=20, span_m=80e3,
    noise_figure_db=5.0, roll_off=0.1, forward="ADAPTIVE, max 0.005 rad/step, max 1 km",
    sino_radius=75, prune=1e-3, train_symbols=2 ** 16, fit="normal equations on the GPU, FP64 solve",
    angle_steps=720, cut=100, seed=4,
)


def ppe_section(fg, ctx, stream):
    """Perturbation (triplet) equalizer against 1- and 100-step/span DBP on
    one single-channel link: 2^20 received 16QAM symbols (4 realizations of
    2^18), 32 GBaud, 20 x 80 km SSMF with ASE at 3 dBm.  The coefficients
    come from SINO::train on an independent training realization (normal
    equations formed on the GPU, R = 75 diamond |m|+|n| <= R, 2889 features),
    pruned below 1e-3 of the largest; the equalizer runs on the CDC +
    matched-filter symbols."""
    import torch
    from focss_gb300 import dsp, sino
    alpha, beta2, gamma = fiber_params()
    c = PPE
    fib = fg.Fiber(alpha, beta2, gamma, c["span_m"])
    G = 10 ** (W["alpha_db_per_km"] * c["span_m"] / 1e3 / 10)
    NF = 10 ** (c["noise_figure_db"] / 10)
    osf, spans, ro = c["samples_per_symbol"], c["spans"], c["roll_off"]
    p = np.sqrt(1e-3 * 10 ** (c["power_dbm"] / 10))
    rng = np.random.default_rng(c["seed"])
    ssfm = fg.SSFM(fib)
    ssfm.set_grid(fg.SSFM.ADAPTIVE)
    ssfm.set_maximum_phase_shift(W["max_phase_shift"])
    ssfm.set_maximum_step_size(W["max_step_m"])

    def link(ns, batch, seed):
        codes = rng.integers(0, 16, (batch, 1, ns))
        sym = dsp.qam16_map(codes, fg.Domain(1, ns, 1 / 32e9, F0), batch=batch, ctx=ctx)
        sym *= p
        sig = dsp.rrc_shaping(sym, osf, ro)
        fg.span_loop([sig], fib, ssfm, spans, after=fg.Amplifier.AMPLIFY, amplifier=fg.Amplifier(G, NF, seed=seed))
        return sym, sig

    pse = dsp.PhaseShiftEqualizer(c["angle_steps"])

    def cdc_symbols(sig):
        f = sig.copy()
        fg.cd_compensation(f, fib, spans)
        return dsp.rrc_sampling(f, osf, ro)

    # training realization and coefficient fit (host least squares)
    tx_t, sig_t = link(c["train_symbols"], 1, 41)
    y_t = pse.train_equalize(tx_t, cdc_symbols(sig_t))
    t0 = time.perf_counter()
    model = sino.SINO(c["sino_radius"], 0.0, sino.SinoType.ORDINARY).train(tx_t, y_t, solver="gpu")
    fit_s = time.perf_counter() - t0
    m, n, cf = model.terms(c["prune"])

    # test set: 2^20 symbols
    ns = c["symbols"] // c["realizations"]
    tx, sig = link(ns, c["realizations"], 42)
    y = pse.train_equalize(tx, cdc_symbols(sig))
    q_cdc = float(np.mean(dsp.q2_factor(tx, y, c["cut"])))
    model.equalize(y, tx, c["prune"])  # warm-up
    eq, ppe_ms = _stream_ms(torch, stream, lambda: model.equalize(y, tx, c["prune"]))
    q_ppe = float(np.mean(dsp.q2_factor(tx, pse.train_equalize(tx, eq), c["cut"])))
    import ctypes as C
    peak = C.c_double()
    fg.lib().focss_measure_fp32_fma(ctx.h, C.byref(peak))
    tflops = 8.0 * m.size * c["symbols"] / ppe_ms / 1e9
    out = {"config": c, "terms": int(m.size), "fit_s": fit_s, "q_db_cdc": q_cdc,
           "ppe": {"q_db": q_ppe, "ms": ppe_ms, "msymbols_per_s": c["symbols"] / ppe_ms / 1e3,
                   "gflops": tflops * 1e3, "fp32_fma_peak_tflops_measured": peak.value,
                   "frac_of_fp32_peak": tflops / peak.value if peak.value > 0 else None}}
    rx2 = dsp.decimate(sig, osf // 2)
    for k in (1, 100):
        f = rx2.copy()
        ctx.sync()
        _, ms = _stream_ms(torch, stream, lambda: fg.backward_propagation(f, fib, fg.SSFM(fib, k), G, spans))
        yk = pse.train_equalize(tx, dsp.rrc_sampling(f, 2, ro))
        out["dbp_%d_steps_per_span" % k] = {"q_db": float(np.mean(dsp.q2_factor(tx, yk, c["cut"]))), "ms": ms}
    return out


DBP_SWEEP = dict(
    workload="learned_dbp_sweep_wdm5_centre_2^20sym_-2..+4dBm",
    powers_dbm=[-2, -1, 0, 1, 2, 3, 4], realizations=32, symbols_per_realization=2 ** 15, steps_per_span=4,
    taps=63, mf_taps=255, iters=300, lr=3e-4, cnn_iters=1000, cnn_lr=3e-4,
)


def dbp_sweep_section(fg, ctx):
    """Learned DBP at 4 steps/span against plain DBP at 1 / 4 / 100 steps/span
    over the launch-power sweep of the WDM link (centre channel, 2 samples/
    symbol): per power an independent training set and test set of 32
    realizations x 2^15 symbols (2^20 symbols each), the learned DBP trained
    on the training set (300 Adam steps), then the correction CNN."""
    from focss_gb300 import links
    c = DBP_SWEEP
    link = links.Link(spans=W["spans"], span_m=W["span_m"], noise_figure_db=W["noise_figure_db"],
                      max_phase=W["max_phase_shift"], max_step=W["max_step_m"], channels=W["channels"],
                      spacing=W["spacing_hz"], osf=W["samples_per_symbol"], roll_off=W["roll_off"])
    B, ns = c["realizations"], c["symbols_per_realization"]
    rows = []
    for i, p in enumerate(c["powers_dbm"]):
        a, ta = links.wdm_transmitter(link, ns, B, p, seed=1000 + 2 * i, ctx=ctx)
        b, tb = links.wdm_transmitter(link, ns, B, p, seed=1001 + 2 * i, ctx=ctx)
        links.propagate(link, a, seed=500 + 2 * i)
        links.propagate(link, b, seed=501 + 2 * i)
        ra, rb = links.centre_channel(link, a), links.centre_channel(link, b)
        del a, b
        row = {"power_dbm": p}
        for k in (1, 4, 100):
            q, ms = links.plain_dbp_q(link, rb, tb, k)
            row["plain_%d" % k] = {"q_db": float(np.mean(q)), "ms": ms}
        r = links.learned_dbp(link, ra, ta, rb, tb, steps_per_span=c["steps_per_span"], taps=c["taps"],
                              mf_taps=c["mf_taps"], iters=c["iters"], lr=c["lr"], cnn_iters=c["cnn_iters"],
                              cnn_lr=c["cnn_lr"])
        row["learned_%d" % c["steps_per_span"]] = {"q_db": float(np.mean(r["q_learned"])), "ms": r["ms_learned"],
                                                   "train_s": r["train_s"]}
        row["learned_%d_cnn" % c["steps_per_span"]] = {"q_db": float(np.mean(r["q_learned_cnn"])),
                                                       "ms": r["ms_learned_cnn"], "train_s": r["cnn_train_s"]}
        rows.append(row)
    return {"config": c, "powers": rows}


WDM_PPE = dict(
    workload="wdm_ppe_3ch_dualpol_16qam_32GBd_2^15sym_20x100km_2dBm",
    channels=3, polarizations=2, symbols=2 ** 15, samples_per_symbol=16, spacing_hz=37.5e9, power_index=16,
    power_dbm=2.0, spans=20, span_m=1e5, kappa=8 / 9, noise_figure_db=4.5, roll_off=0.01,
    forward="ADAPTIVE, max 0.001 rad/step, max 1 km", radii=[[30, 0], [30, 3]], cut=36,
    fit="normal equations on the GPU, FP64 solve", train_seed=1, test_seed=2,
)


def wdm_ppe_section(fg, ctx, stream):
    """The dual-polarization WDM dataset and scoring pipeline
    (src/tasks/wdm_run.cpp:79-141, src/tasks/wdm_scoring.cpp:158-187) on
    the GPU: 3 channels x 2 polarizations of 2^15 16QAM symbols, 16
    samples/symbol (N = 2^19 per polarization), 20 x 100 km SSMF with the
    Manakov factor 8/9 and ASE at 2 dBm per channel; CDC, channel selection,
    matched filter and phase-shift equalizer; WdmPPE fitted on a training
    realization and applied to a test realization with the received symbols
    and with their hard decisions as the triplet inputs (Q over both
    polarizations of the centre channel, cut 36)."""
    import torch
    from focss_gb300 import dsp, links
    c = WDM_PPE
    link = links.DualPolLink(spans=c["spans"], channels=c["channels"], osf=c["samples_per_symbol"])
    tx_t, rx_t, _ = links.wdm_dataset(link, c["symbols"], c["power_dbm"], c["train_seed"], ctx=ctx)
    ctx.sync()
    (tx, rx, steps), gen_ms = _stream_ms(
        torch, stream, lambda: links.wdm_dataset(link, c["symbols"], c["power_dbm"], c["test_seed"], ctx=ctx))
    n = c["symbols"] * c["samples_per_symbol"]
    tc = links.centre_rows(tx)
    out = {"config": c, "steps": steps, "dataset_ms": gen_ms,
           "forward_gsample_steps_per_s": 2 * n * steps / gen_ms / 1e6,
           "q_db_cdc": float(dsp.q2_factor(tc, links.centre_rows(rx), c["cut"])[0])}
    hd = dsp.hd(rx)
    for cr, dr in c["radii"]:
        ctx.sync()
        t0 = time.perf_counter()
        ppe = fg.WdmPPE(cr, dr).train(tx_t, rx_t)
        fit_s = time.perf_counter() - t0
        ppe.equalize(rx, rx)  # warm-up
        e_rx, ms_rx = _stream_ms(torch, stream, lambda: ppe.equalize(rx, rx))
        e_hd, ms_hd = _stream_ms(torch, stream, lambda: ppe.equalize(hd, rx))
        out["c%d_d%d" % (cr, dr)] = {
            "features": int(fg.lib().focss_wdm_ppe_num_features(cr, dr)), "fit_s": fit_s,
            "q_db_ppe_rx": float(dsp.q2_factor(tc, e_rx, c["cut"])[0]),
            "q_db_ppe_hd": float(dsp.q2_factor(tc, e_hd, c["cut"])[0]),
            "equalize_ms": ms_rx, "equalize_hd_ms": ms_hd,
            "abs_linear_weight": abs(ppe.get_linear_weight())}
    return out


def run_ncu_case(args):
    """Small fixed cases for ncu captures (one kernel family each):
    ssfm  UNIFORM split steps on `--ncu-batch` realizations of the N=2^19 WDM
          field (40 -> 168 MB, above the L2 size), 4 steps, then one EDFA;
    ppe   triplet equalizer on 2^20 symbols (4 x 2^18), 2113 diamond terms
          |m|+|n| <= 32 with decaying random coefficients;
    ldbp  learned-DBP forward + backward, 20 spans x 2 steps, 63/255 taps,
          8 x 2^16 samples;
    cnn   correction-CNN forward + backward, 8 x 2^15 symbols;
    dsp   transmitter / receiver DSP chain on 4 x 2^17 16QAM symbols at 8
          samples/symbol (2^20 samples): map, RRC shaping, channel selection,
          decimation, matched filter, phase search, decisions, certainty,
          error counts, Q;
    single one realization of N = 2^17 (the plain single-channel shape),
          UNIFORM 20 steps: the latency-bound small launches (narrow CTAs);
    block single-CTA split-step kernel, 304 realizations of N = 2^14 (2 CTAs
          per SM of work, 40 MB), UNIFORM 10 steps in one launch;
    fit   SINO normal equations (features, z-scores, FP64-accumulated Gram),
          R = 32 (577 features) on 2^17 symbols x 2 modes;
    wdmppe  WdmPPE (c, d) = (30, 3): equalizer on 16 x 6-row realizations of
          2^18 symbols (201 MB in, 67 MB out), then the fit's features on one
          6-row realization of 2^16 symbols;
    aux   the remaining kernels: field scale / power / natural-order FFT on
          40 x 2^19, a UNIFORM span loop graph with EDFA, the allocation-free
          entry point, WDM mux, RRC taps, hard-decision codes, one learned-DBP
          and one CNN training step (with Adam), SINO and WdmPPE fits."""
    import focss_gb300 as fg
    from focss_gb300 import dsp
    ctx = fg.Context(0)
    alpha, beta2, gamma = fiber_params()
    fib = fg.Fiber(alpha, beta2, gamma, W["span_m"])
    rng = np.random.default_rng(5)
    kind = args.ncu_case
    fg.set_pass_staging({"loads": fg.STAGING_LOADS, "bulk": fg.STAGING_BULK, "tma": fg.STAGING_TMA}[args.staging],
                        ctx=ctx)
    if kind == "ssfm":
        x = (synth_wdm() * np.sqrt(1e-3)).astype(np.complex64)
        B = args.ncu_batch
        if args.split:
            fg.set_fft_split(N, args.split, ctx=ctx)
        f = fg.Field(fg.Domain(1, N, DT, F0), data=np.broadcast_to(x, (B, 1, N)), batch=B, ctx=ctx)
        fg.SSFM(fib, 4).run(f)
        fg.Amplifier(10 ** 1.6, 10 ** 0.5, seed=1).amplify(f)
    elif kind == "single":
        n1 = 1 << 17
        if args.split:
            fg.set_fft_split(n1, args.split, ctx=ctx)
        x = ((rng.standard_normal(n1) + 1j * rng.standard_normal(n1)) * np.sqrt(0.8e-3)).astype(np.complex64)
        f = fg.Field(fg.Domain(1, n1, 1 / 256e9, F0), data=x[None, None], ctx=ctx)
        fg.SSFM(fib, 20).run(f)
    elif kind == "ppe":
        from focss_gb300 import sino
        R, ns, B = 32, 2 ** 18, 4
        y = dsp.qam16_map(rng.integers(0, 16, (B, 1, ns)), fg.Domain(1, ns, 1 / 32e9, F0), batch=B, ctx=ctx)
        mm, nn = np.meshgrid(np.arange(-R, R + 1), np.arange(-R, R + 1), indexing="ij")
        Wc = (rng.standard_normal(mm.shape) + 1j * rng.standard_normal(mm.shape)) * np.exp(-(abs(mm) + abs(nn)) / 8.0)
        m, n, c = sino.diamond_terms(Wc * 1e-2, R, 1e-3)
        for _ in range(2):
            sino.triplet_apply(y, R, m, n, c)
    elif kind == "ldbp":
        from focss_gb300.ldbp import LearnedDBP, rrc_response
        n2, B = 2 ** 16, 8
        dt2 = 1 / 64e9
        x = (rng.standard_normal((B, 1, n2)) + 1j * rng.standard_normal((B, 1, n2))) * 1e-2
        rx = fg.Field(fg.Domain(1, n2, dt2, F0), data=x, batch=B, ctx=ctx)
        tx = dsp.qam16_map(rng.integers(0, 16, (B, 1, n2 // 2)), fg.Domain(1, n2 // 2, 1 / 32e9, F0), batch=B,
                           ctx=ctx)
        model = LearnedDBP(20, 2, 63, 255, n2, B, 10 ** -0.8, ctx=ctx)
        model.init_from_dbp(alpha, beta2, gamma, 1.0, W["span_m"], dt2, rrc_response(n2 // 2, 2, 0.1, ctx=ctx))
        model.forward(rx)
        model.loss_grad(rx, tx)
    elif kind == "cnn":
        from focss_gb300.cnn import CorrectionCNN, he_init
        ns, B = 2 ** 15, 8
        y = dsp.qam16_map(rng.integers(0, 16, (B, 1, ns)), fg.Domain(1, ns, 1 / 32e9, F0), batch=B, ctx=ctx)
        net = CorrectionCNN(ns, B, 1.0, ctx=ctx)
        net.set_params(he_init(rng))
        net.forward(y)
        net.loss_grad(y, y)
    elif kind == "block":
        n, B = 1 << 14, 304
        x = (rng.standard_normal((B, 1, n)) + 1j * rng.standard_normal((B, 1, n))) * 0.02
        f = fg.Field(fg.Domain(1, n, DT, F0), data=x.astype(np.complex64), batch=B, ctx=ctx)
        fg.set_fft_split(n, fg.SPLIT_SINGLE_CTA, ctx=ctx)
        fg.SSFM(fib, 10).run(f)
    elif kind == "dsp":
        ns, osf, B = 2 ** 17, 8, 4
        codes = rng.integers(0, 16, (B, 1, ns))
        sym = dsp.qam16_map(codes, fg.Domain(1, ns, 1 / 32e9, F0), batch=B, ctx=ctx)
        sig = dsp.rrc_shaping(sym, osf, 0.1)
        sel = dsp.wdm_select(sig, 0, 50e9)
        dec = dsp.decimate(sel, osf // 2)
        y = dsp.rrc_sampling(sig, osf, 0.1)
        y = dsp.PhaseShiftEqualizer(720).train_equalize(sym, y)
        dsp.hard_decision_16qam(y)
        dsp.soft_decision_16qam(y, 0.05)
        dsp.certainty_decision(y, float(dsp.find_certainty(sym, y)[0]))
        dsp.error_counts(sym, y, 100)
        dsp.q2_factor(sym, y, 100)
        del dec
    elif kind == "fit":
        from focss_gb300 import sino
        ns = 2 ** 17
        tx = dsp.qam16_map(rng.integers(0, 16, (1, 2, ns)), fg.Domain(2, ns, 1 / 32e9, F0), ctx=ctx)
        rx = tx.copy()
        sino.SINO(32).train(tx, rx, solver="gpu")
    elif kind == "wdmppe":
        c, d, ns, B = 30, 3, 2 ** 18, 16
        codes = rng.integers(0, 16, (B, 6, ns))
        tx = dsp.qam16_map(codes, fg.Domain(6, ns, 1 / 32e9, F0), batch=B, ctx=ctx)
        ppe = fg.WdmPPE(c, d)
        nf = int(fg.lib().focss_wdm_ppe_num_features(c, d))
        ppe.install((rng.standard_normal(nf) + 1j * rng.standard_normal(nf)) * 1e-3)
        ppe.linear_weight = 1.0
        for _ in range(2):
            ppe.equalize(tx, tx)
        t1 = dsp.qam16_map(codes[:1, :, :2 ** 16], fg.Domain(6, 2 ** 16, 1 / 32e9, F0), ctx=ctx)
        fg.WdmPPE(c, d).train(t1, t1)
    elif kind == "aux":
        import ctypes as C
        from focss_gb300 import sino
        from focss_gb300._lib import check
        from focss_gb300.cnn import CorrectionCNN, he_init
        from focss_gb300.ldbp import LearnedDBP, rrc_response
        # field utilities on 40 realizations of N = 2^19 (168 MB)
        B = 40
        x = (synth_wdm() * np.sqrt(1e-3)).astype(np.complex64)
        f = fg.Field(fg.Domain(1, N, DT, F0), data=np.broadcast_to(x, (B, 1, N)), batch=B, ctx=ctx)
        f *= 0.5
        f.power_stats()
        f.fft_inplace()
        f.ifft_inplace()
        # span loop on a UNIFORM grid (no conditional node, so its kernel nodes can be profiled)
        fg.span_loop([f], fib, fg.SSFM(fib, 2), 2, amplifier=fg.Amplifier(10 ** 1.6, 10 ** 0.5, seed=1),
                     after=0)
        # allocation-free entry point, 8 x 2^17 samples, 4 UNIFORM steps
        n17 = 1 << 17
        g = fg.Field(fg.Domain(1, n17, DT, F0), data=x[None, None, :n17].repeat(8, 0), batch=8, ctx=ctx)
        steps = np.zeros(8, np.int32)
        fb, op = fib.c(), fg.SSFM(fib, 4).opts()
        check(fg.lib().focss_ssfm_run_noalloc(ctx.stream, g.device_ptr(), n17, 8, DT, C.byref(fb), C.byref(op),
                                              1.0, steps.ctypes.data_as(C.c_void_p)), ctx.h)
        # WDM multiplexer (5 channels of 2^19 samples), RRC taps, hard-decision codes on 16 x 2^18 symbols
        dsp.wdm_mux(f.slice(0, 5), 50e9)
        dsp.rrc_pulse(2 ** 12, 8, 0.1, ctx=ctx)
        y = dsp.qam16_map(rng.integers(0, 16, (16, 1, 2 ** 18)), fg.Domain(1, 2 ** 18, 1 / 32e9, F0), batch=16,
                          ctx=ctx)
        dsp.hd_sequence_16qam(y)
        # learned DBP training step (8 x 2^16 samples, 20 spans x 2 steps)
        n2, dt2 = 2 ** 16, 1 / 64e9
        rx = fg.Field(fg.Domain(1, n2, dt2, F0), data=(rng.standard_normal((8, 1, n2)) + 0j) * 1e-2, batch=8,
                      ctx=ctx)
        tx = dsp.qam16_map(rng.integers(0, 16, (8, 1, n2 // 2)), fg.Domain(1, n2 // 2, 1 / 32e9, F0), batch=8,
                           ctx=ctx)
        model = LearnedDBP(20, 2, 63, 255, n2, 8, 10 ** -0.8, ctx=ctx)
        model.init_from_dbp(alpha, beta2, gamma, 1.0, W["span_m"], dt2, rrc_response(n2 // 2, 2, 0.1, ctx=ctx))
        model.loss_grad(rx, tx)
        model.adam_step(1e-3)
        # correction-CNN training step (8 x 2^15 symbols)
        y15 = dsp.qam16_map(rng.integers(0, 16, (8, 1, 2 ** 15)), fg.Domain(1, 2 ** 15, 1 / 32e9, F0), batch=8,
                            ctx=ctx)
        net = CorrectionCNN(2 ** 15, 8, 1.0, ctx=ctx)
        net.set_params(he_init(rng))
        net.loss_grad(y15, y15)
        net.adam_step(1e-3)
        # SINO / WdmPPE fits: responses, z-scores, residual refinement (design apply / adjoint)
        ns = 2 ** 17
        t2 = dsp.qam16_map(rng.integers(0, 16, (1, 2, ns)), fg.Domain(2, ns, 1 / 32e9, F0), ctx=ctx)
        sino.SINO(16).train(t2, t2.copy(), solver="gpu")
        t6 = dsp.qam16_map(rng.integers(0, 16, (1, 6, 2 ** 16)), fg.Domain(6, 2 ** 16, 1 / 32e9, F0), ctx=ctx)
        fg.WdmPPE(8, 2).train(t6, t6)
    else:
        raise SystemExit("unknown ncu case %r" % kind)
    ctx.sync()
    print("ncu case %s done" % kind)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ncu-case", nargs="?", const="ssfm", default=None,
                    help="small fixed case for ncu captures: ssfm (default), single, ppe, ldbp, cnn, dsp, block, fit, wdmppe, aux")
    ap.add_argument("--ncu-batch", type=int, default=40)
    ap.add_argument("--split", type=int, default=0, help="ncu case: log2 N1 of the FFT split (0: balanced)")
    ap.add_argument("--staging", default="loads", choices=["loads", "bulk", "tma"],
                    help="ncu case: how the split-step passes move their data (focss_set_pass_staging)")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-dbp", action="store_true", help="skip the learned-vs-plain DBP section")
    ap.add_argument("--no-precision", action="store_true",
                    help="skip the FP32-vs-FP64 field error on the replayed grid (about 20 s)")
    ap.add_argument("--no-sweep", action="store_true", help="skip the uneven-length batched sweep section")
    ap.add_argument("--no-ppe", action="store_true", help="skip the perturbation-equalizer section")
    ap.add_argument("--no-wdm-ppe", action="store_true",
                    help="skip the dual-polarization WDM dataset and WdmPPE scoring section")
    ap.add_argument("--dbp-sweep", action="store_true",
                    help="add the learned-vs-plain DBP launch-power sweep (-2..+4 dBm, 2^20 symbols per set; minutes)")
    ap.add_argument("--single-channel", action="store_true",
                    help="add the plain single-channel link (N=2^17, 10 x 80 km, 1 km steps): GPU throughput at "
                         "batch 1 and 512, then field, Q and decisions against the FP64 oracle (about 10 s of CPU)")
    ap.add_argument("--host-loop", action="store_true",
                    help="drive the spans from the host (one SSFM run + EDFA per span) instead of one graph")
    args = ap.parse_args()
    if args.ncu_case:
        return run_ncu_case(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
