#!/usr/bin/env python
"""Benchmark of the BICOS matching path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload: the production stack, 1936x1216 uint8, n=33, limited descriptors
(126 bits -> 128-bit words), nxcorr_threshold 0.96, min_variance 2.0,
subpixel step 0.1, NoDuplicates; precision single (headline) and double.
Seeded synthetic scenes (libbicos_gb300.scenes) stand in for the
reference's dataset.  A step is one full match of one stereo stack.

`value` is whole-job stereo Mpx/s with inputs resident in HBM; `e2e` is the
same metric through the host-buffer C-ABI call (bicos_match_host_v1, what
pybicos.match uses) with the H2D upload of both stacks and the D2H download
of disparity + corrmap inside the timed region.  Under torchrun each rank
matches its own stack (weak scaling, no collective on the data path).

--impl reference times the reference's CPU implementation of the path on
the host cores (the reference CPU backend compiled from source where the
sources exist, else the project's C restatement of it), on a bounded sample
of rows of the same workload per step.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "mv1936_n33"
METRIC = "stereo Mpx/s"
THRESHOLD, MIN_VAR, STEP = 0.96, 2.0, 0.1


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-double", action="store_true")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned subpixel form")
    ap.add_argument("--no-batch", action="store_true", help="skip the 16-stack batch comparison")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the 640x480 and the 2048x1536 12-bit precision-form workloads")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="target CPU work of the baseline sample")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    return int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")), ws


def max_over_ranks(v, ws, device="cpu"):
    """The slowest rank's time (a replica run is as fast as its slowest
    rank); works over NCCL (device = the rank's GPU) and gloo (CPU)."""
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(px_per_rank, seconds, ws):
    """Whole-job rate of ws replicas each processing px_per_rank in
    `seconds` (the max over ranks), in Mpx/s."""
    return ws * px_per_rank / seconds / 1e6


def workload_config(double=False):
    return {"workload": f"{WORKLOAD}: 1936x1216 uint8 stereo stack, n=33, limited descriptors (128-bit), "
                        f"threshold {THRESHOLD}, min_variance {MIN_VAR}, subpixel step {STEP}, NoDuplicates, "
                        f"precision {'double' if double else 'single'}",
            "rows": 1216, "cols": 1936, "n": 33, "input": "uint8",
            "l2": "inputs larger than L2: 155 MB of frames streamed per step (L2 129 MB)"}


def oracle_mpx(scene, rows, cfg, use_ref=False, nthreads=0):
    from oracle import oracle as O
    t = time.perf_counter()
    O.match(scene.left[:, :rows], scene.right[:, :rows], cfg, nthreads=nthreads, use_ref=use_ref)
    dt = time.perf_counter() - t
    return rows * scene.left.shape[2] / dt / 1e6, dt


def cpu_sample_rows(scene, cfg, target_s, use_ref=False):
    probe = 8
    _, dt = oracle_mpx(scene, probe, cfg, use_ref)
    return int(max(probe, min(scene.left.shape[1], target_s / max(dt / probe, 1e-6))))


# The C restatement (oracle/bicos_oracle.c, "port") against libBICOS's own
# CPU backend built from its sources (oracle/ref_build.sh), same host, same
# 48 rows of the production stack, all threads: measured on an 8-core x86
# host (the GPU hosts carry no reference sources), port 0.38-0.40 Mpx/s,
# reference build 0.29-0.36 Mpx/s.  Where only the port runs, the CPU
# numbers here are, if anything, faster than the reference's own.
PORT_VS_REFERENCE = ("the port ran at about 1.2x the reference build's speed on the same 8-core x86 host "
                     "(0.38 vs 0.31 Mpx/s on 48 rows of this stack), so it does not flatter the GPU ratio")


def cpu_baseline(scene, target_s):
    from oracle import oracle as O
    cfg = O.make_config(threshold=THRESHOLD, step=STEP, min_variance=MIN_VAR)
    use_ref = O.ref_available()
    rows = cpu_sample_rows(scene, cfg, target_s / 3, use_ref)
    runs = [oracle_mpx(scene, rows, cfg, use_ref) for _ in range(3)]
    mpx = float(np.median([r[0] for r in runs]))
    dt = sum(r[1] for r in runs)
    whole = " (the whole frame: the sample is capped at one full match)" if rows == scene.left.shape[1] else ""
    return {"value": round(mpx, 4), "unit": "Mpx/s", "cores": O.lib().orc_num_threads(0) if not use_ref else os.cpu_count(),
            "kind": "reference" if use_ref else "port",
            "sample": f"rows 0..{rows - 1} of the {WORKLOAD} stack (all 1936 columns, n=33){whole}, "
                      f"median of 3 runs, {dt:.1f} s in all"
                      + ("" if use_ref else f"; {PORT_VS_REFERENCE}")}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.proc = None
        self.lines = []
        self.dev = device_index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p["hbm_gbs"], p["bf16_tflops"], "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, 1900.0, "fallback"


# FP8 tensor-core rates of this GPU (TFLOP/s by MMA N: 128 the search's
# shape, 256 the largest single-CTA shape), measured once per run by
# bicos_tc_fp8_rate_v1 before any timed region; empty when not measured
FP8_RATE = {}


def measure_fp8_rate(lbg):
    for nn in (128, 256):
        try:
            FP8_RATE[nn] = round(lbg.tc_fp8_rate(nn), 1)
        except Exception as e:  # the roofline then falls back to 2 x bf16
            print(f"bench: FP8 rate probe (N={nn}) failed: {e}", file=sys.stderr)
            FP8_RATE.clear()
            return


def profile_traffic(kernel):
    """DRAM bytes per launch of `kernel` from the committed ncu summaries
    (a line "traffic_bytes_per_launch <kernel>: <bytes>")."""
    key = f"traffic_bytes_per_launch {kernel}:"
    for name in sorted(os.listdir(os.path.join(ROOT, "profiles"))):
        try:
            for line in open(os.path.join(ROOT, "profiles", name)):
                if line.startswith(key):
                    return float(line.split(":", 1)[1].split()[0])
        except OSError:
            pass
    return None


def sweep_positions(step):
    """Sweep points per pixel: x = -1, then x += step in float32 (the
    reference's loop) while x <= 1 -- 20 at step 0.1, whose 21st sum is
    1.0000001."""
    x, s, k = np.float32(-1.0), np.float32(step), 0
    while x <= np.float32(1.0):
        k += 1
        x = np.float32(x + s)
    return k


def stage_rooflines(stages, rows, cols, n, clk, valid=0.806, eb=1, nwords=4, dirs=1, full=False,
                    agree="subpixel_f32", positions=None):
    """Roofline of each stage from its live CUDA-event time (ms per launch).

    transform: HBM, bytes 2*px*n*eb (stack in) + 2*px*4*nwords (words out)
               + the FP8 candidate tiles it writes for the tensor-core
               search (words up to 256 bits, rows up to 4096 columns):
               dirs*rows*128*ceil(cols/128)*32*nwords
    search:    tensor, 2*rows*cols^2*32*nwords FLOP per direction (+-1 FP8
               dot products over the padded descriptor width) against the
               FP8 rate measured on this GPU (tcgen05.mma kind::f8f6f4,
               M=128 N=256 K=32 issued alone), with the rate of the search's
               own N=128 shape beside it; twice the measured bf16 GEMM rate
               when the probe did not run
    agreement: HBM, bytes 2*px*n*eb (stack in) + px*(2 or 4) disparity
               out + px*(4 or 8) corrmap out (+ px*2 raw disparity in);
               the single-precision sweep's FP32 view (12 flops per valid
               pixel, sweep position and frame, against the FP32 vector
               peak 152 SMs x 128 lanes x 2 x SM clock) rides along under
               "fp32"
    agree: the agreement kernel ("subpixel_f32", "subpixel_f64", "agree",
    "moments"); positions: sweep positions per pixel (default: those of
    the workload's step, 20 at step 0.1).
    """
    if positions is None:
        positions = sweep_positions(STEP)
    hbm, bf16, src = peaks()
    px = rows * cols
    sm_mhz = clk.get("sm_mhz") or 2070.0
    t_tf, t_se, t_ag = [max(x, 1e-9) for x in stages]
    tf_bytes = 2 * px * n * eb + 2 * px * 4 * nwords
    if nwords <= 8 and cols <= 4096:
        # the transform also writes the searched sides' FP8 candidate tiles
        # (one byte per descriptor bit slot, whole 128-column tiles)
        tf_bytes += dirs * rows * ((cols + 127) // 128) * 128 * 32 * nwords
    se_flop = 2.0 * rows * cols * cols * 32 * nwords * dirs
    dbl = agree in ("subpixel_f64", "moments")
    sweep = agree.startswith("subpixel") or agree == "moments"
    ag_bytes = 2 * px * n * eb + px * (4 if sweep else 2) + px * (8 if dbl else 4) + px * 2
    fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
    if FP8_RATE:
        fp8_peak = FP8_RATE[256]
        fp8_src = "measured FP8 tcgen05.mma rate, M128 N256 K32 issued alone (bicos_tc_fp8_rate_v1)"
    else:
        fp8_peak = 2 * bf16
        fp8_src = f"FP8 dense = 2 x {src} bf16 GEMM rate"
    tf_kernel = "k_transform_full" if full else "k_transform_limited"
    ag_kernel = {"subpixel_f32": "k_subpixel_f32", "subpixel_f64": "k_subpixel_f64", "agree": "k_agree",
                 "moments": "k_moments"}[agree]

    def gbs(b, t):
        return b / (t * 1e-3) / 1e9
    out = {
        "transform": {"kernel": tf_kernel, "bound": "hbm", "ms": round(t_tf, 4),
                      "achieved": round(gbs(tf_bytes, t_tf), 1), "peak": hbm, "unit": "GB/s",
                      "frac": round(gbs(tf_bytes, t_tf) / hbm, 4), "peak_source": f"{src} HBM copy bandwidth",
                      "traffic": profile_traffic(tf_kernel), "algorithmic_bytes": tf_bytes},
        "search": {"kernel": "k_search_tc", "bound": "tensor", "ms": round(t_se, 4),
                   "achieved": round(se_flop / (t_se * 1e-3) / 1e12, 1), "peak": round(fp8_peak, 1),
                   "unit": "TFLOP/s", "frac": round(se_flop / (t_se * 1e-3) / 1e12 / fp8_peak, 4),
                   "peak_source": fp8_src,
                   "traffic": profile_traffic("k_search_tc"), "algorithmic_flop": se_flop,
                   "directions": dirs},
        "agreement": {"kernel": ag_kernel, "bound": "hbm", "ms": round(t_ag, 4),
                      "achieved": round(gbs(ag_bytes, t_ag), 1), "peak": hbm, "unit": "GB/s",
                      "frac": round(gbs(ag_bytes, t_ag) / hbm, 4), "peak_source": f"{src} HBM copy bandwidth",
                      "traffic": profile_traffic(ag_kernel), "algorithmic_bytes": ag_bytes},
    }
    if FP8_RATE:
        se = out["search"]
        se["shape_peak"] = FP8_RATE[128]
        se["frac_of_shape_peak"] = round(se["achieved"] / FP8_RATE[128], 4)
        se["peak_2x_bf16"] = round(2 * bf16, 1)
    if agree == "subpixel_f32":
        ag_flop = 12.0 * valid * px * positions * n
        out["agreement"]["fp32"] = {
            "achieved": round(ag_flop / (t_ag * 1e-3) / 1e12, 2), "peak": round(fp32_peak, 1),
            "unit": "TFLOP/s", "frac": round(ag_flop / (t_ag * 1e-3) / 1e12 / fp32_peak, 4),
            "peak_source": f"FP32 vector peak at the median SM clock {sm_mhz:.0f} MHz",
            "algorithmic_flop": ag_flop}
    return out


def batch_bench(lbg, pybicos, scenes, seed, rounds=3, specs=None):
    """Stacks of mixed size, depth, input type, mode and step (default: the
    16-stack workload): one bicos_match_batch_v1 graph replay (autotuned
    launch shapes) against one bicos_match_v1 call per stack, same GPU,
    same outputs (checked bit for bit)."""
    import torch
    specs = scenes.batch_specs(16, seed) if specs is None else specs
    jobs, px = [], 0
    for k, (rows, cols, n, bits, full, step) in enumerate(specs):
        left, right = scenes.make_scene_device(rows, cols, n, seed=seed * 100 + k, bits=bits, d_range=(20.0, 120.0))
        c = pybicos.Config()
        c.nxcorr_threshold, c.min_variance, c.subpixel_step = 0.9, 2.0, step
        c.mode = pybicos.Full if full else pybicos.Limited
        jobs.append((left, right, c))
        px += rows * cols
    stream = torch.cuda.current_stream()
    seq_outs = lbg.Batch.outputs(jobs)

    def sequential():
        for (l, r, c), out in zip(jobs, seq_outs):
            lbg.match_device(l, r, c, out=out, max_bits=512)

    b = lbg.Batch()
    outs = b.match(jobs, max_bits=512)
    tuning = b.autotune(jobs, outs, max_bits=512)
    sequential()
    b.match(jobs, outs, max_bits=512)

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(rounds):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / rounds

    ms_seq = timed(sequential)
    ms_batch = timed(lambda: b.match(jobs, outs, max_bits=512))

    def bits(t):
        return t.view(torch.int16 if t.element_size() == 2 else torch.int32 if t.element_size() == 4 else torch.int64)

    exact = all(torch.equal(bits(a), bits(bb)) and (ca is None or torch.equal(bits(ca), bits(cb)))
                for (a, ca), (bb, cb) in zip(outs, seq_outs))
    return {"stacks": len(jobs), "megapixels": round(px / 1e6, 3),
            "specs": [f"{c}x{r} n={n} {'u16(12-bit)' if bits_ == 12 else 'u8'} {'full' if full else 'limited'} "
                      f"step={step}" for r, c, n, bits_, full, step in specs],
            "batched": {"value": round(px / (ms_batch * 1e-3) / 1e6, 3), "unit": "Mpx/s", "ms": round(ms_batch, 3)},
            "sequential": {"value": round(px / (ms_seq * 1e-3) / 1e6, 3), "unit": "Mpx/s", "ms": round(ms_seq, 3)},
            "batched_vs_sequential": round(ms_seq / ms_batch, 3), "bit_exact": bool(exact), "tuning": tuning,
            "graph_captures": b.captures,
            "data": "seeded synthetic stacks generated on the GPU (make_scene_device), threshold 0.9, "
                    "min_variance 2.0"}


def moment_form_error(d_ref, c_ref, d_mom, c_mom):
    """|d rho| and |d disparity| of the moment form against the reference
    form (both double precision) on pixels valid in both, and the share of
    pixels whose validity agrees."""
    import torch
    both = torch.isfinite(d_ref) & torch.isfinite(d_mom)
    dd = (d_mom[both].double() - d_ref[both].double()).abs()
    dr = (c_mom[both] - c_ref[both]).abs()

    def q(v, p):
        return float(torch.quantile(v[torch.randperm(v.numel(), device=v.device)[:1 << 24]], p))
    return {"pixels_valid_in_both": int(both.sum()),
            "validity_agreement": round(float((torch.isfinite(d_ref) == torch.isfinite(d_mom)).double().mean()), 6),
            "rho_abs_err": {"median": q(dr, 0.5), "p95": q(dr, 0.95), "max": float(dr.max())},
            "disparity_abs_err_px": {"median": q(dd, 0.5), "p95": q(dd, 0.95), "max": float(dd.max()),
                                     "rms": float(torch.sqrt(torch.mean(dd ** 2)))}}


def config_benches(lbg, pybicos, scenes, timed_match, clk, seed, steps):
    """The two other seeded workloads, each timed like the headline one:
    c0 -- 640x480 uint8, n=12, limited (64-bit words), threshold 0.9,
    min_variance 2.0, no subpixel, NoDuplicates, single precision;
    c2 -- 2048x1536 12-bit (uint16), n=20, FULL descriptors (363 bits, the
    512-bit extension), Consistency{1}, threshold 0.9, step 0.1: the
    reference form in double precision and the moment form (Sxy on the
    tensor cores, exact int64 moments, FP64 cross term), with the moment
    form's error against the reference form's FP64 results."""
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())
    out = {}
    sc = scenes.workload_scene("vga_n12", seed=seed)
    n, rows, cols = sc.left.shape
    left, right = torch.from_numpy(sc.left).to(dev), torch.from_numpy(sc.right).to(dev)
    c = pybicos.Config()
    c.nxcorr_threshold, c.min_variance = 0.9, 2.0
    ms, st, o = timed_match(left, right, c, steps * 4, 5, stage_times=True)
    valid = float((o[0] != -32768).float().mean())
    c0 = {"value": round(rows * cols / (ms * 1e-3) / 1e6, 3), "unit": "Mpx/s", "ms_per_step": round(ms, 4),
          "config": "640x480 uint8, n=12, limited (41 bits -> 64-bit words), threshold 0.9, min_variance 2.0, "
                    "no subpixel, NoDuplicates, single precision",
          "l2": "inputs (7.4 MB) fit in L2: back-to-back calls, warm L2",
          "valid_fraction": round(valid, 4),
          "stage_ms": {"transform": round(st[0], 4), "search": round(st[1], 4), "agreement": round(st[2], 4)},
          "stage_rooflines": stage_rooflines(st, rows, cols, n, clk, valid, nwords=2, agree="agree")}
    del left, right

    sc = scenes.workload_scene("qxga12_n20", seed=seed)
    n, rows, cols = sc.left.shape
    left, right = torch.from_numpy(sc.left).to(dev), torch.from_numpy(sc.right).to(dev)
    res = {"config": "2048x1536 12-bit samples in uint16, n=20, FULL descriptors (363 bits -> 384-bit words, "
                     "the max_bits=512 extension: libBICOS throws for this stack), Consistency{max_lr_diff=1}, "
                     "threshold 0.9, step 0.1, precision double",
           "l2": "inputs larger than L2: 252 MB of frames per step (L2 129 MB)"}
    outs = {}
    for name, form in (("reference_form", 0), ("moment_form", 1)):
        c = pybicos.Config()
        c.nxcorr_threshold, c.subpixel_step = 0.9, 0.1
        c.mode, c.precision, c.nxcorr_form = pybicos.Full, pybicos.Double, form
        c.variant = pybicos.Variant.Consistency(1, False)
        ms, st, o = timed_match(left, right, c, steps, 2, stage_times=True, max_bits=512)
        outs[name] = o
        valid = float(torch.isfinite(o[0]).float().mean())
        res[name] = {"value": round(rows * cols / (ms * 1e-3) / 1e6, 3), "unit": "Mpx/s",
                     "ms_per_step": round(ms, 4), "valid_fraction": round(valid, 4),
                     "stage_ms": {"transform": round(st[0], 4), "search": round(st[1], 4),
                                  "agreement": round(st[2], 4)},
                     "stage_rooflines": stage_rooflines(st, rows, cols, n, clk, valid, eb=2, nwords=12, dirs=2,
                                                        full=True,
                                                        agree="subpixel_f64" if form == 0 else "moments")}
    (d_ref, c_ref), (d_mom, c_mom) = outs["reference_form"], outs["moment_form"]
    res["moment_form_error_vs_fp64_reference"] = moment_form_error(d_ref, c_ref, d_mom, c_mom)
    return c0, res


def learned_error(lbg, pybicos, left, right, plain, learned, n):
    """RMS subpixel error (px) of the learned form and of the plain step-0.1
    sweep against the reference sweep with step 0.01 in double precision,
    on interior pixels valid in all three."""
    import torch
    c = pybicos.Config()
    c.nxcorr_threshold = None
    raw, _ = lbg.match_device(left, right, c)
    ref, _ = lbg.agree_subpixel(raw, left, right, THRESHOLD, 0.01, MIN_VAR * n, double=True)
    cols = raw.shape[1]
    col1 = torch.arange(cols, device=raw.device)[None, :] - raw.to(torch.int32)
    m = torch.isfinite(ref) & torch.isfinite(plain) & torch.isfinite(learned) & (col1 > 0) & (col1 < cols - 1)

    def rms(v):
        return round(float(torch.sqrt(torch.mean((v[m].double() - ref[m].double()) ** 2))), 5)
    return {"reference": "reference sweep, step 0.01, double precision, same threshold and min_variance",
            "learned_rms_px": rms(learned), "plain_sweep_rms_px": rms(plain), "pixels": int(m.sum())}


def run_ours(args):
    import torch
    import torch.distributed as dist

    rank, local_rank, ws = dist_env()
    if ws > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local_rank)
    device = torch.device("cuda", local_rank)

    import libbicos_gb300 as lbg
    from libbicos_gb300 import _native as N
    from libbicos_gb300 import build as B
    from libbicos_gb300 import pybicos, scenes
    import ctypes as C

    B.build()
    L = lbg.load_library()
    measure_fp8_rate(lbg)
    scene = scenes.workload_scene(WORKLOAD, seed=args.seed + rank)
    n, rows, cols = scene.left.shape
    px = rows * cols
    left = torch.from_numpy(scene.left).to(device)
    right = torch.from_numpy(scene.right).to(device)

    def cfg_of(double):
        c = pybicos.Config()
        c.nxcorr_threshold, c.min_variance, c.subpixel_step = THRESHOLD, MIN_VAR, STEP
        c.precision = pybicos.Double if double else pybicos.Single
        return c

    def barrier():
        if ws > 1:
            dist.barrier()

    def ranks_max(v):
        return max_over_ranks(v, ws, device)

    def timed(double, steps, warmup, stage_times=False, form=0):
        cfg = cfg_of(double)
        cfg.nxcorr_form = form
        return timed_match(left, right, cfg, steps, warmup, stage_times)

    def timed_match(left, right, cfg, steps, warmup, stage_times=False, max_bits=256):
        out = lbg.match_device(left, right, cfg, max_bits=max_bits)
        for _ in range(warmup):
            lbg.match_device(left, right, cfg, out=out, max_bits=max_bits)
        stream = torch.cuda.current_stream()
        if stage_times:
            N.check(L.bicos_stage_timing(1))
        barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            lbg.match_device(left, right, cfg, out=out, max_bits=max_bits)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        ms = e0.elapsed_time(e1) / steps
        st = None
        if stage_times:
            arr = (C.c_float * 3)()
            calls = C.c_int32()
            N.check(L.bicos_stage_times(arr, C.byref(calls)))
            N.check(L.bicos_stage_timing(0))
            st = [arr[i] / max(calls.value, 1) for i in range(3)]
        return ranks_max(ms), st, out

    dev_index = torch.cuda.current_device()
    try:
        uuid = str(torch.cuda.get_device_properties(dev_index).uuid)
        smi_dev = uuid if uuid.startswith("GPU-") else f"GPU-{uuid}"
    except Exception:
        smi_dev = dev_index
    with ClockSampler(smi_dev) as clocks:
        ms, stages, out = timed(False, args.steps, args.warmup, stage_times=True)
    clk = clocks.summary()
    value = replica_rate(px, ms * 1e-3, ws)

    valid = float(torch.isfinite(out[0]).float().mean().item())
    result = {
        "metric": METRIC, "value": round(value, 3), "unit": "Mpx/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": f"synthetic (seeded scene, seed {args.seed}+rank)",
        "config": dict(workload_config(False), parallelism=f"replicas x{ws}" if ws > 1 else "single GPU"),
        "valid_fraction": round(valid, 4),
    }
    result["stage_ms"] = {"transform": round(stages[0], 4), "search": round(stages[1], 4),
                          "agreement": round(stages[2], 4)}
    # per step: the descriptor transform (which also writes the search's FP8
    # candidate tiles), the tensor-core search, the subpixel sweep
    result["gpu_launches"] = 3 * args.steps

    # per-stage rooflines; the headline one is the stage that takes longest
    result["stage_rooflines"] = stage_rooflines(stages, rows, cols, n, clk, valid)
    dom = max(result["stage_rooflines"], key=lambda k: result["stage_rooflines"][k]["ms"])
    result["roofline"] = dict(result["stage_rooflines"][dom], stage=dom)

    if not args.no_double:
        ms_d, st_d, _ = timed(True, max(1, args.steps // 2), 2, stage_times=True)
        result["double"] = {"value": round(ws * px / (ms_d * 1e-3) / 1e6, 3), "unit": "Mpx/s",
                            "ms_per_step": round(ms_d, 4),
                            "stage_ms": {"transform": round(st_d[0], 4), "search": round(st_d[1], 4),
                                         "agreement": round(st_d[2], 4)},
                            "stage_rooflines": stage_rooflines(st_d, rows, cols, n, clk, valid,
                                                               agree="subpixel_f64")}
        # the moment form (extension): exact integer moments, Sxy on the
        # tensor cores, closed-form sweep of the unrounded interpolant, FP64
        ms_m, st_m, _ = timed(True, max(1, args.steps // 2), 2, stage_times=True, form=1)
        result["moment_form_double"] = {
            "value": round(ws * px / (ms_m * 1e-3) / 1e6, 3), "unit": "Mpx/s", "ms_per_step": round(ms_m, 4),
            "stage_ms": {"transform": round(st_m[0], 4), "search": round(st_m[1], 4),
                         "agreement": round(st_m[2], 4)}}

    if not args.no_configs and ws == 1:
        result["c0_vga"], result["c2_precision"] = config_benches(lbg, pybicos, scenes, timed_match, clk,
                                                                  args.seed, max(5, args.steps // 2))

    if not args.no_learned and N.load().bicos_learned_model_installed():
        # the learned subpixel form (extension): network proposal, one
        # reference NCC check, the reference sweep where the check fails
        ms_l, st_l, out_l = timed(False, args.steps, 2, stage_times=True, form=2)
        result["learned_form"] = {
            "value": round(ws * px / (ms_l * 1e-3) / 1e6, 3), "unit": "Mpx/s", "ms_per_step": round(ms_l, 4),
            "vs_plain_sweep": round(ms / ms_l, 3),
            "stage_ms": {"transform": round(st_l[0], 4), "search": round(st_l[1], 4),
                         "agree_learned": round(st_l[2], 4)},
            "agree_stage_vs_plain_sweep": round(stages[2] / st_l[2], 3),
            # transform, search, sweep offsets, k_learned, the list's sweep
            # (and one cudaMemsetAsync of the list's counters)
            "gpu_launches_per_step": 5,
            "error": learned_error(lbg, pybicos, left, right, out[0], out_l[0], n)}

    if not args.no_batch and ws == 1:
        result["batch"] = batch_bench(lbg, pybicos, scenes, args.seed)
        # many small stacks, where per-call overhead and kernel tails dominate
        rng = np.random.default_rng(args.seed + 7)
        small = [(240, 320, int(rng.choice([8, 12])), 8, bool(rng.random() < 0.5), 0.1 if rng.random() < 0.5 else None)
                 for _ in range(64)]
        sm = batch_bench(lbg, pybicos, scenes, args.seed, rounds=10, specs=small)
        sm.pop("specs")
        result["batch_small_stacks"] = dict(sm, workload="64 stacks 320x240 u8, n in {8, 12}, mixed mode and step")

    if not args.no_e2e:
        # host path: pinned host stacks -> bicos_match_host_v1 (upload, match, download)
        cfg = cfg_of(False)
        nc = cfg.native()
        lh = torch.from_numpy(scene.left).pin_memory().numpy()
        rh = torch.from_numpy(scene.right).pin_memory().numpy()
        dh = torch.empty((rows, cols), dtype=torch.float32).pin_memory().numpy()
        ch = torch.empty((rows, cols), dtype=torch.float32).pin_memory().numpy()
        p0 = (C.c_void_p * n)(*[lh[t].ctypes.data for t in range(n)])
        p1 = (C.c_void_p * n)(*[rh[t].ctypes.data for t in range(n)])
        sptr = C.c_void_p(torch.cuda.current_stream().cuda_stream)

        def host_call():
            N.check(L.bicos_match_host_v1(p0, p1, n, rows, cols, N.BICOS_8U, cols, dh.ctypes.data, cols * 4,
                                          ch.ctypes.data, cols * 4, C.byref(nc), sptr))
        for _ in range(2):
            host_call()
        k_e = max(3, min(args.steps, 20))
        barrier()
        t0 = time.perf_counter()
        for _ in range(k_e):
            host_call()
        t_e = ranks_max((time.perf_counter() - t0) / k_e)
        result["e2e"] = {"value": round(ws * px / t_e / 1e6, 3), "unit": "Mpx/s",
                         "h2d_bytes_per_step": int(2 * n * px), "d2h_bytes_per_step": int(px * 8),
                         "ms_per_step": round(t_e * 1e3, 3), "api": "bicos_match_host_v1 (pinned host buffers)"}

    if rank == 0 and ws == 1 and not args.no_cpu:
        result["cpu_baseline"] = cpu_baseline(scene, args.cpu_seconds)
    result["clocks"] = clk
    if rank == 0:
        print(json.dumps(result), flush=True)
    if ws > 1:
        dist.destroy_process_group()


def run_reference(args):
    rank, _, ws = dist_env()
    if rank != 0:
        return
    from libbicos_gb300 import scenes
    from oracle import oracle as O
    O.build()
    use_ref = O.ref_available()
    scene = scenes.workload_scene(WORKLOAD, seed=args.seed)
    cfg = O.make_config(threshold=THRESHOLD, step=STEP, min_variance=MIN_VAR)
    # each step: a bounded sample of rows, ~1.5 s of CPU work
    rows = cpu_sample_rows(scene, cfg, 1.5, use_ref)
    for _ in range(args.warmup):
        oracle_mpx(scene, rows, cfg, use_ref)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle_mpx(scene, rows, cfg, use_ref)
    dt = (time.perf_counter() - t0) / args.steps
    value = rows * scene.left.shape[2] / dt / 1e6
    cores = os.cpu_count() if use_ref else O.lib().orc_num_threads(0)
    kind = "reference" if use_ref else "port"
    sample = f"rows 0..{rows - 1} of the {WORKLOAD} stack (all columns, n=33) per step" + \
        ("" if use_ref else f"; {PORT_VS_REFERENCE}")
    config = dict(workload_config(False),
                  sample=f"each step matches rows 0..{rows - 1} ({rows} of 1216 rows, all 1936 columns) of the "
                         f"stack on the host cores; Mpx/s = the sample's pixels / its time")
    print(json.dumps({
        "metric": METRIC, "value": round(value, 4), "unit": "Mpx/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(dt * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": f"synthetic (seeded scene, seed {args.seed})",
        "config": config, "impl": "reference",
        "cpu_baseline": {"value": round(value, 4), "unit": "Mpx/s", "cores": cores, "kind": kind, "sample": sample},
        "e2e": {"value": round(value, 4), "unit": "Mpx/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
