"""Learned subpixel form: model files, training data and training.

The network (csrc/learned.cu) proposes a match's subpixel offset from the
correlations at the integer disparities d-2..d+2 and the left/right
per-frame variances.  Its training targets are the offsets the reference's
subpixel sweep (include/impl/cuda/agree.cuh:161-259) picks with step 0.01
in double precision, on seeded synthetic scenes; its forward and backward
passes and the Adam update run in the library's own kernels
(bicos_mlp_grad_v1, bicos_mlp_adam_v1), and validation uses the
tensor-core inference kernel the matcher runs (bicos_mlp_propose_v1).

Model file ("BICOSMLP", version 1, little endian): magic, u32 version,
u32 inputs (7), u32 hidden units (64), u32 parameter count, f32 input
means[7], f32 input standard deviations[7], BF16 parameters.

    python -m libbicos_gb300.learned train --out model.bsm
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import struct
import sys
import time

import numpy as np

from . import _native as N

MAGIC = b"BICOSMLP"
VERSION = 1
N_IN, N_H = 7, 64
N_PARAMS = N_H * N_IN + N_H + N_H * N_H + N_H + N_H + 1
MODEL_FLOATS = N_PARAMS + 2 * N_IN
MODEL_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "learned_subpixel.bsm")
LABEL_STEP = 0.01
LABEL_THRESHOLD = 0.5


# ---------------------------------------------------------------- model files

def bf16_bits(a) -> np.ndarray:
    """float32 -> BF16 bit patterns, round to nearest even."""
    b = np.asarray(a, np.float32).view(np.uint32).astype(np.uint64)
    return (((b + 0x7FFF + ((b >> 16) & 1)) >> 16) & 0xFFFF).astype(np.uint16)


def model_bytes(params, mean, std) -> bytes:
    params = np.asarray(params, np.float32)
    if params.shape != (N_PARAMS,):
        raise ValueError(f"expected {N_PARAMS} parameters, got {params.shape}")
    head = MAGIC + struct.pack("<4I", VERSION, N_IN, N_H, N_PARAMS)
    stats = np.concatenate([np.asarray(mean, "<f4"), np.asarray(std, "<f4")]).tobytes()
    return head + stats + bf16_bits(params).astype("<u2").tobytes()


def parse_model(data: bytes):
    """(params as float32, mean, std) of a model file image."""
    if data[:8] != MAGIC:
        raise ValueError("not a BICOSMLP file")
    version, nin, nh, npar = struct.unpack("<4I", data[8:24])
    if version != VERSION or nin != N_IN or nh != N_H or npar != N_PARAMS:
        raise ValueError(f"unsupported model: version {version}, shape {nin}/{nh}/{npar}")
    stats = np.frombuffer(data[24:24 + 8 * N_IN], "<f4")
    bits = np.frombuffer(data[24 + 8 * N_IN:], "<u2")
    if bits.size != N_PARAMS:
        raise ValueError("truncated model file")
    params = (bits.astype(np.uint32) << 16).view(np.float32)
    return params, stats[:N_IN].copy(), stats[N_IN:].copy()


def model_floats(params, mean, std) -> np.ndarray:
    return np.concatenate([np.asarray(params, np.float32), np.asarray(mean, np.float32),
                           np.asarray(std, np.float32)])


def install(data: bytes | None) -> None:
    """Installs a model file image in the library (None: uninstall)."""
    lib = N.load()
    if data is None:
        N.check(lib.bicos_learned_model_v1(None, 0))
        return
    buf = C.create_string_buffer(data, len(data))
    N.check(lib.bicos_learned_model_v1(C.cast(buf, C.c_void_p), len(data)))


def installed_model() -> np.ndarray:
    """The installed model as floats (parameters, means, deviations)."""
    out = np.empty(MODEL_FLOATS, np.float32)
    N.check(N.load().bicos_learned_model_floats_v1(out.ctypes.data_as(C.c_void_p), MODEL_FLOATS))
    return out


# ------------------------------------------------------------ training data

def scene_specs(count: int = 200, seed: int = 1000):
    """Seeded scene parameters around the production workload (1936x1216
    projected-pattern stacks, n about 33): stack depths 24..40, a fifth of
    the scenes 12-bit, per-frame blur and contrast drawn per scene, sensor
    noise 1..3 DN (x4 for 12 bit), disparities 30..250 px."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(count):
        bits = 12 if rng.random() < 0.2 else 8
        n = int(rng.choice([24, 33, 33, 40]))
        specs.append(dict(rows=24, cols=640, n=n, seed=seed + i, bits=bits,
                          sigma=(float(rng.uniform(0.8, 1.2)), float(rng.uniform(1.6, 2.4))),
                          contrast=(float(rng.uniform(0.4, 0.6)), 1.0),
                          noise=float(rng.uniform(1.0, 3.0)) * (4.0 if bits == 12 else 1.0),
                          d_range=(30.0, 250.0)))
    return specs


def scene_samples(sc, device="cuda"):
    """(features with the sweep's offset in the last slot) of one scene's
    interior matches that pass the label threshold, as an (N, 8) float32
    CUDA tensor."""
    import torch

    from . import agree_subpixel, match_device, subpixel_features
    from .pybicos import Config
    left = torch.from_numpy(sc.left).to(device)
    right = torch.from_numpy(sc.right).to(device)
    cfg = Config()
    cfg.nxcorr_threshold = None
    raw, _ = match_device(left, right, cfg)
    sub, _ = agree_subpixel(raw, left, right, LABEL_THRESHOLD, LABEL_STEP, None, double=True)
    feats = subpixel_features(raw, left, right)
    rows, cols = raw.shape
    col1 = torch.arange(cols, device=device)[None, :] - raw.to(torch.int32)
    keep = (feats[..., 7] == 1) & torch.isfinite(sub) & (col1 > 0) & (col1 < cols - 1)
    target = raw.to(torch.float64) - sub.to(torch.float64)
    s = feats.clone()
    s[..., 7] = target.to(torch.float32)
    return s[keep].contiguous()


def make_samples(specs, device="cuda", limit: int | None = None, seed: int = 0):
    import torch

    from .scenes import make_scene
    parts = []
    for sp in specs:
        sc = make_scene(sp["rows"], sp["cols"], sp["n"], seed=sp["seed"], bits=sp["bits"], sigma=sp["sigma"],
                        contrast=sp["contrast"], noise=sp["noise"], d_range=sp["d_range"])
        parts.append(scene_samples(sc, device))
    s = torch.cat(parts)
    if limit is not None and s.shape[0] > limit:
        g = torch.Generator(device="cpu").manual_seed(seed)
        s = s[torch.randperm(s.shape[0], generator=g)[:limit].to(device)].contiguous()
    return s


def input_stats(samples) -> tuple[np.ndarray, np.ndarray]:
    """Means and standard deviations of the network inputs (the kernels'
    input transform, restated in numpy)."""
    f = samples[:, :7].double().cpu().numpy()
    r = np.where(np.isfinite(f[:, :5]), f[:, :5], -1.0)
    x = np.stack([r[:, 2], r[:, 1] - r[:, 2], r[:, 3] - r[:, 2], r[:, 0] - r[:, 2], r[:, 4] - r[:, 2],
                  np.log1p(np.maximum(f[:, 5], 0.0)), np.log1p(np.maximum(f[:, 6], 0.0))], axis=1)
    return x.mean(0).astype(np.float32), np.maximum(x.std(0), 1e-6).astype(np.float32)


# ------------------------------------------------------------------ training

def init_params(seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    p = np.zeros(N_PARAMS, np.float32)
    o = 0
    p[o:o + N_H * N_IN] = rng.normal(0, 1 / math.sqrt(N_IN), N_H * N_IN)
    o += N_H * N_IN + N_H
    p[o:o + N_H * N_H] = rng.normal(0, 1 / math.sqrt(N_H), N_H * N_H)
    o += N_H * N_H + N_H
    p[o:o + N_H] = rng.normal(0, 0.5 / math.sqrt(N_H), N_H)
    return p


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _check(t, name, min_numel=None, row=None):
    """The MLP entry points take bare device pointers and a row count:
    each buffer must be a contiguous float32 CUDA tensor of the size the
    kernel reads or writes."""
    if not t.is_cuda or not t.is_contiguous() or str(t.dtype) != "torch.float32":
        raise ValueError(f"{name}: expected a contiguous float32 CUDA tensor")
    if row is not None and (t.dim() != 2 or t.shape[1] != row):
        raise ValueError(f"{name}: expected (count, {row}) rows, got shape {tuple(t.shape)}")
    if min_numel is not None and t.numel() < min_numel:
        raise ValueError(f"{name}: expected at least {min_numel} floats, got {t.numel()}")


def grad(model, samples, grad_buf, loss_buf, stream=None):
    """Adds the batch's gradient to grad_buf and its loss to loss_buf."""
    import torch
    _check(model, "model", MODEL_FLOATS)
    _check(samples, "samples", row=N_IN + 1)
    _check(grad_buf, "grad_buf", N_PARAMS)
    _check(loss_buf, "loss_buf", 1)
    st = C.c_void_p((stream or torch.cuda.current_stream()).cuda_stream)
    N.check(N.load().bicos_mlp_grad_v1(_ptr(model), _ptr(samples), samples.shape[0], _ptr(grad_buf),
                                       _ptr(loss_buf), st))


def adam(model, grad_buf, m, v, step, lr, scale, stream=None):
    import torch
    for t, name in ((model, "model"), (grad_buf, "grad_buf"), (m, "m"), (v, "v")):
        _check(t, name, N_PARAMS)
    st = C.c_void_p((stream or torch.cuda.current_stream()).cuda_stream)
    N.check(N.load().bicos_mlp_adam_v1(_ptr(model), _ptr(grad_buf), _ptr(m), _ptr(v), step, lr, scale, st))


def propose(model, feats, stream=None):
    """Proposals of the inference kernel for (N, 8) feature rows."""
    import torch
    _check(model, "model", MODEL_FLOATS)
    _check(feats, "feats", row=N_IN + 1)
    out = torch.empty(feats.shape[0], dtype=torch.float32, device=feats.device)
    st = C.c_void_p((stream or torch.cuda.current_stream()).cuda_stream)
    N.check(N.load().bicos_mlp_propose_v1(_ptr(model), _ptr(feats), feats.shape[0], _ptr(out), st))
    return out


def parabola(feats):
    """The offset of the parabola through rho(-1), rho(0), rho(+1) (the
    method without the network), clipped to [-1, 1]; 0 where it has no
    maximum."""
    import torch
    rm, r0, rp = feats[:, 1].double(), feats[:, 2].double(), feats[:, 3].double()
    den = rm - 2 * r0 + rp
    x = torch.where(den < 0, (rm - rp) / (2 * den), torch.zeros_like(den))
    return torch.nan_to_num(x, nan=0.0).clamp(-1, 1).float()


def train(samples, val, epochs: int = 80, batch: int = 4096, lr: float = 3e-3, seed: int = 0, log=print):
    import torch
    dev = samples.device
    mean, std = input_stats(samples)
    model = torch.from_numpy(model_floats(init_params(seed), mean, std)).to(dev)
    g = torch.zeros(N_PARAMS, device=dev)
    m = torch.zeros(N_PARAMS, device=dev)
    v = torch.zeros(N_PARAMS, device=dev)
    loss = torch.zeros(1, device=dev)
    gen = torch.Generator(device=dev).manual_seed(seed)
    count = samples.shape[0]
    per_epoch = (count + batch - 1) // batch
    total = epochs * per_epoch
    step = 0
    history = []
    for ep in range(epochs):
        perm = torch.randperm(count, device=dev, generator=gen)
        loss.zero_()
        for b in range(per_epoch):
            idx = perm[b * batch:(b + 1) * batch]
            chunk = samples.index_select(0, idx)
            grad(model, chunk, g, loss)
            step += 1
            rate = lr * (0.05 + 0.95 * 0.5 * (1 + math.cos(math.pi * step / total)))
            adam(model, g, m, v, step, rate, 1.0 / chunk.shape[0])
        train_rms = math.sqrt(2 * loss.item() / count)
        val_rms = float(torch.sqrt(torch.mean((propose(model, val) - val[:, 7]) ** 2)))
        history.append((ep, train_rms, val_rms))
        log(f"epoch {ep:3d}  train rms {train_rms:.5f}  val rms (bf16 inference) {val_rms:.5f}")
    return model.cpu().numpy(), history


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train", help="train the network and write a model file")
    t.add_argument("--out", required=True)
    t.add_argument("--scenes", type=int, default=200)
    t.add_argument("--samples", type=int, default=2_000_000)
    t.add_argument("--val-scenes", type=int, default=10)
    t.add_argument("--epochs", type=int, default=80)
    t.add_argument("--batch", type=int, default=4096)
    t.add_argument("--lr", type=float, default=3e-3)
    t.add_argument("--seed", type=int, default=0)
    a = ap.parse_args(argv)
    import torch
    t0 = time.time()
    specs = scene_specs(a.scenes + a.val_scenes)
    samples = make_samples(specs[:a.scenes], limit=a.samples, seed=a.seed)
    val = make_samples(specs[a.scenes:])
    torch.cuda.synchronize()
    t1 = time.time()
    params, hist = train(samples, val, a.epochs, a.batch, a.lr, a.seed)
    torch.cuda.synchronize()
    t2 = time.time()
    mean, std = params[N_PARAMS:N_PARAMS + N_IN], params[N_PARAMS + N_IN:]
    data = model_bytes(params[:N_PARAMS], mean, std)
    with open(a.out, "wb") as f:
        f.write(data)
    # validation of the stored (BF16) model through the inference kernel
    p_bf16, mu, sd = parse_model(data)
    stored = torch.from_numpy(model_floats(p_bf16, mu, sd)).to(val.device)
    err = propose(stored, val) - val[:, 7]
    par = parabola(val) - val[:, 7]
    summary = {
        "train_samples": int(samples.shape[0]), "val_samples": int(val.shape[0]),
        "scenes": a.scenes, "val_scenes": a.val_scenes, "epochs": a.epochs, "batch": a.batch,
        "label": f"offset of the reference sweep, step {LABEL_STEP}, double precision, threshold {LABEL_THRESHOLD}",
        "val_rms_network_bf16": float(torch.sqrt(torch.mean(err ** 2))),
        "val_rms_parabola": float(torch.sqrt(torch.mean(par ** 2))),
        "val_rms_integer": float(torch.sqrt(torch.mean(val[:, 7] ** 2))),
        "data_s": round(t1 - t0, 2), "train_s": round(t2 - t1, 2), "history": hist,
    }
    print(json.dumps(summary))
    return 0


if __name__ == "__main__":
    sys.exit(main())
