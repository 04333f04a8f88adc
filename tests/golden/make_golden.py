"""Generates the golden vectors in this folder from libBICOS's own CPU backend.

Runs the reference CPU code compiled from its sources (oracle/_ref, built by
oracle/ref_build.sh where the reference tree exists) on small seeded
inputs and stores inputs + outputs as .npz.  Tests check the oracle
restatement and the CUDA path against these files; they need neither the
reference tree nor the _ref build.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from libbicos_gb300 import scenes  # noqa: E402
from oracle import oracle as O  # noqa: E402


def transform_cases(rng):
    out = {}
    i = 0
    for dt in (np.uint8, np.uint16):
        for full in (False, True):
            ns = [2, 3, 4, 5, 9, 10, 17, 18, 33, 34, 65] if not full else [2, 3, 4, 6, 7, 8, 9, 12, 13, 16]
            for n in ns:
                s = rng.integers(0, np.iinfo(dt).max + 1, size=(n, 6, 40), dtype=dt)
                if i % 3 == 0:  # ties and repeated values
                    s = (s % 7).astype(dt)
                nw = O.descriptor_words(O.required_bits(n, full))
                d = O.transform(s, full, nw, use_ref=True)
                out[f"t{i}_stack"] = s
                out[f"t{i}_desc"] = d
                out[f"t{i}_full"] = np.array(int(full))
                i += 1
    return out


def search_cases(rng):
    out = {}
    i = 0
    for nw in (1, 2, 4, 8):
        for flags in (0, 1, 2, 3):
            for lr in (1, 3):
                # 8 random bits per word, as the reference's test does: many ties
                d0 = rng.integers(0, 256, size=(4, 150, nw), dtype=np.uint32)
                d1 = rng.integers(0, 256, size=(4, 150, nw), dtype=np.uint32)
                if i % 2:
                    d0 = d0 | (rng.integers(0, 2**32, size=d0.shape, dtype=np.uint64) & 0xFFFFFF00).astype(np.uint32)
                    d1 = d1 | (rng.integers(0, 2**32, size=d1.shape, dtype=np.uint64) & 0xFFFFFF00).astype(np.uint32)
                out[f"s{i}_d0"] = d0
                out[f"s{i}_d1"] = d1
                out[f"s{i}_flags"] = np.array(flags)
                out[f"s{i}_lr"] = np.array(lr)
                out[f"s{i}_disp"] = O.search(d0, d1, flags, lr, use_ref=True)
                i += 1
    return out


def agree_cases(rng):
    out = {}
    i = 0
    for dt in (np.uint8, np.uint16):
        for step in (None, 0.25, 0.1):
            for mv in (None, 1):
                n = 10
                rows, cols = 12, 96
                s0 = rng.integers(0, np.iinfo(dt).max + 1, size=(n, rows, cols), dtype=dt)
                s1 = rng.integers(0, np.iinfo(dt).max + 1, size=(n, rows, cols), dtype=dt)
                # correlated pairs so thresholds bite both ways
                disp = rng.integers(-1, cols, size=(rows, cols)).astype(np.int16)
                disp[rng.random((rows, cols)) < 0.1] = O.INVALID_I16
                for r in range(rows):
                    for c in range(cols):
                        c1 = c - int(disp[r, c])
                        if disp[r, c] != O.INVALID_I16 and 0 <= c1 < cols and rng.random() < 0.6:
                            s1[:, r, c1] = np.clip(s0[:, r, c].astype(np.int64) + rng.integers(-3, 4, size=n), 0,
                                                   np.iinfo(dt).max).astype(dt)
                thr = float(np.float32(rng.uniform(-0.9, 0.9)))
                minvar = float(np.float32(rng.uniform(0.0, 75.0))) * n if mv else None
                if step is None:
                    d, c = O.agree(disp, s0, s1, thr, minvar, use_ref=True)
                else:
                    d, c = O.agree_subpixel(disp, s0, s1, thr, step, minvar, use_ref=True)
                out[f"a{i}_s0"], out[f"a{i}_s1"], out[f"a{i}_raw"] = s0, s1, disp
                out[f"a{i}_thr"] = np.float32(thr)
                out[f"a{i}_step"] = np.float32(step if step else -1)
                out[f"a{i}_minvar"] = np.float32(minvar if minvar is not None else -1)
                out[f"a{i}_disp"], out[f"a{i}_corr"] = d, c
                i += 1
    return out


def match_cases():
    out = {}
    i = 0
    sc8 = scenes.make_scene(32, 128, 12, seed=7)
    sc16 = scenes.make_scene(24, 112, 12, seed=8, bits=12)
    for sc, label in ((sc8, "u8"), (sc16, "u16")):
        out[f"{label}_left"], out[f"{label}_right"] = sc.left, sc.right
        for full in (False, True):
            for thr, step, mv, cons in ((0.9, None, 2.0, None), (0.5, 0.1, None, None), (0.9, 0.25, 2.0, (1, False)),
                                        (0.75, None, None, (2, True)), (None, None, None, None),
                                        (0.9, 0.5, 2.0, (1, True))):
                cfg = O.make_config(threshold=thr, step=step, min_variance=mv, consistency=cons, full=full)
                d, c = O.match(sc.left, sc.right, cfg, use_ref=True)
                out[f"m{i}_scene"] = np.array(label)
                out[f"m{i}_cfg"] = np.array([thr if thr is not None else np.nan, step if step else np.nan,
                                             mv if mv else np.nan, int(full), -1 if cons is None else cons[0],
                                             0 if cons is None else int(cons[1])], np.float64)
                out[f"m{i}_disp"] = d
                if c is not None:
                    out[f"m{i}_corr"] = c
                i += 1
    return out


def main():
    if not O.ref_available():
        O.build_ref()
    if not O.ref_available():
        raise SystemExit("reference CPU build not available (needs the libBICOS sources)")
    rng = np.random.default_rng(20241203)
    np.savez_compressed(os.path.join(HERE, "transform.npz"), **transform_cases(rng))
    np.savez_compressed(os.path.join(HERE, "search.npz"), **search_cases(rng))
    np.savez_compressed(os.path.join(HERE, "agree.npz"), **agree_cases(rng))
    np.savez_compressed(os.path.join(HERE, "match.npz"), **match_cases())
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
