"""Batch API (bicos_match_batch_v1): stacks of mixed size, depth, input type
and configuration in one CUDA graph with persistent multi-stack launches;
every stack's disparity and corrmap bit-identical to its own
bicos_match_v1 call, on the first (captured) call, on graph replays with new
frame contents, and under every tuning the autotuner may pick."""
import numpy as np
import pytest

import libbicos_gb300 as lbg
from gpu_util import assert_same, dev, host
from libbicos_gb300 import pybicos, scenes

pytestmark = pytest.mark.gpu


def cfg(thr=0.9, step=None, mv=2.0, double=False, full=False, consistency=False, form=0):
    c = pybicos.Config()
    c.nxcorr_threshold = thr
    c.subpixel_step = step
    c.min_variance = mv
    c.precision = pybicos.Double if double else pybicos.Single
    c.mode = pybicos.Full if full else pybicos.Limited
    if consistency:
        c.variant = pybicos.Variant.Consistency(max_lr_diff=2, no_dupes=True)
    c.nxcorr_form = form
    return c


# (rows, cols, n, bits, seed, config)
SPECS = [
    (48, 200, 12, 8, 1, cfg()),
    (40, 256, 20, 12, 2, cfg(0.8, 0.1, double=True)),
    (32, 160, 8, 8, 3, cfg(0.5, 0.1, full=True)),
    (40, 300, 33, 8, 4, cfg(0.9, None, consistency=True)),
    (24, 128, 12, 12, 5, cfg(None, full=True)),
    (40, 300, 16, 8, 6, cfg(0.9, 0.25, double=True, form=1)),
    (40, 320, 20, 8, 7, cfg(0.5, 0.1, form=2)),
    (30, 200, 65, 8, 8, cfg(0.6, 0.1)),
    (36, 260, 24, 12, 9, cfg(0.7, None, double=True)),
    (20, 96, 40, 8, 10, cfg(0.5, 0.1, mv=None)),
]


def make_jobs(cuda, seed_shift=0):
    jobs, host_scenes = [], []
    for rows, cols, n, bits, seed, c in SPECS:
        sc = scenes.make_scene(rows, cols, n, seed=seed + seed_shift, bits=bits, d_range=(5.0, 60.0))
        jobs.append((dev(sc.left, cuda), dev(sc.right, cuda), c))
        host_scenes.append(sc)
    return jobs, host_scenes


def assert_same_as_sequential(jobs, outs):
    for k, ((l, r, c), (d, corr)) in enumerate(zip(jobs, outs)):
        wd, wc = lbg.match_device(l, r, c)
        assert_same(host(d), host(wd), f"job {k} disparity")
        if wc is None:
            assert corr is None
        else:
            assert_same(host(corr), host(wc), f"job {k} corrmap")


def test_batch_equals_sequential(cuda):
    jobs, _ = make_jobs(cuda)
    b = lbg.Batch()
    outs = b.match(jobs)
    assert b.captures == 1
    assert_same_as_sequential(jobs, outs)


def test_batch_replay_with_new_frames(cuda):
    import torch
    jobs, _ = make_jobs(cuda)
    b = lbg.Batch()
    outs = b.match(jobs)
    # new frame contents in the same buffers: the captured graph replays
    new_jobs, _ = make_jobs(cuda, seed_shift=100)
    for (l, r, _), (nl, nr, _) in zip(jobs, new_jobs):
        l.copy_(nl)
        r.copy_(nr)
    b.match(jobs, outs)
    torch.cuda.synchronize()
    assert b.captures == 1
    assert_same_as_sequential(jobs, outs)


def test_batch_autotune_and_fixed_tunings(cuda):
    jobs, _ = make_jobs(cuda)
    b = lbg.Batch()
    outs = b.match(jobs)
    chosen = b.autotune(jobs, outs)
    assert chosen["transform_block"] in (64, 128, 256) and chosen["branches"] in (1, 2, 4)
    assert_same_as_sequential(jobs, b.match(jobs, outs))
    for t in ({"transform_block": 64, "ctas_per_sm": 1, "claim": 1, "branches": 1, "persistent": 3},
              {"transform_block": 256, "ctas_per_sm": 32, "claim": 64, "branches": 3, "persistent": 1},
              {"transform_block": 128, "ctas_per_sm": 4, "claim": 2, "branches": 2, "persistent": 0}):
        b.set_tuning(t)
        assert_same_as_sequential(jobs, b.match(jobs, outs))


def test_batch_errors_name_the_item(cuda):
    jobs, _ = make_jobs(cuda)
    b = lbg.Batch()
    bad = list(jobs)
    l, r, _ = bad[1]
    bad[1] = (l, r, cfg(0.5, 0.1, full=True))  # FULL with n = 20 needs 363 bits
    with pytest.raises(ValueError, match="batch item 1: input stacks too large"):
        b.match(bad)
    assert b.captures == 0
    with pytest.raises(ValueError, match="batch tuning out of range"):
        b.set_tuning({"transform_block": 100, "ctas_per_sm": 1, "claim": 1, "branches": 1, "persistent": 3})


def test_batch_single_item_and_streams(cuda):
    import torch
    jobs, _ = make_jobs(cuda)
    b = lbg.Batch()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        outs = b.match(jobs[:1], stream=s)
    s.synchronize()
    assert_same_as_sequential(jobs[:1], outs)
