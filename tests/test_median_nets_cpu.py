"""The generated median block networks (csrc/gen_median_nets.py) on the CPU:
the committed header is what the generator writes, and every emitted block
network selects the exact median of each of its windows -- on 0-1 inputs
(the 0-1 principle: a min/max network selects rank m of every input iff it
does so for every 0-1 input; sampled at every density here, exhaustively for
the smallest block), on values with many ties and on distinct values."""
import importlib.util
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GEN = os.path.join(ROOT, "imagefiltering.jl_gb300", "csrc", "gen_median_nets.py")


@pytest.fixture(scope="module")
def gen():
    spec = importlib.util.spec_from_file_location("gen_median_nets", GEN)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def run_network(net, outs, footprint):
    """Evaluate the network on a batch of footprints (trials x rows x cols)."""
    val = {}
    for i, (kind, a, b) in enumerate(net.ops):
        if kind == "in":
            val[i] = footprint[:, a, b]
        elif kind == "lo":
            val[i] = np.minimum(val[a], val[b])
        else:
            val[i] = np.maximum(val[a], val[b])
    return np.stack([np.stack([val[w] for w in row], axis=1) for row in outs], axis=1)


def window_medians(footprint, k, tw, th):
    t = footprint.shape[0]
    out = np.empty((t, th, tw), footprint.dtype)
    for y in range(th):
        for x in range(tw):
            win = footprint[:, y:y + k, x:x + k].reshape(t, -1)
            out[:, y, x] = np.sort(win, axis=1)[:, (k * k - 1) // 2]
    return out


def test_header_is_generated(gen):
    with open(gen.OUT) as f:
        assert f.read() == gen.header(), "ifx_median_nets.cuh differs from the generator's output"


@pytest.mark.parametrize("block", [(3, 4, 2), (5, 4, 2), (5, 4, 1), (5, 2, 2)])
def test_block_selects_median(gen, block):
    k, tw, th = block
    assert block in gen.BLOCKS
    net, outs = gen.block_network(k, tw, th)
    rows, cols = th + k - 1, tw + k - 1
    rng = np.random.default_rng(k * 100 + tw * 10 + th)
    n = rows * cols
    if n <= 24:                                  # every 0-1 footprint
        codes = np.arange(1 << n, dtype=np.int64)
        zo = ((codes[:, None] >> np.arange(n)) & 1).astype(np.int8).reshape(-1, rows, cols)
    else:                                        # 0-1 footprints at every density
        dens = rng.random((200000, 1, 1))
        zo = (rng.random((200000, rows, cols)) < dens).astype(np.int8)
    for fp in (zo, rng.integers(0, 4, (20000, rows, cols)), rng.permutation(
            np.arange(20000 * n)).reshape(20000, rows, cols)):
        got = run_network(net, outs, fp)
        assert np.array_equal(got, window_medians(fp, k, tw, th))


def test_operation_counts(gen):
    """Sharing between the windows of a block: fewer operations per output than
    one pruned 25-input Batcher network per 5 x 5 window (about 200)."""
    per = {}
    for k, tw, th in gen.BLOCKS:
        net, outs = gen.block_network(k, tw, th)
        per[(k, tw, th)] = sum(1 for i in gen.live_ops(net, outs) if net.ops[i][0] != "in") / (tw * th)
    assert per[(5, 4, 2)] < 75 and per[(5, 4, 1)] < 85 and per[(3, 4, 2)] < 19
