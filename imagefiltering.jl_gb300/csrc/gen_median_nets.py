"""Generate ``ifx_median_nets.cuh``: median networks for blocks of k x k windows.

A thread that computes a block of tw x th outputs of a k x k median filter
reads the (th + k - 1) x (tw + k - 1) input values of the block's footprint and
runs one straight-line network of min/max operations.  The network shares
work between the block's windows:

1. Columns.  For every footprint column the values of each output row's
   window (k values) are sorted, sharing the rows common to several output
   rows: the rows shared by all of them are sorted once and the remaining
   rows are merged in down a binary tree over the output rows.
2. Rows of windows.  For one output row, the windows of outputs x0..x1 share
   the columns x1 .. x0 + k - 1.  Their sorted columns are merged (smallest
   groups first), then the extra columns of each half of the output range are
   merged in down a binary tree, until every output holds the merge of its
   own k columns.
3. Pruning.  A sorted group of t values out of a window of N = k*k values
   whose median has rank m (0-based) can only contribute ranks r with
   m - (N - t) <= r <= m: a value of lower rank has at most N - t values
   joining below it and stays below the median, a value of higher rank stays
   above it.  Such values are dropped, and the dropped-below count is kept, so
   that the median is rank m - dropped of the final group.

Merges are Batcher's odd-even merges of two sorted lists (lists padded to a
power of two with +infinity, whose comparators vanish), sorts are merge sorts
made of them, and only the operations the outputs depend on are emitted.
Every step is a sorting or merging network or a rank argument, so the
network selects the exact median for all inputs (ties included); the tests
run the emitted networks against sorted windows on random and 0-1 inputs.

Run ``python gen_median_nets.py`` to rewrite the header beside this file
(``--check`` only compares).
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "ifx_median_nets.cuh")

# (k, tw, th) blocks emitted into the header
BLOCKS = [(3, 4, 2), (5, 4, 2), (5, 4, 1), (5, 2, 2)]


class Net:
    """A DAG of min/max operations on input wires."""

    def __init__(self):
        self.ops = []              # ("in", r, c) | ("lo"/"hi", a, b)

    def inp(self, r, c):
        self.ops.append(("in", r, c))
        return len(self.ops) - 1

    def cx(self, a, b):
        self.ops.append(("lo", a, b))
        lo = len(self.ops) - 1
        self.ops.append(("hi", a, b))
        return lo, len(self.ops) - 1


def _oem(lo, n, r, out):
    """Batcher's odd-even merge comparators on positions lo..lo+n-1 (n a power of two)."""
    m = r * 2
    if m < n:
        _oem(lo, n, m, out)
        _oem(lo + r, n, m, out)
        for i in range(lo + r, lo + n - r, m):
            out.append((i, i + r))
    else:
        out.append((lo, lo + r))


def merge(net, a, b):
    """Merge sorted wire lists a and b; None stands for +infinity."""
    if not a:
        return list(b)
    if not b:
        return list(a)
    p = 1
    while p < max(len(a), len(b)):
        p *= 2
    v = list(a) + [None] * (p - len(a)) + list(b) + [None] * (p - len(b))
    comps = []
    _oem(0, 2 * p, 1, comps)
    for i, j in comps:
        x, y = v[i], v[j]
        if y is None:
            continue
        if x is None:
            v[i], v[j] = y, None
            continue
        v[i], v[j] = net.cx(x, y)
    out = [w for w in v if w is not None]
    assert len(out) == len(a) + len(b)
    return out


def sort(net, wires):
    if len(wires) <= 1:
        return list(wires)
    h = len(wires) // 2
    return merge(net, sort(net, wires[:h]), sort(net, wires[h:]))


class Group:
    """Sorted wires holding ranks lo .. lo+len-1 of a multiset of `total` values."""

    def __init__(self, wires, lo, total):
        self.wires, self.lo, self.total = wires, lo, total


def prune(g, n, m):
    keep_lo = max(m - (n - g.total), 0)
    wires = [w for i, w in enumerate(g.wires) if keep_lo <= g.lo + i <= m]
    return Group(wires, max(g.lo, keep_lo), g.total)


def gmerge(net, a, b, n, m):
    return prune(Group(merge(net, a.wires, b.wires), a.lo + b.lo, a.total + b.total), n, m)


def tree_merge(net, groups, n, m):
    groups = list(groups)
    if not groups:
        return Group([], 0, 0)
    while len(groups) > 1:
        groups.sort(key=lambda g: g.total)
        a = groups.pop(0)
        b = groups.pop(0)
        groups.append(gmerge(net, a, b, n, m))
    return groups[0]


def block_network(k, tw, th):
    """Network for the medians of a tw x th block of k x k windows.  Returns
    (net, outputs) with outputs[y][x] the wire of output (x, y); input (r, c)
    is footprint row r, column c."""
    net = Net()
    n, m = k * k, (k * k - 1) // 2
    width, height = tw + k - 1, th + k - 1
    x_in = [[net.inp(r, c) for c in range(width)] for r in range(height)]
    cols = {}                                    # (column, output row) -> sorted k values
    for c in range(width):
        col = [x_in[r][c] for r in range(height)]

        def down(a, b, core, rows):
            if a == b:
                cols[(c, a)] = core
                return
            mid = (a + b) // 2
            for lo, hi in ((a, mid), (mid + 1, b)):
                need = set(range(hi, lo + k))
                extra = sorted(need - rows)
                down(lo, hi, merge(net, core, sort(net, [col[r] for r in extra])), need)

        rows = set(range(th - 1, k))
        down(0, th - 1, sort(net, [col[r] for r in sorted(rows)]), rows)
    outs = [[None] * tw for _ in range(th)]
    for y in range(th):
        def across(a, b, grp, have):
            if a == b:
                assert grp.total == n
                outs[y][a] = grp.wires[m - grp.lo]
                return
            mid = (a + b) // 2
            for lo, hi in ((a, mid), (mid + 1, b)):
                need = set(range(hi, lo + k))
                extra = [Group(cols[(c, y)], 0, k) for c in sorted(need - have)]
                g = gmerge(net, grp, tree_merge(net, extra, n, m), n, m) if extra else grp
                across(lo, hi, g, need)

        have = set(range(tw - 1, k))
        across(0, tw - 1, tree_merge(net, [Group(cols[(c, y)], 0, k) for c in sorted(have)], n, m), have)
    return net, outs


def live_ops(net, outs):
    """Indices of the operations the outputs depend on, in order."""
    live = set()
    stack = [w for row in outs for w in row]
    while stack:
        i = stack.pop()
        if i in live:
            continue
        live.add(i)
        kind, a, b = net.ops[i]
        if kind != "in":
            stack += [a, b]
    return sorted(live)


def emit(k, tw, th):
    net, outs = block_network(k, tw, th)
    live = live_ops(net, outs)
    nops = sum(1 for i in live if net.ops[i][0] != "in")
    name = "median%d_block%dx%d" % (k, tw, th)
    lines = ["// %d x %d medians of a %d x %d block of outputs: %d min/max operations (%.1f per output)."
             % (k, k, tw, th, nops, nops / (tw * th)),
             "// in[r][c]: footprint row r, column c; out[y][x]: the median of the window at (x, y).",
             "template <class CX>",
             "__device__ __forceinline__ void %s(const typename CX::T (&in)[%d][%d], typename CX::T (&out)[%d][%d])"
             % (name, th + k - 1, tw + k - 1, th, tw),
             "{",
             "    using T = typename CX::T;"]
    names = {}
    for i in live:
        kind, a, b = net.ops[i]
        if kind == "in":
            names[i] = "in[%d][%d]" % (a, b)
            continue
        v = "v%d" % i
        names[i] = v
        lines.append("    const T %s = CX::%s(%s, %s);" % (v, kind, names[a], names[b]))
    for y in range(th):
        for x in range(tw):
            lines.append("    out[%d][%d] = %s;" % (y, x, names[outs[y][x]]))
    lines.append("}")
    return "\n".join(lines), nops


def header():
    parts = ["// ifx_median_nets.cuh -- generated by gen_median_nets.py; do not edit.",
             "//",
             "// Exact median networks for blocks of k x k windows (see the generator's",
             "// description).  CX supplies the element type T and the two halves of a",
             "// compare-exchange, CX::lo(a, b) = min and CX::hi(a, b) = max in the order",
             "// being selected in (order-preserving integer keys, or 16-bit lanes of",
             "// 8-bit codes, two independent blocks per word).",
             "#pragma once",
             "",
             "namespace ifx {",
             ""]
    for k, tw, th in BLOCKS:
        text, _ = emit(k, tw, th)
        parts += [text, ""]
    parts.append("} // namespace ifx")
    return "\n".join(parts) + "\n"


if __name__ == "__main__":
    text = header()
    if "--check" in sys.argv:
        with open(OUT) as f:
            sys.exit(0 if f.read() == text else 1)
    with open(OUT, "w") as f:
        f.write(text)
    for k, tw, th in BLOCKS:
        print("k=%d block %dx%d: %d ops" % (k, tw, th, emit(k, tw, th)[1]))
