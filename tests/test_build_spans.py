"""The tree facts the single-scene build's spanning-node pass relies on,
checked on the oracle's trees (CPU only).

The refit takes 512 consecutive sorted leaves per block and forms every node
inside a block; a node whose leaf range crosses a block edge (a spanning
node) gets its box as the union of the edge box at its first leaf (leaves
lo..end of lo's block), the boxes of the whole blocks in between and the edge
box at its last leaf (leaves start of hi's block..hi).  The refit writes those
edge boxes only at the two ends of each maximal block-local node (a node
inside one block whose parent spans), so every spanning node's first leaf
must start such a node, and its last leaf end one."""
import numpy as np
import pytest

from crt import data
from oracle.oracle import OracleScene

BLOCK = 512


def _ranges(nodes, n):
    lo = np.zeros(2 * n - 1, np.int64)
    hi = np.zeros(2 * n - 1, np.int64)
    lo[n - 1:] = hi[n - 1:] = np.arange(n)
    order, stack = [], [0]
    while stack:
        x = stack.pop()
        order.append(x)
        if x < n - 1:
            stack += [nodes[x, 1], nodes[x, 2]]
    for x in reversed(order):
        if x < n - 1:
            lo[x], hi[x] = lo[nodes[x, 1]], hi[nodes[x, 2]]
    return lo, hi


@pytest.mark.parametrize("n,block", [(600, BLOCK), (5000, BLOCK), (20000, BLOCK), (3000, 16), (2049, 64)])
def test_spanning_node_ends_are_maximal_node_ends(n, block):
    m = data.soup(n, seed=n + block)
    ex = OracleScene(m).export()
    nodes = ex["nodes"].reshape(-1, 3)
    boxes = ex["node_boxes"].reshape(-1, 6).astype(np.float64)
    lo, hi = _ranges(nodes, n)
    spans = lo // block != hi // block
    starts, ends = set(), set()
    for x in range(1, 2 * n - 1):
        if not spans[x] and spans[nodes[x, 0]]:  # a maximal block-local node
            starts.add(int(lo[x]))
            ends.add(int(hi[x]))
    leaf = boxes[n - 1:]

    def union(a, b):
        u = leaf[a:b + 1]
        return np.concatenate([u[:, :3].min(0), u[:, 3:].max(0)])

    for x in np.nonzero(spans[:n - 1])[0]:
        assert lo[x] in starts and hi[x] in ends, x
        # the box as the refit assembles it: two edge boxes and whole blocks
        b0, b1 = lo[x] // block, hi[x] // block
        parts = [union(lo[x], min(n, (b0 + 1) * block) - 1), union(b1 * block, hi[x])]
        parts += [union(k * block, (k + 1) * block - 1) for k in range(b0 + 1, b1)]
        p = np.array(parts)
        assert np.array_equal(np.concatenate([p[:, :3].min(0), p[:, 3:].max(0)]), boxes[x]), x
