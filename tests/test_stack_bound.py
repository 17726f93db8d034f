"""The wide-node stack of the kNN and radius traversals cannot overflow.

A step enters up to four wide nodes (one per group of 8 lanes) and pushes
their internal children; the next step pops four entries only while the stack
has room for their children and for a depth-first descent below them (7
entries per wide level), else one.  This is a host model of that rule
(constants as in datatransferkit_gb300/csrc/dtk_search.cu: STACK = 256,
NODE_GROUPS = 4, WIDE = 8), run on the worst case for the stack: trees in
which every node passes the bound, complete or with random fan-out, up to
36 wide levels.  No GPU is involved.
"""
import random

STACK, NODE_GROUPS, WIDE = 256, 4, 8


def take(sp, levels):
    return NODE_GROUPS if sp + (NODE_GROUPS + levels) * (WIDE - 1) <= STACK else 1


def traverse(children, levels, max_steps=15_000):
    """Largest stack size seen; children(node) lists the internal children."""
    stack, nodes, peak = [], [(0, 0)], 0
    for _ in range(max_steps):
        for n in nodes:
            stack.extend(children(n))
            assert len(stack) <= STACK, (levels, len(stack))
        peak = max(peak, len(stack))
        t = min(take(len(stack), levels), len(stack))
        if t == 0:
            break
        nodes = [stack.pop() for _ in range(t)]
    return peak


def test_complete_trees_never_overflow():
    for levels in range(0, 37):
        def children(n, levels=levels):
            lvl, _ = n
            return [(lvl + 1, c) for c in range(WIDE)] if lvl < levels else []
        peak = traverse(children, levels)
        assert peak <= STACK
        if levels <= 6:  # shallow trees (8M uniform points: 6 levels) keep taking four nodes
            assert all(take(s, levels) == NODE_GROUPS for s in range(0, peak - WIDE + 1))


def test_random_trees_never_overflow():
    rng = random.Random(7)
    for _ in range(80):
        levels = rng.randint(1, 36)
        fan = {}

        def children(n, levels=levels):
            lvl, key = n
            if lvl >= levels:
                return []
            if n not in fan:
                fan[n] = [(lvl + 1, rng.random()) for _ in range(rng.randint(0, WIDE))]
            return fan[n]
        traverse(children, levels)
