"""Python restatements of the block ILU(0) cuts and of the block-restricted
dependency levels (test helpers shared by the CPU and GPU tests)."""
import numpy as np


def level_counts(IA, JA, blk, lower=True):
    """Dependency levels of each block with the couplings between blocks dropped."""
    n = len(IA) - 1
    lev = np.zeros(n, np.int64)
    order = range(n) if lower else range(n - 1, -1, -1)
    for i in order:
        cols = JA[IA[i]:IA[i + 1]]
        cols = cols[((cols < i) if lower else (cols > i)) & (blk[cols] == blk[i])]
        lev[i] = lev[cols].max() + 1 if cols.size else 0
    return np.array([lev[blk == b].max() + 1 for b in range(blk.max() + 1)])


def level_cut(IA, JA, P):
    """First rows of the default cut: run b starts where the running maximum
    of the full factor's forward level first reaches ceil(b * levels / P)."""
    n = len(IA) - 1
    lev = np.zeros(n, np.int64)
    for i in range(n):
        cols = JA[IA[i]:IA[i + 1]]
        cols = cols[cols < i]
        lev[i] = lev[cols].max() + 1 if cols.size else 0
    run = np.maximum.accumulate(lev)
    nl = int(run[-1]) + 1
    cut = np.zeros(P + 1, np.int64)
    cut[P] = n
    i = 0
    for b in range(1, P):
        fl = (nl * b + P - 1) // P
        while i < n and run[i] < fl:
            i += 1
        cut[b] = i
    for b in range(1, P):
        cut[b] = max(cut[b], cut[b - 1] + 1)
    for b in range(P - 1, 0, -1):
        cut[b] = min(cut[b], cut[b + 1] - 1)
    return cut


def rows_cut(n, P):
    """Equal row counts: row r in run floor(r * P / n)."""
    return np.array([(b * n + P - 1) // P for b in range(P)] + [n], np.int64)


def block_ids(first):
    blk = np.zeros(first[-1], np.int64)
    for b in range(len(first) - 1):
        blk[first[b]:first[b + 1]] = b
    return blk
