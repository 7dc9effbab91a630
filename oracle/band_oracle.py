"""ORACLE (test infrastructure only): the band layout of the plain form's
reduced camera system, restated in numpy.

The reference factors the dense (9C)^2 Schur complement with Eigen's LLT
(src/lm.cu:598-604) whatever the camera graph. The library's band layout
computes the same factor of the same matrix with the cameras renumbered, so
its parity is checked against the reference-pinned oracle step (oracle.py
schur_step) and, here, the renumbering itself: the reverse Cuthill-McKee
ordering (E. Cuthill and J. McKee, 1969; reversed as in A. George, 1971) with
the library's tie-breaking, and the block bandwidth it gives. Only tests/
import this module.
"""
from __future__ import annotations

import numpy as np

TILE = 64


def camera_graph(prob) -> tuple[np.ndarray, np.ndarray]:
    """Distinct camera pairs (a > b) that share a point: the nonzero
    off-diagonal 9 x 9 blocks of S (reference src/lm.cu:522-560 adds one term
    per pair of observations of a point)."""
    order = np.argsort(prob.obs_point, kind="stable")
    pts = prob.obs_point[order]
    cams = prob.obs_camera[order]
    starts = np.flatnonzero(np.r_[True, pts[1:] != pts[:-1]])
    ends = np.r_[starts[1:], len(pts)]
    pairs = set()
    for s, e in zip(starts, ends):
        track = np.unique(cams[s:e])
        for i in range(len(track)):
            for j in range(i):
                pairs.add((int(track[i]), int(track[j])))
    if not pairs:
        return np.zeros(0, np.int64), np.zeros(0, np.int64)
    arr = np.array(sorted(pairs), np.int64)
    return arr[:, 0], arr[:, 1]


def rcm(num_cameras: int, a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """perm[c] = position of camera c. Components are started from the
    unvisited camera of least degree (ties: lower index), neighbours are queued
    in increasing degree (ties: lower index), and the whole order is reversed."""
    C = num_cameras
    deg = np.zeros(C, np.int64)
    np.add.at(deg, a, 1)
    np.add.at(deg, b, 1)
    adj = [[] for _ in range(C)]
    for x, y in zip(a.tolist(), b.tolist()):
        adj[x].append(y)
        adj[y].append(x)
    for c in range(C):
        adj[c].sort(key=lambda v: (deg[v], v))
    seen = np.zeros(C, bool)
    order = []
    for start in sorted(range(C), key=lambda v: (deg[v], v)):
        if seen[start]:
            continue
        head = len(order)
        order.append(start)
        seen[start] = True
        while head < len(order):
            u = order[head]
            head += 1
            for v in adj[u]:
                if not seen[v]:
                    seen[v] = True
                    order.append(v)
    perm = np.empty(C, np.int32)
    perm[np.array(order[::-1])] = np.arange(C, dtype=np.int32)
    return perm


def band_plan(num_cameras: int, a: np.ndarray, b: np.ndarray) -> dict:
    """The ordering (reverse Cuthill-McKee, or the cameras' own order when its
    bandwidth is no larger) and the band storage the library derives from it:
    block bandwidth w (cameras), bt (64-row tiles below the diagonal tile holding
    nonzeros) and ldb = (bt + 2) 64 rows per column."""
    perm = rcm(num_cameras, a, b)
    w = int(np.max(np.abs(perm[a] - perm[b]))) if len(a) else 0
    w_given = int(np.max(np.abs(a - b))) if len(a) else 0
    if w_given <= w:  # the cameras' own order is at least as narrow
        perm, w = np.arange(num_cameras, dtype=np.int32), w_given
    rows = 9 * (w + 1)
    bt = (rows - 1 + TILE - 1) // TILE
    return dict(perm=perm, w=w, bt=bt, ldb=(bt + 2) * TILE)


def to_band(A: np.ndarray, ldb: int) -> np.ndarray:
    """Lower band storage of a symmetric n x n matrix: (i, j), 0 <= i - j <
    ldb, at AB[(i - j) + j ldb]."""
    n = A.shape[0]
    AB = np.zeros(n * ldb)
    for j in range(n):
        m = min(ldb, n - j)
        AB[j * ldb:j * ldb + m] = A[j:j + m, j]
    return AB


def from_band(AB: np.ndarray, n: int, ldb: int, rows: int | None = None) -> np.ndarray:
    """Inverse of to_band for the lower triangle, reading the first `rows`
    rows of each column (default ldb)."""
    rows = ldb if rows is None else rows
    L = np.zeros((n, n))
    for j in range(n):
        m = min(rows, n - j)
        L[j:j + m, j] = AB[j * ldb:j * ldb + m]
    return L
