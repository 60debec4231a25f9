"""Bypass statistics of the single-root BFS (alb_level_rec), counted by the
kernels, against a CPU count from the oracle's levels and the exported SELL
layout. The reference records per level how many slices its pull skipped
because every row was visited and how many column blocks its sparse-x
kernel skipped (bfs/src/bfs_SELLCSv2.c:773-818, counted at
bfs/src/bfs_par_kernels.c:192 and 630). Here a bottom-up level skips 32-row
words whose rows are all visited (slice bypass) and stops each row at its
first frontier source or its end (column bypass, counted in 4-column
groups); a top-down level skips pushes onto visited targets. Every count is
a function of the level sets alone, so it is compared exactly."""
from __future__ import annotations

import numpy as np
import pytest

import albba_gb300 as ab
import oracle

pytestmark = pytest.mark.gpu


class Model:
    """The kernels' counting rules restated on the CPU."""

    def __init__(self, g, sell, C_):
        self.n = g.n
        self.C = C_
        self.perm = sell.perm
        self.nwords = (g.n + 31) // 32
        deg = np.diff(g.rowptr)
        rows = np.repeat(np.arange(g.n), deg)
        loops = np.bincount(rows[g.col == rows], minlength=g.n)
        self.ideg_pos = (deg - loops)[self.perm]
        inv = np.empty(g.n, np.int64)
        inv[self.perm] = np.arange(g.n)
        self.inv = inv
        # every position's SELL row: blocks of C rows x w4 entries per slice
        self.blocks = []
        for s in range(sell.nslices):
            lo, hi = int(sell.slice_off[s]), int(sell.slice_off[s + 1])
            w4 = (hi - lo) // C_
            b = sell.col[lo:hi].reshape(w4 // 4, C_, 4).transpose(1, 0, 2).reshape(C_, w4)
            self.blocks.append((s * C_, int(sell.width[s]), b))
        self.g = g

    def level(self, lv, L, dir_):
        """(words_bypassed, rows_scanned, groups_read, groups_bypassed, edges_bypassed)."""
        lvp = lv[self.perm]
        vis = (lvp >= 0) & (lvp <= L) | (self.ideg_pos == 0)
        if dir_ == ab.DIR_TOPDOWN:
            g = self.g
            rows = np.repeat(np.arange(g.n), np.diff(g.rowptr))
            src = lv[rows] == L
            tgt = g.col[src]
            keep = tgt != rows[src]  # self-loops are not pushed
            t = lv[tgt[keep]]
            return 0, 0, 0, 0, int(np.count_nonzero((t >= 0) & (t <= L)))
        bypass = dir_ == ab.DIR_BOTTOMUP
        visw = np.ones(self.nwords * 32, bool)
        visw[: self.n] = vis
        full = visw.reshape(-1, 32).all(axis=1)
        wbyp = int(full.sum()) if bypass else 0
        front = lvp == L
        skipped_word = np.repeat(full if bypass else np.zeros_like(full), 32)[: self.n]
        rows_scanned = read = total = 0
        for p0, wd, b in self.blocks:
            ng = (wd + 3) // 4
            if ng == 0:
                continue
            pos = np.arange(p0, min(p0 + self.C, self.n))
            act = ~vis[pos] & ~skipped_word[pos]
            if not act.any():
                continue
            pos = pos[act]
            blk = b[pos - p0][:, : 4 * ng]
            k = act.sum()
            rows_scanned += int(k)
            total += int(k) * ng
            if bypass:
                stop = (blk == pos[:, None]) | front[blk]
                first = np.where(stop.any(axis=1), stop.argmax(axis=1), 4 * ng)
                read += int(np.minimum(ng, first // 4 + 1).sum())
            else:
                read += int(k) * ng
        return wbyp, rows_scanned, read, total - read, 0


@pytest.fixture(scope="module")
def setup(rmat16):
    g, roots = rmat16
    dg = ab.Graph(g)
    dg.sell_build(32, 1024, 1024)
    model = Model(g, dg.sell_export(), 32)
    yield g, roots, dg, model
    dg.close()


@pytest.mark.parametrize("policy", ["beamer", "bottomup", "bottomup_nobypass", "topdown"])
@pytest.mark.parametrize("loop", ["host", "graph", "persistent"])
def test_bypass_counts_match_cpu_model(setup, policy, loop):
    g, roots, dg, model = setup
    for r in roots[:3]:
        lv, pa, st = dg.bfs(int(r), ab.bfs_opts(policy, loop, trace=True))
        olv, _, _ = oracle.bfs(g.rowptr, g.col, int(r))
        assert np.array_equal(lv, olv)
        tr = dg.level_trace()
        assert len(tr) == st.num_levels
        for t in tr:
            want = model.level(olv, t.level, t.dir)
            got = (t.words_bypassed, t.rows_scanned, t.groups_read, t.groups_bypassed,
                   t.edges_bypassed)
            assert got == want, (policy, loop, int(r), t.level, t.dir, got, want)
        if policy == "bottomup":
            # the reference's pull skips slices once they are fully visited:
            # after the first pull level most words are skipped
            assert any(t.words_bypassed > 0 for t in tr[2:])
            assert any(t.groups_bypassed > 0 for t in tr)
