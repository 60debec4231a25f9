"""The learned direction selector: its hand-written CUDA forward/backward/Adam
kernels against the CPU oracle, the per-level profiles it trains on, and what
it gains over the Beamer rule. Policies change speed only: every BFS here is
also checked bit for bit against the oracle."""
from __future__ import annotations

import numpy as np
import pytest

import albba_gb300 as ab
import oracle
from albba_gb300 import selector as sel

pytestmark = pytest.mark.gpu

# fp32 kernels with atomic (unordered) gradient sums: relative tolerance
RTOL = 1e-4
ATOL = 1e-5


def rand_problem(seed, batch=300):
    rng = np.random.default_rng(seed)
    p = (rng.standard_normal(oracle.NPARAM) * 0.3).astype(np.float32)
    x = rng.random((batch, 8)).astype(np.float32)
    y = rng.standard_normal((batch, 3)).astype(np.float32)
    m = (rng.random((batch, 3)) > 0.2).astype(np.float32)
    return p, x, y, m


def test_forward_matches_oracle():
    p, x, _, _ = rand_problem(1)
    assert np.allclose(ab.mlp_forward(p, x), oracle.mlp_forward(p, x), rtol=RTOL, atol=ATOL)


@pytest.mark.parametrize("seed", [2, 3, 4])
def test_gradient_matches_oracle(seed):
    p, x, y, m = rand_problem(seed)
    lg, gg = ab.mlp_loss_grad(p, x, y, m)
    lc, gc = oracle.mlp_loss_grad(p, x, y, m)
    assert np.isclose(lg, lc, rtol=RTOL)
    scale = np.abs(gc).max()
    assert np.allclose(gg, gc, rtol=1e-3, atol=1e-5 * scale)


def test_adam_matches_oracle():
    p, x, y, m = rand_problem(5)
    _, g = oracle.mlp_loss_grad(p, x, y, m)
    pg, mg, vg = p.copy(), np.zeros_like(p), np.zeros_like(p)
    pc, mc, vc = p.copy(), np.zeros_like(p), np.zeros_like(p)
    for t in range(1, 4):
        ab.adam_step(pg, g, mg, vg, t, lr=1e-2)
        oracle.adam_step(pc, g, mc, vc, t, lr=1e-2)
    assert np.allclose(pg, pc, rtol=1e-5, atol=1e-6)
    assert np.allclose(mg, mc, rtol=1e-5, atol=1e-7) and np.allclose(vg, vc, rtol=1e-5, atol=1e-9)


def test_training_fits_a_known_rule():
    rng = np.random.default_rng(7)
    x = rng.random((2000, 8)).astype(np.float32)
    # cost of variant k is a simple function of the features
    y = np.stack([4 * x[:, 0] + 1, 4 * x[:, 1] + 1, 2 * x[:, 0] + 2 * x[:, 1] + 1.5], 1).astype(np.float32)
    m = np.ones_like(y)
    p0, loss0 = ab.selector_train(x, y, m, steps=0, seed=1)
    p, loss = ab.selector_train(x, y, m, steps=3000, lr=3e-3, seed=1)
    assert loss < 0.01 * loss0 and loss < 0.02
    acc = np.mean(np.argmin(ab.mlp_forward(p, x), 1) == np.argmin(y, 1))
    assert acc > 0.95


def test_profile_records_are_consistent():
    g = ab.gen_rmat(15, 16, seed=9)
    root = int(g.pick_roots(1, 2)[0])
    lv_ref, pa_ref, nl = oracle.bfs(g.rowptr, g.col, root)
    with ab.Graph(g) as dg:
        dg.sell_build(32, 1024)
        prof = dg.bfs_profile(root)
        assert len(prof) == nl
        assert [p.rec.nf for p in prof] == np.bincount(lv_ref[lv_ref >= 0]).tolist()
        for p in prof:
            assert p.best == int(np.argmin(p.us)) and min(p.us) > 0
        lv, pa, _ = dg.bfs(root)
        assert np.array_equal(lv, lv_ref) and np.array_equal(pa, pa_ref)
        roots = g.pick_roots(64, 3)
        mp = dg.msbfs64_profile(roots)
        assert len(mp) >= 2 and all(p.best == int(np.argmin(p.us)) for p in mp)
        levels, _ = dg.msbfs64(roots)
        ref = np.stack([oracle.bfs(g.rowptr, g.col, int(r))[0] for r in roots], 1)
        assert np.array_equal(levels, ref)


@pytest.fixture(scope="module")
def trained():
    """Plain and batched selectors trained on small RMAT/grid/ER graphs."""
    specs = [{"kind": "rmat", "scale": s, "edgefactor": e, "seed": 500 + i}
             for i, (s, e) in enumerate([(14, 8), (15, 16), (16, 4), (16, 32), (17, 16), (18, 8)])]
    specs += [{"kind": "grid", "rows": 256, "cols": 256, "drop": 0.1, "shortcut_frac": 1e-4,
               "seed": 9}, {"kind": "er", "n": 1 << 17, "mean_degree": 8.0, "seed": 9}]
    out = {}
    for form in ("plain", "batched"):
        data = sel.Profiles()
        for i, sp in enumerate(specs):
            data.extend(sel.profile_graph(sel.make_graph(sp), form, 3, seed=i))
        feat, us, state, group = data.arrays()
        params, loss = sel.train(feat, us, steps=3000)
        out[form] = params
    yield out
    ab.selector_clear(0)
    ab.selector_clear(1)


def test_learned_policy_is_bit_exact(trained):
    ab.selector_load(0, trained["plain"])
    ab.selector_load(1, trained["batched"])
    g = ab.gen_rmat(16, 16, seed=2024)
    roots = g.pick_roots(8, 7)
    with ab.Graph(g) as dg:
        dg.sell_build(32, 1024)
        for r in roots:
            olv, opa, _ = oracle.bfs(g.rowptr, g.col, int(r))
            for loop in ("graph", "persistent", "host"):
                lv, pa, _ = dg.bfs(int(r), ab.bfs_opts("learned", loop))
                assert np.array_equal(lv, olv) and np.array_equal(pa, opa)
        r64 = g.pick_roots(64, 8)
        levels, _ = dg.msbfs64(r64, ab.bfs_opts("learned"))
        ref = np.stack([oracle.bfs(g.rowptr, g.col, int(r))[0] for r in r64], 1)
        assert np.array_equal(levels, ref)


@pytest.mark.parametrize("form", ["plain", "batched"])
def test_selector_gain_over_beamer_on_heldout(trained, form):
    """On a held-out graph the per-level choices of a network trained here (on
    eight small graphs, in seconds) cost at most 5 % more than Beamer's, both
    judged by the same per-level oracle timings, and their regret is within
    the 10 % bound or within 5 points of Beamer's (the levels of this small
    graph take tens of microseconds, where a variant's timing varies by a few
    per cent between runs); the shipped network, trained on 400 graphs, is
    judged on held-out graphs by `python -m albba_gb300.configs selector`."""
    ho = sel.make_graph({"kind": "rmat", "scale": 19, "edgefactor": 16, "seed": 77})
    hp = sel.profile_graph(ho, form, 3, seed=5)
    feat, us, state, group = hp.arrays()
    mlp = sel.regret(us, sel.mlp_choices(trained[form], feat))
    beam = sel.regret(us, sel.beamer_choices(state, group, us.argmin(1)))
    print(form, "mlp", mlp, "beamer", beam)
    assert mlp["chosen_us"] <= 1.05 * beam["chosen_us"]
    assert mlp["total"] <= max(0.10, beam["total"] + 0.05)


def test_selector_gains_over_beamer_where_beamer_misjudges(trained):
    """What the trained network gains over the method without it: on held-out
    RMAT graphs of other edge factors, Beamer's fixed alpha/beta (tuned for
    single-root CPU BFS) picks slow directions for the 64-root batched BFS;
    the network, trained on this GPU's per-level timings (here the small
    training set of the fixture), picks faster ones. Judged by the per-level
    oracle timings of the same run, summed over the held-out graphs; the
    choices change speed only (levels bit-exact, tested above)."""
    mlp_us = beam_us = best_us = 0.0
    for sp in ({"kind": "rmat", "scale": 19, "edgefactor": 8, "seed": 901},
               {"kind": "rmat", "scale": 18, "edgefactor": 32, "seed": 902}):
        g = sel.make_graph(sp)
        feat, us, state, group = sel.profile_graph(g, "batched", 3, seed=5).arrays()
        mlp = sel.regret(us, sel.mlp_choices(trained["batched"], feat))
        beam = sel.regret(us, sel.beamer_choices(state, group, us.argmin(1)))
        print(sp, "mlp", mlp, "beamer", beam)
        mlp_us += mlp["chosen_us"]
        beam_us += beam["chosen_us"]
        best_us += mlp["best_us"]
    # a clear gain (beyond timing noise) over the rule the network replaces
    assert mlp_us < 0.97 * beam_us, (mlp_us, beam_us, best_us)
