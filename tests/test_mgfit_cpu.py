"""The V-cycle parameter fit's coordinate search (ofblend_gb300/mgfit.py),
on a synthetic objective instead of GPU solves."""
from ofblend_gb300 import mgfit


class FakeCtx:
    def __init__(self):
        self.params = None

    def set_mg_params(self, *p):
        self.params = p


def _grid_distance(p, target):
    return sum(abs(mgfit.GRID[k].index(p[k]) - mgfit.GRID[k].index(target[k])) for k in target)


def test_fit_finds_the_grid_optimum(monkeypatch):
    target = {"omega0": 0.85, "omegac": 0.95, "lam": 0.7, "coarse_sweeps": 16}

    def evaluate(ctx, data, p, sp):
        it = 100 + 3 * _grid_distance(p, target)
        return it, 1e-3 * it, 0

    monkeypatch.setattr(mgfit, "cases", lambda n, dims, ctx=None: [None] * n)
    monkeypatch.setattr(mgfit, "evaluate", evaluate)
    ctx = FakeCtx()
    best, hist = mgfit.fit(ctx, train=2, max_rounds=3)
    assert best == target
    assert ctx.params == (0.85, 0.95, 0.7, 16)
    assert hist[0][0] == mgfit.START  # the search starts from START


def test_fit_rejects_moves_that_need_the_plain_finisher(monkeypatch):
    """A candidate with fewer iterations whose solves the plain PCG had to
    finish scores worse than any candidate without such solves."""
    bad = {"omega0": 1.0}

    def evaluate(ctx, data, p, sp):
        if p["omega0"] == bad["omega0"]:
            return 50, 0.05, 1
        return 100 + 3 * _grid_distance(p, mgfit.DEFAULT), 0.1, 0

    monkeypatch.setattr(mgfit, "cases", lambda n, dims, ctx=None: [None] * n)
    monkeypatch.setattr(mgfit, "evaluate", evaluate)
    best, _ = mgfit.fit(FakeCtx(), train=1, max_rounds=4)
    assert best == mgfit.DEFAULT


def test_fit_ties_go_to_clearly_faster_candidates(monkeypatch):
    """Equal iteration counts: a move is taken only when it is at least 3%
    faster."""
    def evaluate(ctx, data, p, sp):
        sec = 1.0 - (0.10 if p["coarse_sweeps"] == 8 else 0.0) - (0.01 if p["lam"] == 1.0 else 0.0)
        return 100, sec, 0

    monkeypatch.setattr(mgfit, "cases", lambda n, dims, ctx=None: [None] * n)
    monkeypatch.setattr(mgfit, "evaluate", evaluate)
    best, _ = mgfit.fit(FakeCtx(), train=1, max_rounds=2)
    assert best["coarse_sweeps"] == 8
    assert best["lam"] == mgfit.START["lam"]  # 1% faster is not enough
