"""Why the device's GUI scoring is the GUI generator's choice, on the CPU.

The device keeps one walk (the CLI's decision rule, main.rs:335-475: for each
cell in row-major order, the first strict minimum of list distance + penalty
over the eligible candidates, then the usage reset and the two fallbacks) and,
under MG_SCORING_GUI, hands it candidate lists whose distances are the square
roots of the squared ones (k_scan.cu sqrt_inplace_kernel).  Here that rule is
restated in Python over explicit lists, fed the square-rooted lists of the
oracle's k-nearest search, and compared with the oracle's GUI placement
(gui/app_full.rs:1396-1568, orc_place_greedy_gui) cell for cell; fed the
squared lists it must give the oracle's CLI placement.
"""
import numpy as np
import pytest


def walk(orc, pal, cells, gw, gh, max_usage, weight, idx, dist):
    """The CLI decision rule over given candidate lists (float32 scores)."""
    p = len(pal)
    usage = np.zeros(p, np.int64)
    grid = -np.ones((gh, gw), np.int32)
    resets = 0
    k = idx.shape[1]

    def can_place(t, x, y):
        for nx, ny in ((x - 1, y), (x + 1, y), (x, y - 1), (x, y + 1)):
            if 0 <= nx < gw and 0 <= ny < gh and grid[ny, nx] == t:
                return False
        return True

    for y in range(gh):
        for x in range(gw):
            c = y * gw + x
            best, best_score = -1, np.float32(0)
            for j in range(k):
                t = int(idx[c, j])
                if usage[t] >= max_usage or not can_place(t, x, y):
                    continue
                pen = np.float32(orc.penalty(pal, grid, t, x, y, weight)) if weight > 0 else np.float32(0)
                score = np.float32(dist[c, j]) + pen
                if best < 0 or score < best_score:
                    best, best_score = t, score
            if best < 0:
                resets += 1
                usage[:] = 0
                best = next((int(t) for t in idx[c] if can_place(int(t), x, y)), int(idx[c, 0]))
            usage[best] += 1
            grid[y, x] = best
    return grid, resets


def _rand_lab(rng, n):
    lab = np.empty((n, 3), np.float32)
    lab[:, 0] = rng.uniform(0, 100, n)
    lab[:, 1:] = rng.uniform(-80, 80, (n, 2))
    return lab


@pytest.mark.parametrize("p,gw,gh,max_usage,weight,step", [
    (60, 6, 9, 2, 1.0, 3.0), (150, 12, 10, 1, 0.3, 3.0), (400, 16, 12, 2, 5.0, 0.5), (800, 20, 10, 3, 2.0, 0.05),
    (300, 14, 9, 2, 0.0, 1.0)])
def test_square_rooted_lists_give_the_gui_choice(orc, p, gw, gh, max_usage, weight, step):
    rng = np.random.default_rng(p + gw * 7 + int(weight * 10))
    pal = _rand_lab(rng, p)
    base = _rand_lab(rng, 1)[0]
    cells = (base + np.cumsum(rng.normal(0, step, (gw * gh, 3)), axis=0)).astype(np.float32)
    idx, dist = orc.nearest_n(pal, cells, 100)
    gui, gui_resets = orc.place_greedy(pal, cells, gw, gh, max_usage, weight, gui=True)
    cli, cli_resets = orc.place_greedy(pal, cells, gw, gh, max_usage, weight)
    g, r = walk(orc, pal, cells, gw, gh, max_usage, weight, idx, np.sqrt(dist))
    assert np.array_equal(g, gui) and r == gui_resets
    g, r = walk(orc, pal, cells, gw, gh, max_usage, weight, idx, dist)
    assert np.array_equal(g, cli) and r == cli_resets
    if weight >= 2.0:
        assert not np.array_equal(gui, cli)  # the case separates the two scorings
