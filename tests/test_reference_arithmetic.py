"""How far the oracle's defined arithmetic is from the reference's own.

The oracle (and the CUDA path, bit for bit) defines two things the reference
leaves to its FP32 arithmetic and libraries:
  * Lab means: per-pixel Lab from a transfer table and the library's own cube
    root, summed exactly in fixed point; the reference folds palette's FP32
    per-pixel Lab sequentially in FP32 and divides once (lib.rs:99-118);
  * the annealing acceptance exp(-delta/T): the library's own exp; the
    reference calls f32::exp, the C library's expf (optimizer.rs:81).
Here the oracle runs each configuration both ways (orc_job.ref_arith) and the
test counts what changes downstream: Lab (ΔE), k-nearest candidate lists,
greedy cells, final cells, and -- on the same start grid, so that only the exp
differs -- annealing chains.  Configurations: the five golden fixtures' reduced
configurations and the small, recommended and large workloads at full size.
Run with -s to print the table.
"""
import sys
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(GOLDEN))

CASES = ["small", "recommended", "large", "batched", "served", "full:small", "full:recommended", "full:large"]


def _inputs(name):
    from mosaic_gpu import job

    if name.startswith("full:"):
        cfg = job.WORKLOADS[name[5:]]
        return [(cfg, job.make_inputs(cfg), 0)]
    import make_golden as mg

    return mg.cases(name)


def _candidates(orc, pal, cells):
    idx, _ = orc.nearest_n(pal, cells, min(100, pal.shape[0]))
    return idx


@pytest.mark.parametrize("name", CASES)
def test_reference_arithmetic_gap(built, orc, name):
    rows = []
    for cfg, inp, stream in _inputs(name):
        d = orc.generate(inp, threads=8, stream=stream, want_image=False)
        r = orc.generate(inp, threads=8, stream=stream, want_image=False, ref_arith=True)
        assert d["p"] == r["p"]
        de_pal = float(np.linalg.norm(d["pal_lab"].astype(np.float64) - r["pal_lab"], axis=1).max())
        de_cell = float(np.linalg.norm(d["cell_lab"].astype(np.float64) - r["cell_lab"], axis=1).max())
        cand_d = _candidates(orc, d["pal_lab"], d["cell_lab"])
        cand_r = _candidates(orc, r["pal_lab"], r["cell_lab"])
        cand_diff = int((cand_d != cand_r).any(axis=1).sum())
        greedy_diff = int((d["greedy_grid"] != r["greedy_grid"]).sum())
        final_diff = int((d["grid"] != r["grid"]).sum())
        # the exp alone: every chain from the defined greedy grid, defined Lab
        chains_diff, chains = 0, 0
        if cfg.enable_optimization and cfg.weight > 0 and cfg.chains > 0:
            for c in range(cfg.chains):
                g1, res1, n1 = orc.anneal(d["pal_lab"], d["greedy_grid"], cfg.iterations, seed=cfg.seed,
                                          stream=stream, chain=c)
                g2, res2, n2 = orc.anneal(d["pal_lab"], d["greedy_grid"], cfg.iterations, seed=cfg.seed,
                                          stream=stream, chain=c, libm_exp=True)
                chains += 1
                chains_diff += int(not (np.array_equal(g1, g2) and np.array_equal(n1, n2)))
        n = cfg.grid_w * cfg.grid_h
        rows.append((cfg.name, n, d["p"], de_pal, de_cell, cand_diff, greedy_diff, final_diff, chains_diff, chains))
        # the gap is the reference fold's own rounding: its FP32 running sums of
        # 49 152- and 65 536-pixel materials drift up to ~1e-3 from FP64, while
        # the defined means stay within 1e-5 (test_oracle_kat.py); a sanity bound
        assert de_pal <= 1e-2 and de_cell <= 1e-2, rows[-1]
    for (nm, n, p, dp, dc, cd, gd, fd, xd, xc) in rows:
        print(f"{nm:>14} cells {n:6d} P {p:5d}  dE pal {dp:.2e} cell {dc:.2e}  candidate lists {cd:5d}  "
              f"greedy cells {gd:5d}  final cells {fd:5d}  chains (exp only) {xd}/{xc}")
