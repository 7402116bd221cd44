"""Golden outputs of the oracle on reduced versions of the five measured
configurations (plain small / recommended / large, batched, served).

The inputs are regenerated from their seeds by the library's own synthetic
generator (portable arithmetic: identical on x86 and Arm), so a fixture holds
the configuration, hashes of its inputs and the oracle's outputs: palette and
cell Lab, the greedy grid, every chain's final cost, the final grid, the output
image's SHA-256 and the annealing summary.  tests/test_golden.py checks the
oracle (CPU) and the CUDA path (GPU) against these files bit for bit.

    python tests/golden/make_golden.py        # rewrites tests/golden/*.npz
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO / "mosaic-art-rust_gb300"))
sys.path.insert(0, str(REPO))

SEED = 20251203

# name: (target w, h, blobs, materials n, side, mode, grid w, h, max usage, weight, colour, iterations,
#        chains, tile w, h)
SINGLE = {
    "small": (256, 192, 8, 64, 64, 0, 32, 24, 3, 0.25, 0.0, 500, 1, 8, 8),
    "recommended": (480, 360, 32, 200, 64, 1, 20, 15, 3, 0.25, 0.4, 500, 4, 12, 12),
    "large": (640, 480, 64, 300, 32, 0, 40, 30, 8, 0.25, 0.4, 2000, 8, 8, 8),
}
# the batched and served streams: mosaics over one palette, 8 px cells, 8x8 tiles
STREAMS = {
    "batched": dict(n=6, lo=8, hi=40, materials=150, max_usage=4, iterations=500, chains=2, served=False),
    "served": dict(n=4, lo=50, hi=800, materials=200, max_usage=5, iterations=400, chains=4, served=True),
}
CELL_PX, TILE = 8, 8


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def single_case(name: str):
    from mosaic_gpu import job, synth

    (w, h, blobs, n, side, mode, gw, gh, mu, wt, col, it, ch, tw, th) = SINGLE[name]
    cfg = job.JobConfig(name, w, h, blobs, n, side, mode, gw, gh, mu, wt, col, it, ch, tw, th, seed=SEED)
    return [(cfg, job.make_inputs(cfg), 0)]


def stream_cases(name: str):
    from mosaic_gpu import job, synth

    s = STREAMS[name]
    mats = synth.materials(s["materials"], 32, 0, SEED, 2)
    thumbs = synth.thumbnails(mats, TILE, TILE)
    if s["served"]:
        gw, gh = job.served_grids(s["n"], SEED, s["lo"], s["hi"])
    else:
        gw, gh = job.uneven_grids(s["n"], s["lo"], s["hi"], SEED)
    out = []
    for i in range(s["n"]):
        w, h = int(gw[i]) * CELL_PX, int(gh[i]) * CELL_PX
        tgt = synth.target(w, h, 8, SEED, 100 + i)
        cfg = job.JobConfig(f"{name}{i}", w, h, 8, len(mats), 32, 0, int(gw[i]), int(gh[i]), s["max_usage"], 0.25,
                            0.4, s["iterations"], s["chains"], TILE, TILE, seed=SEED)
        out.append((cfg, job.Inputs(cfg, tgt, mats, thumbs), i))  # stream id = position in the stream
    return out


def cases(name: str):
    return single_case(name) if name in SINGLE else stream_cases(name)


def oracle_record(cfg, inp, stream: int, orc) -> dict:
    from dataclasses import asdict

    r = orc.generate(inp, threads=8, stream=stream)
    return {
        "config": np.array(json.dumps(asdict(cfg))),
        "stream": np.int64(stream),
        "target_sha": np.array(sha(inp.target)),
        "materials_sha": np.array(sha(inp.mats.buf)),
        "grid": r["grid"].astype(np.int32),
        "greedy_grid": r["greedy_grid"].astype(np.int32),
        "cell_lab": r["cell_lab"].astype(np.float32),
        "pal_lab": r["pal_lab"].astype(np.float32),
        "chain_res": r["chain_res"].astype(np.float32),
        "image_sha": np.array(sha(r["image"])),
        "image_shape": np.array(r["image"].shape, np.int64),
        "scalars": np.array([r["p"], r["n_resets"], r["best_chain"]], np.int64),
        "costs": np.array([r["initial_cost"], r["final_cost"], r["best_cost"]], np.float32),
    }


def main():
    import oracle.binding as orc

    orc.build_oracle()
    for name in list(SINGLE) + list(STREAMS):
        recs = {}
        for j, (cfg, inp, stream) in enumerate(cases(name)):
            for k, v in oracle_record(cfg, inp, stream, orc).items():
                recs[f"{j}/{k}"] = v
        recs["count"] = np.int64(len(cases(name)))
        path = HERE / f"{name}.npz"
        np.savez_compressed(path, **recs)
        print(f"wrote {path} ({path.stat().st_size} bytes)")


if __name__ == "__main__":
    main()
