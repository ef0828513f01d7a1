"""Regenerates the golden films in this directory from the CPU oracle (replay mode).

    python tests/golden/make_golden.py

Each film is the oracle's FP64 render of a seeded synthetic scene with Philox-keyed paths,
single-threaded and with brute-force traversal, so it is reproducible bit for bit. The GPU
parity tests compare the plain FP64 GPU path against these files, and test_oracle_kat checks
that the oracle still reproduces them.
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from nanogi_gb300 import scenegen  # noqa: E402
from oracle.oracle import OracleScene  # noqa: E402

CASES = [
    {"scene": "cornell_box", "renderer": "pt", "width": 20, "height": 16, "spp": 16, "max_vertices": 8, "seed": 21},
    {"scene": "cornell_box", "renderer": "ptdirect", "width": 20, "height": 16, "spp": 16, "max_vertices": 8,
     "seed": 22},
    {"scene": "material_box", "renderer": "pt", "width": 16, "height": 16, "spp": 16, "max_vertices": 12, "seed": 23},
    {"scene": "material_box", "renderer": "ptdirect", "width": 16, "height": 16, "spp": 16, "max_vertices": 12,
     "seed": 24},
    {"scene": "area_sensor_box", "renderer": "ptdirect", "width": 12, "height": 12, "spp": 16, "max_vertices": -1,
     "seed": 25},
]


def main() -> None:
    out = []
    for c in CASES:
        desc = scenegen.WORKLOADS[c["scene"]]()
        o = OracleScene.from_desc(desc, c["width"] / c["height"])
        n = c["width"] * c["height"] * c["spp"]
        film = o.render(c["renderer"], num_samples=n, max_vertices=c["max_vertices"], width=c["width"],
                        height=c["height"], seed=c["seed"], rng_mode="replay", use_bvh=False, threads=1)
        fn = f"{c['scene']}_{c['renderer']}_{c['width']}x{c['height']}_{c['spp']}spp.npy"
        np.save(HERE / fn, film)
        out.append({**c, "num_samples": n, "file": fn, "mean": film.mean(axis=(0, 1)).tolist()})
        print(fn, film.mean(axis=(0, 1)))
    (HERE / "films.json").write_text(json.dumps({"generator": "tests/golden/make_golden.py", "cases": out},
                                                indent=1) + "\n")


if __name__ == "__main__":
    main()
