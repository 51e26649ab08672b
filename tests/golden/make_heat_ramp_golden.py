"""Golden outputs of the reference's get_heatmap_colour (src/tracer.cpp:25-45)
for tests/golden/heat_ramp.npz.  Run on x86-64 where the reference tree
exists, after `make -C oracle ref`:

    python tests/golden/make_heat_ramp_golden.py

The inputs: the normalised values of every box-test count 0..1000 (count /
200), the six stops and their float neighbours, values just outside [0, 1],
and 4,000 seeded uniform values in [0, 1].  The outputs are the reference's
float colours, computed by its own function (-ffp-contract=off build).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402


def inputs():
    counts = np.arange(0, 1001, dtype=np.float32) / np.float32(200)
    stops = np.array([0.0, 0.2, 0.4, 0.6, 0.8, 1.0], np.float32)
    near = np.concatenate([np.nextafter(stops, np.float32(-1)), np.nextafter(stops, np.float32(2))])
    edges = np.array([-1.0, -0.0, 1e-30, 0.999999, 1.0000001, 3.5], np.float32)
    rnd = np.random.default_rng(17).random(4_000).astype(np.float32)
    return np.concatenate([counts, stops, near, edges, rnd]).astype(np.float32)


def main():
    if not O.ref_available("b8"):
        raise SystemExit("reference not built: run `make -C oracle ref` first")
    x = inputs()
    rgb = O.ref_heatmap_colour(x, "b8")
    path = os.path.join(HERE, "heat_ramp.npz")
    np.savez_compressed(path, x=x, rgb=rgb)
    print(path, os.path.getsize(path))


if __name__ == "__main__":
    main()
