"""Regenerate tests/golden/unet_wet256.npy on a GB300: the network
parameters that the default bench line trains (the 256^2 / 400-cell wet
monolayer's plain FP64 solves harvested over 320 steps, 7680 samples, 30
epochs on the GPU; the whole pipeline is deterministic, so a rerun gives
the same floats).  Runs `bench.py` once with --save-params and stores the
parameters as float32 (they are FP32 on the device).

    python tests/golden/make_unet_params.py
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def main() -> None:
    with tempfile.TemporaryDirectory() as d:
        txt = os.path.join(d, "params.txt")
        subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--steps", "1", "--warmup", "3",
                        "--no-cpu-baseline", "--save-params", txt], check=True, cwd=ROOT)
        p = np.loadtxt(txt)
    f = p.astype(np.float32)
    assert np.array_equal(f.astype(np.float64), p), "the device parameters are FP32"
    np.save(os.path.join(HERE, "unet_wet256.npy"), f)


if __name__ == "__main__":
    main()
