"""Regenerate the golden fixtures of tests/golden from the reference's own code.

noise_gradients.npz holds seeded noise volumes and the RGBA (quantised gradient, noise) that
the reference's gradient.cpp (computeGradients -> filterGradients -> quantizeGradients, both the
SOBEL 1 default and the SOBEL 0 central-difference branch) produces for them, packed as
NoiseDataSet::createTexture does.  The reference is compiled from its sources by
oracle/build_ref.sh; run this script where the reference checkout is available:

    python tests/golden/make_golden.py [reference-root]
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyoracle  # noqa: E402
from vectorvisualization_gb300 import capi, workloads as wl  # noqa: E402

CASES = [
    # name, (mx, my, mz), kind, seed, slice distances
    ("dense_11x13x17", (11, 13, 17), "dense", 3, (1.0, 1.0, 1.0)),
    ("sparse_24", (24, 24, 24), "sparse", 7, (1.0, 1.0, 1.0)),
    ("dense_16_aniso", (16, 16, 16), "dense", 9, (1.0, 0.5, 2.0)),
    ("tiny_3x4x5", (3, 4, 5), "dense", 11, (1.0, 1.0, 1.0)),
]


def main(argv):
    ref_root = argv[1] if len(argv) > 1 else None
    cmd = ["sh", os.path.join(ROOT, "oracle", "build_ref.sh")] + ([ref_root] if ref_root else [])
    subprocess.run(cmd, check=True)
    out = {}
    for name, dims, kind, seed, sd in CASES:
        noise = wl.dense_noise(dims, seed) if kind == "dense" else wl.sparse_noise(dims, seed)
        out[f"{name}/noise"] = noise
        out[f"{name}/slice_dist"] = np.asarray(sd, np.float32)
        for mode, tag in ((capi.NOISE_GRAD_SOBEL, "sobel"), (capi.NOISE_GRAD_CENTRAL, "central")):
            out[f"{name}/{tag}"] = pyoracle.ref_noise_gradients(noise, mode, sd)
    np.savez_compressed(os.path.join(HERE, "noise_gradients.npz"), **out)
    print("wrote", os.path.join(HERE, "noise_gradients.npz"), len(out), "arrays")


if __name__ == "__main__":
    main(sys.argv)
