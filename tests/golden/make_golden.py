"""Copy the reference's data fixtures used as golden inputs.

Run in a container where the reference is mounted; writes psf.npy (the
TinyTim F140W PSF, 13x13) and demo.npy (the 60x60 observed image of the demo
lens) from ``src/gigalens/assets/`` of GIGA-Lens, and prints their sha256.
The demo's true parameters are in tests/helpers.py (``demo_truth``).
"""
import hashlib
import os
import sys

import numpy as np

SRC = sys.argv[1] if len(sys.argv) > 1 else "/root/reference/src/gigalens/assets"
HERE = os.path.dirname(os.path.abspath(__file__))

for name in ("psf.npy", "demo.npy"):
    a = np.load(os.path.join(SRC, name))
    np.save(os.path.join(HERE, name), a)
    print(name, a.dtype, a.shape, hashlib.sha256(open(os.path.join(HERE, name), "rb").read()).hexdigest())
