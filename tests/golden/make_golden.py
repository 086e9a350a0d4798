"""Copy the reference's data fixtures used as golden inputs.

    python tests/golden/make_golden.py <GIGA-Lens checkout>/src/gigalens/assets

Writes psf.npy (the TinyTim F140W PSF, 13x13) and demo.npy (the 60x60
observed image of the demo lens) from ``src/gigalens/assets/`` of GIGA-Lens,
and prints their sha256.  The demo's true parameters are in
tests/helpers.py (``demo_truth``).
"""
import hashlib
import os
import sys

import numpy as np

if len(sys.argv) != 2:
    sys.exit("usage: make_golden.py <path to GIGA-Lens src/gigalens/assets>")
SRC = sys.argv[1]
HERE = os.path.dirname(os.path.abspath(__file__))

for name in ("psf.npy", "demo.npy"):
    a = np.load(os.path.join(SRC, name))
    np.save(os.path.join(HERE, name), a)
    print(name, a.dtype, a.shape, hashlib.sha256(open(os.path.join(HERE, name), "rb").read()).hexdigest())
