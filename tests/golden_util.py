"""Loading of the golden vectors in tests/golden (made by tests/golden/make_golden.py
from the reference's own src/fluid.cpp)."""
import glob
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def cases():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def clamp_cases():
    """Cases of the reference's clamp mode (golden/clamp)."""
    return sorted("clamp/" + os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "clamp", "*.npz")))


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(str(z["meta"]))
    arrays = {k: z[k] for k in z.files if k != "meta"}
    return meta, arrays


def c0_digests():
    with open(os.path.join(GOLDEN, "c0_256_it40_digests.json")) as f:
        return json.load(f)
