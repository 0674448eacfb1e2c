"""Reading the golden fixtures under tests/golden/ (written by
tests/golden/make_golden.py)."""
import hashlib
import json
import os

import numpy as np

import configs as cf

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_all():
    out = []
    for name in sorted(os.listdir(GOLDEN)):
        if name.endswith(".npz"):
            z = np.load(os.path.join(GOLDEN, name))
            case = {k: z[k] for k in z.files}
            case["name"] = name[:-4]
            case["cutoff"] = float(case["cutoff"])
            case["pbc"] = tuple(bool(b) for b in case["pbc"])
            out.append(case)
    return out


def load_digests():
    with open(os.path.join(GOLDEN, "digests.json")) as f:
        return json.load(f)


def digest_input(d):
    """Regenerates the (seeded) input of a digest entry and checks its bits."""
    if d["kind"] == "uniform":
        X, C, _ = cf.rand_config(d["N"], seed=d["seed"])
        pbc = (True, True, True)
    elif d["kind"] == "fcc_sheared":
        X, C, pbc = cf.fcc_sheared(n=d["n"], seed=d["seed"])
    else:
        raise ValueError(d["kind"])
    h = hashlib.sha256(np.ascontiguousarray(X, dtype="<f8").tobytes()).hexdigest()
    assert h == d["input_sha256"], f"generator drift for {d['name']}"
    return X, C, pbc, d["cutoff"]


def digest(out):
    """sha256 over first, i, j, S (int64) and the bits of R, in output order."""
    h = hashlib.sha256()
    for a in (out.first, out.i, out.j, out.S):
        h.update(np.ascontiguousarray(a, dtype="<i8").tobytes())
    h.update(np.ascontiguousarray(out.R, dtype="<f8").tobytes())
    return h.hexdigest()
