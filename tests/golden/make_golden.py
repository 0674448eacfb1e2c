"""Writes the golden fixtures of tests/golden/ from the CPU oracle.

The oracle is first pinned against the reference's known answers by
tests/test_oracle.py; these fixtures then freeze its exact output bits
(i, j, S, R, first) on small inputs, and sha256 digests on two larger ones,
so that every machine (x86 here, aarch64 on the GPU host) must reproduce them.

Run from the repository root:  python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(HERE)), "oracle"))

import configs as cf  # noqa: E402
import golden_io  # noqa: E402
import oracle as orc  # noqa: E402


def save(name, X, cell, pbc, rc):
    out = orc.neighbour_list(X, rc, cell, pbc)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), X=np.asarray(X, dtype=np.float64), cell=cell,
                        pbc=np.array(pbc, dtype=bool), cutoff=np.float64(rc), i=out.i, j=out.j, S=out.S,
                        first=out.first, R=out.R)
    print(name, out.npairs)


def main():
    X, C = cf.diamond_primitive()
    save("diamond_rc6", X, C, (True, True, True), 6.0)
    X, C = cf.fcc_cubic(3.61, (2, 2, 2))
    save("fcc_cu_2x2x2_rc3.5", X, C, (True, True, True), 3.5)
    X = np.array([[0.0, 0.0, 0.0], [0.0, 0.0, 2.0], [0.0, 10.0, 0.0]])
    save("h3_isolated", X, np.diag(X.max(0) - X.min(0) + 1), (False, False, False), 5.0)
    X, C = cf.rand_config_triclinic(80, seed=3)
    save("triclinic_80_pbc_TFT", X, C, (True, False, True), 3.0)
    L = 8.0
    save("issue6_fp_boundary", np.array([[0.5, L - 0.3, 0.5], [0.5, -5e-17 * L, 0.5]]), np.diag([L] * 3),
         (True, True, True), 1.5)
    X, C, pbc = cf.fcc_sheared(n=4, seed=1)
    save("fcc_sheared_n4", X, C, pbc, 5.0)
    X, C, L = cf.rand_config(200, seed=12)
    idx = np.arange(1, 201)
    X = X + np.stack([(idx % 3) - 1, ((idx + 1) % 3) - 1, ((idx + 2) % 3) - 1], 1) * L
    save("outside_box_200", X, C, (True, True, True), 5.0)

    digests = []
    for d in ({"name": "uniform_10k_rc5", "kind": "uniform", "N": 10000, "seed": 0, "cutoff": 5.0},
              {"name": "fcc_sheared_32k_rc5", "kind": "fcc_sheared", "n": 20, "seed": 0, "cutoff": 5.0}):
        if d["kind"] == "uniform":
            X, C, _ = cf.rand_config(d["N"], seed=d["seed"])
            pbc = (True, True, True)
        else:
            X, C, pbc = cf.fcc_sheared(n=d["n"], seed=d["seed"])
        d["input_sha256"] = hashlib.sha256(np.ascontiguousarray(X, dtype="<f8").tobytes()).hexdigest()
        out = orc.neighbour_list(X, d["cutoff"], C, pbc, nthreads=8)
        d["npairs"] = int(out.npairs)
        d["sha256"] = golden_io.digest(out)
        digests.append(d)
        print(d["name"], d["npairs"])
    with open(os.path.join(HERE, "digests.json"), "w") as f:
        json.dump(digests, f, indent=1)


if __name__ == "__main__":
    main()
