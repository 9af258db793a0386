"""Generates tests/golden/oracle_small.npz from the C oracle.

The reference cannot be built here (PETSc/MPI absent) and ships no golden
vectors, so these fixtures freeze the oracle's FP64 results on a 4x2x2
cantilever (seeded density, every objective) for regression and for the GPU
parity tests.  Run:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402


def main():
    rng = np.random.default_rng(1234)
    x = 0.2 + 0.6 * rng.random(16)
    out = {"x": x}
    for obj in range(7):
        le = O.LinearElasticity(4, 2, 2, ncp=2, tsc=3, t1=0.6, objective=obj, loadsignal=1, dalpha=0.01, dbeta=0.01)
        rc, fx, df = le.objective_sensitivities(x)
        assert rc == 0
        out["fx%d" % obj] = fx
        out["df%d" % obj] = df
    KE, ME = O.hex8_ke_me()
    out["KE"] = KE
    out["ME"] = ME
    out["xfilt"] = O.pde_filter(4, 2, 2, x, 2.0)
    np.savez(os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle_small.npz"), **out)


if __name__ == "__main__":
    main()
