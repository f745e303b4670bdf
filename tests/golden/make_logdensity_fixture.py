"""Generates tests/golden/logdensity_exact.npz: log densities of the four
families at seeded points, computed by the extended-precision restatement in
tests/logdensity_exact.py, for the GPU test of the device's FP64 form.

Per dataset <name>: __kind, __X, __y, __group (hierarchical), __J, __hp,
__intercept, __theta (P points), __lp (4 x P: propto/jacobian = 11, 10, 01,
00) and __grad (4 x P x D).  Run from the repository root:

    python tests/golden/make_logdensity_fixture.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from stan_gb300 import workloads  # noqa: E402
from tests import logdensity_exact as exact  # noqa: E402

DATASETS = {
    "logistic_1k": lambda: workloads.logistic(1000, 25, seed=31),
    "logistic_f32": lambda: workloads.logistic(600, 12, seed=32, x_dtype="f32", standardise=True),
    "poisson": lambda: workloads.poisson(800, 16, seed=33, x_dtype="f64"),
    "poisson_bf16": lambda: workloads.poisson(500, 24, seed=34, x_dtype="bf16"),
    "hier_normal": lambda: workloads.hier_normal(40, 4, 12, seed=35),
    "hier_logistic": lambda: workloads.hier_logistic(900, 6, seed=36),
}
POINTS = 4


def main():
    out = {}
    for name, make in DATASETS.items():
        ds = make()
        rng = np.random.default_rng(7)
        th = rng.normal(size=(POINTS, ds.D)) * 0.3
        lps = np.zeros((4, POINTS))
        grads = np.zeros((4, POINTS, ds.D))
        for v, (propto, jac) in enumerate([(1, 1), (1, 0), (0, 1), (0, 0)]):
            for i in range(POINTS):
                lps[v, i], grads[v, i] = exact.for_dataset(ds, th[i], bool(propto), bool(jac))
        out[name + "__kind"] = np.int64(ds.kind)
        out[name + "__X"] = ds.X
        out[name + "__y"] = ds.y
        if ds.group is not None:
            out[name + "__group"] = ds.group.astype(np.int32)
        out[name + "__J"] = np.int64(ds.J)
        out[name + "__hp"] = np.asarray(ds.hp, dtype=np.float64)
        out[name + "__intercept"] = np.int64(1 if ds.intercept else 0)
        out[name + "__xdtype"] = np.array(ds.x_dtype)
        out[name + "__theta"] = th
        out[name + "__lp"] = lps
        out[name + "__grad"] = grads
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "logdensity_exact.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst, os.path.getsize(dst), "bytes")


if __name__ == "__main__":
    main()
