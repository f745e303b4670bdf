"""Generates tests/golden/bern_draws.npz from the reference's ESS test fixtures.

Reads src/test/unit/analyze/mcmc/test_csv_files/bern{1..4}.csv of the reference
tree (4 chains x 1000 post-warmup draws of the CmdStan bernoulli example) and
keeps the columns its tests use: lp__ (col 0), divergent__ (col 5), theta
(col 7).  Run once where the reference tree is present:

    python tests/golden/make_bern_fixture.py /path/to/stan
"""
import os
import sys

import numpy as np


def main(ref_root):
    cols = {"lp": [], "divergent": [], "theta": []}
    for i in range(1, 5):
        path = os.path.join(ref_root, "src/test/unit/analyze/mcmc/test_csv_files", f"bern{i}.csv")
        rows = []
        with open(path) as f:
            header_seen = False
            for line in f:
                if line.startswith("#") or not line.strip():
                    continue
                if not header_seen:
                    header_seen = True
                    continue
                rows.append([float(v) for v in line.strip().split(",")])
        a = np.array(rows)
        cols["lp"].append(a[:, 0])
        cols["divergent"].append(a[:, 5])
        cols["theta"].append(a[:, 7])
    out = {k: np.stack(v, axis=1) for k, v in cols.items()}  # (1000, 4)
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "bern_draws.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst, {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python make_bern_fixture.py <stan-dev/stan source tree>")
    main(sys.argv[1])
