"""Generates tests/golden/order7_n200_counts.json: the CPU oracle's row counts
and count_nnz (H and S non-zeros; hamiltonian.f90:348-416) of every symmetry
block of the order-7, N=200 workload (exp-linear knots to r_max=200, k=0..10,
l_max=5, L=0..3 with natural parity, singlet and triplet, full blocks).  The
GPU tests compare the library's counts of the same blocks with these.  Takes
a few minutes (the oracle counts row by row):

    python tests/golden/gen_fullsize_counts.py
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402

WL = dict(k=7, n_b=200, r_max=200.0, q=10, max_k=10, l_max=5, max_L=3)


def main():
    out = {"workload": "order 7, N=200, r_max=200, k=0..10, l_max=5, L=0..3 natural parity, "
                       "singlet+triplet, full blocks", "blocks": []}
    t0 = time.time()
    for spin in (0, 1):
        for L in range(WL["max_L"] + 1):
            par = L % 2
            cf = O.count_configs(L, par, WL["l_max"], WL["n_b"], WL["k"], spin=spin)
            nH, nS = O.count_nnz(cf, L, WL["k"], WL["max_k"], True, spin)
            out["blocks"].append({"L": L, "parity": par, "spin": spin, "rows": int(cf.size),
                                  "nnz_H": int(nH), "nnz_S": int(nS)})
            print(out["blocks"][-1], round(time.time() - t0, 1), flush=True)
    with open(os.path.join(HERE, "order7_n200_counts.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
