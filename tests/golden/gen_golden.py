"""Generates the golden fixtures of tests/golden/ (run in a Python with sympy).

wigner.json      exact 3j (a k b; 0 0 0) and 6j {la lb L; ld lc k} values from
                 sympy.physics.wigner, the arithmetic GSL provides to the
                 reference (src/tools/wigner_tools.f90:30-60), plus a few
                 general-m 3j symbols of the dipole factor (src/mat_els/dipole.f90:25).
gauss_legendre.json  nodes/weights from numpy.polynomial.legendre.leggauss for
                 q = 1..24 (the reference's stdlib gauss_legendre, quad_tools.f90:26).
ragged_problems.json the 64 radial problems of the ragged batch, drawn from
                 numpy.random.default_rng(0) in the order: order k from {6,7,8},
                 N in [100, 500], max_k in [4, 16], channel l_max in [0, 8].
"""
import json
import os

import numpy as np
from sympy.physics.wigner import wigner_3j, wigner_6j

HERE = os.path.dirname(os.path.abspath(__file__))


def ragged():
    rng = np.random.default_rng(0)
    probs = []
    for _ in range(64):
        k = int(rng.choice([6, 7, 8]))
        n = int(rng.integers(100, 501))
        kmax = int(rng.integers(4, 17))
        lmax = int(rng.integers(0, 9))
        probs.append({"k": k, "n_b": n, "r_max": float(n), "k_GL": k + 4, "max_k": kmax,
                      "l_max": lmax})
    with open(os.path.join(HERE, "ragged_problems.json"), "w") as f:
        json.dump(probs, f, indent=0)


def main():
    ragged()
    three = []
    for a in range(0, 11):
        for b in range(0, 11):
            for k in range(0, 21):
                if (a + b + k) % 2 == 0 and abs(a - b) <= k <= a + b:
                    three.append([a, k, b, 0, 0, 0, float(wigner_3j(a, k, b, 0, 0, 0))])
    for L1 in range(0, 6):
        for L2 in range(max(0, L1 - 1), L1 + 2):
            for M1 in range(-L1, L1 + 1):
                for q in (-1, 0, 1):
                    M2 = M1 - q
                    if abs(M2) <= L2:
                        three.append([L1, 1, L2, -M1, q, M2,
                                      float(wigner_3j(L1, 1, L2, -M1, q, M2))])
    six = []
    rng = np.random.default_rng(7)
    seen = set()
    # all small cases, then random larger ones up to l=10, L=5, k=20
    for la in range(0, 3):
        for lb in range(0, 3):
            for lc in range(0, 3):
                for ld in range(0, 3):
                    for L in range(0, 3):
                        for k in range(0, 5):
                            key = (la, lb, L, ld, lc, k)
                            seen.add(key)
                            six.append([*key, float(wigner_6j(*key))])
    nonzero = 0
    while nonzero < 2500:
        la, lb, lc, ld = (int(x) for x in rng.integers(0, 11, 4))
        L = int(rng.integers(0, 6))
        k = int(rng.integers(0, 21))
        key = (la, lb, L, ld, lc, k)
        if key in seen:
            continue
        seen.add(key)
        v = float(wigner_6j(*key))
        if v == 0.0 and rng.random() < 0.95:
            continue
        nonzero += v != 0.0
        six.append([*key, v])
    with open(os.path.join(HERE, "wigner.json"), "w") as f:
        json.dump({"three_j": three, "six_j": six}, f)
    gl = {}
    for q in range(1, 25):
        x, w = np.polynomial.legendre.leggauss(q)
        gl[str(q)] = {"x": x.tolist(), "w": w.tolist()}
    with open(os.path.join(HERE, "gauss_legendre.json"), "w") as f:
        json.dump(gl, f)


if __name__ == "__main__":
    main()
