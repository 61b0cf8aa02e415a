"""Generate the golden fixtures that pin the oracle (run where the reference
checkout is mounted; the fixtures are committed, this script with them).

Each fixture is a reference-structured problem (drand48 streams, fixed master
seeds, D + 1e3, one U and one V for every level) solved by fastSolver2's own
hsolve (src/tasks/leaf_solve.cc:73-154) compiled verbatim against scipy's
OpenBLAS (oracle/build.py).  Stored: the problem parameters and seeds (the
inputs are regenerated bit-exactly from them by oracle.problems), the solution
x, the leaf LU factors hsolve leaves in K, and the final U region (small
cases) or its column norms and first rows (the 4096-row case).

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402
from oracle import problems as P  # noqa: E402

CASES = [
    # name, leaf, levels, rank, nrhs, full
    ("ref_m16_L2_r3_k1", 16, 2, 3, 1, True),
    ("ref_m64_L3_r8_k1", 64, 3, 8, 1, True),
    ("ref_m32_L3_r4_k5", 32, 3, 4, 5, True),
    ("ref_m256_L4_r16_k1", 256, 4, 16, 1, False),   # the N=4096 leaf-256 rank-16 shape
    ("ref_m400_L2_r10_k1", 400, 2, 10, 1, False),   # the reference's default leaf size
]
MASTER = 20240601


def region(pr):
    N, L, r, k = pr.n, pr.levels, pr.rank, pr.nrhs
    W = np.zeros((N, k + L * r), order="F")
    W[:, :k] = pr.B
    for l in range(L):
        W[:, k + l * r:k + (l + 1) * r] = pr.U[l]
    return W


def main():
    if O.ref_lib() is None:
        sys.exit("the verbatim reference hsolve cannot be built here")
    for name, m, L, r, k, full in CASES:
        pr = P.reference_problem(m, L, r, nrhs=k, master=MASTER)
        K = np.array(pr.K, order="F")
        W = region(pr)
        V = np.array(pr.V[0], order="F")
        O.ref_hsolve(pr.n, k, r, 1 << L, K, W, V)
        out = dict(leaf=m, levels=L, rank=r, nrhs=k, master=MASTER, offset=1000, x=W[:, :k])
        if full:
            out.update(region=W, K=K)
        else:
            out.update(region_colnorms=np.linalg.norm(W, axis=0), region_head=W[:64], K_head=K[:64])
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(name, pr.n, "rel.resid", P.rel_residual(pr, W[:, :k]))


if __name__ == "__main__":
    main()
