"""Double-double references for large single permanents (the C2 workload at
n = 26, 28, 30), written to tests/golden/c2_dd_large.json.

The C2 workload is 64 output patterns per size n on a seeded Haar unitary of
2n modes with the input in the first n modes (bench.py: haar_unitary(2n,
seed + n), c2_patterns(n, 64, seed + n)); the oracle's double-double
permanent costs ~2^n on the host (about 80 s at n = 26, 6 min at n = 28 and
25 min at n = 30 on 8 x86 cores), so the values are computed once here and
the GPU tests and the benchmark compare against them.  Each record keeps the
pattern and the matrix's first entry, so a change of the generators is
detected rather than silently compared.

    python tests/golden/make_c2_dd.py            # all records
    python tests/golden/make_c2_dd.py 26 28      # only these sizes
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

SEED = 2026
PATTERNS = {26: (0, 1), 28: (0, 1), 30: (0,)}
OUT = os.path.join(HERE, "c2_dd_large.json")


def main(sizes):
    import bench
    from oracle import oracle as O
    from theboss_gb300.utilities import haar_unitary

    O.build()
    records = json.load(open(OUT)) if os.path.exists(OUT) else []
    keep = [r for r in records if r["n"] not in sizes]
    for n in sizes:
        U = haar_unitary(2 * n, SEED + n)
        T = bench.c2_patterns(n, 64, SEED + n)
        S = np.zeros_like(T)
        S[:, :n] = 1
        for k in PATTERNS[n]:
            hi, lo = O.perm_dd(U, S[k], T[k])
            keep.append({"n": n, "seed": SEED + n, "pattern": k, "U00": [U[0, 0].real, U[0, 0].imag],
                         "T": T[k].tolist(), "dd": [hi.real, hi.imag, lo.real, lo.imag]})
            print(n, k, hi, lo, flush=True)
            json.dump(sorted(keep, key=lambda r: (r["n"], r["pattern"])), open(OUT, "w"), indent=1)


if __name__ == "__main__":
    main([int(a) for a in sys.argv[1:]] or sorted(PATTERNS))
