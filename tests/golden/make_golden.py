"""Generates tests/golden/exact64.npz from the reference's golden fields.

Source: tutorials/test/exactSolutions/<t>/alpha.water.exact of
daidezhi/geometricVofExt (OpenFOAM binary volScalarField, 64^3 cells in the
case's renumberMesh cell order, "exact" volume fractions of an advected
icosphere at t = 0, 0.25, ..., 3).  The cell order of those files is not
the blockMesh order this project generates, so only permutation-invariant
data is kept:

  times        the 13 sample times
  volume       sum(alpha) * h^3 per time
  n_mixed      cells with 1e-8 < alpha < 1 - 1e-8 per time
  n_full       cells with alpha >= 1 - 1e-8 per time
  sorted_t<k>  the nonzero alpha values sorted ascending, for t = 0, 1.5, 3
  mixed32      the mixed values (1e-8 < alpha < 1 - 1e-8) of every time,
               each time's values sorted ascending, as float32, one run per
               time; mixed32_off[k] .. mixed32_off[k+1] is time k

Run (reads the reference checkout given as the argument):
  python tests/golden/make_golden.py <geometricVofExt checkout>
"""

import os
import re
import sys

import numpy as np

TIMES = ["0", "0.25", "0.5", "0.75", "1", "1.25", "1.5", "1.75", "2", "2.25", "2.5", "2.75", "3"]
SORTED = {"0": "sorted_t0", "1.5": "sorted_t1p5", "3": "sorted_t3"}


def read_of_binary_scalar_field(path):
    b = open(path, "rb").read()
    i = b.index(b"internalField")
    j = b.index(b"(", i)
    n = int(re.search(rb"List<scalar>\s*(\d+)", b[i:j]).group(1))
    return np.frombuffer(b[j + 1:j + 1 + 8 * n], dtype="<f8").copy()


def main(ref_root):
    base = os.path.join(ref_root, "tutorials", "test", "exactSolutions")
    h3 = (1.0 / 64) ** 3
    out = {"times": np.array([float(t) for t in TIMES])}
    vol, nm, nf, mixed = [], [], [], []
    for t in TIMES:
        a = read_of_binary_scalar_field(os.path.join(base, t, "alpha.water.exact"))
        assert a.size == 64 ** 3
        vol.append(float(np.sum(a)) * h3)
        nm.append(int(np.count_nonzero((a > 1e-8) & (a < 1 - 1e-8))))
        nf.append(int(np.count_nonzero(a >= 1 - 1e-8)))
        mixed.append(np.sort(a[(a > 1e-8) & (a < 1 - 1e-8)]).astype(np.float32))
        if t in SORTED:
            out[SORTED[t]] = np.sort(a[a > 0.0])
    out["volume"] = np.array(vol)
    out["n_mixed"] = np.array(nm)
    out["n_full"] = np.array(nf)
    out["mixed32"] = np.concatenate(mixed)
    out["mixed32_off"] = np.concatenate(([0], np.cumsum([m.size for m in mixed]))).astype(np.int64)
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "exact64.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: python tests/golden/make_golden.py <geometricVofExt checkout>")
    main(sys.argv[1])
