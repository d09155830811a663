"""Writes the golden fixtures under tests/golden/ from the REFERENCE itself.

For each small problem the generator writes the reference-format files, the
compiled reference Minerva (oracle/_ref/libref_minerva.so, built from the
reference sources by oracle/Makefile) computes y = H x for a seeded x, and
the fixture stores x, y, the sha256 of every index list and matrix-element
file, and the ten lowest eigenvalues of the dense matrix assembled from
reference products.  Run it where the reference tree exists:

    python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import jupiterncsm_gb300 as jn  # noqa: E402
import oracle  # noqa: E402

CASES = {
    "he4_n2_2b": dict(Z=2, N=2, nmax=2, nbody=2, M2=0),
    "he4_n2_3b": dict(Z=2, N=2, nmax=2, nbody=3, M2=0),
    "li6_n2_3b": dict(Z=3, N=3, nmax=2, nbody=3, M2=2),
}


def digest_dir(d):
    """sha256 over (name, bytes) of every file of each kind, in sorted name order."""
    out = {}
    for sub in ("index_lists", "matrix_elements"):
        h = hashlib.sha256()
        names = sorted(os.listdir(os.path.join(d, sub)))
        for f in names:
            h.update(f.encode())
            h.update(open(os.path.join(d, sub, f), "rb").read())
        out[sub] = h.hexdigest()
        out[f"{sub}_count"] = len(names)
    for f in ("comb.txt", "evaluation_order.txt"):
        out[f] = hashlib.sha256(open(os.path.join(d, f), "rb").read()).hexdigest()
    return out


def main():
    if not oracle.reference_available():
        oracle.build()
    assert oracle.reference_available(), "the reference tree is needed to write golden fixtures"
    for name, c in CASES.items():
        with tempfile.TemporaryDirectory() as tmp:
            d = os.path.join(tmp, name)
            jn.generate(d, basis_files=False, **c)
            ref = oracle.Reference(d, c["Z"], c["N"], threads=1)
            D = ref.dimension
            x = np.random.default_rng(20261203).standard_normal(D)
            y = ref.matvec(x)
            H = np.zeros((D, D))
            for j in range(D):
                e = np.zeros(D)
                e[j] = 1.0
                H[:, j] = ref.matvec(e)
            ref.close()
            w = np.linalg.eigvalsh(0.5 * (H + H.T))[:10]
            np.savez_compressed(os.path.join(HERE, f"{name}.npz"), x=x, y=y, eig=w)
            meta = dict(config=c, dimension=D, files=digest_dir(d))
            with open(os.path.join(HERE, f"{name}.json"), "w") as f:
                json.dump(meta, f, indent=1, sort_keys=True)
            print(name, D, w[:3])


if __name__ == "__main__":
    main()
