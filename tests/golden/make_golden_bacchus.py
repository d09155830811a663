"""Writes the Bacchus golden fixtures under tests/golden/ from the REFERENCE's
own eigensolver (oracle/_ref/ref_bacchus, built from the reference sources
by oracle/Makefile): for each case the final eigensystem block (its length
is the Lanczos dimension reached), the lowest eigenvector and the case's
generator and run-file settings.  Run it where the reference tree exists:

    python tests/golden/make_golden_bacchus.py
"""
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

# name -> generator config, run-file settings (lanczos group)
CASES = {
    "bacchus_he4_n4_2b": (dict(Z=2, N=2, nmax=4, nbody=2, M2=0), dict(max_iterations=200, tolerance=1e-6)),
    "bacchus_he4_n4_2b_vec": (dict(Z=2, N=2, nmax=4, nbody=2, M2=0),
                              dict(max_iterations=200, tolerance=1e-4, converge_eigenvectors=True)),
    "bacchus_he4_n2_3b": (dict(Z=2, N=2, nmax=2, nbody=3, M2=0), dict(max_iterations=200, tolerance=1e-6)),
    "bacchus_li6_n2_3b_vec": (dict(Z=3, N=3, nmax=2, nbody=3, M2=2),
                              dict(max_iterations=200, tolerance=1e-5, converge_eigenvectors=True)),
}


def main():
    if not oracle.reference_bacchus_available():
        oracle.build()
    assert oracle.reference_bacchus_available(), "the reference tree is needed to write these fixtures"
    for name, (gen, run) in CASES.items():
        with tempfile.TemporaryDirectory() as tmp:
            d = os.path.join(tmp, name)
            jn.generate(d, basis_files=False, **gen)
            r = oracle.reference_bacchus(d, gen["Z"], gen["N"], **run)
            np.savez_compressed(os.path.join(HERE, f"{name}.npz"), eigenvector=r["eigenvectors"][0])
            meta = dict(config=gen, lanczos=run, num_eigenvalues=r["num_eigenvalues"],
                        eigenvalues=[float(v) for v in r["eigenvalues"]], steps=r["steps"])
            with open(os.path.join(HERE, f"{name}.json"), "w") as f:
                json.dump(meta, f, indent=1, sort_keys=True)
            print(name, r["num_eigenvalues"], r["eigenvalues"][:3])


if __name__ == "__main__":
    main()
