"""Writes the golden fixtures of the J -> M transform from the REFERENCE itself.

For each small case the generator writes the reference-format inputs with a
seeded J-scheme interaction in the Antoine format (antoine_2nf.bin), the
reference's own two-body transform (oracle/_ref/ref_mercury, the reference's
src/Mercury + src/Neptune sources compiled unchanged) writes the M-scheme
matrix-element blocks, and the fixture stores every block's elements with
the sha256 of the inputs it was computed from.  Run it where the reference
tree exists:

    python tests/golden/make_golden_transform.py
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
    "transform_he4_n2": dict(Z=2, N=2, nmax=2, M2=0),
    "transform_li6_n2": dict(Z=3, N=3, nmax=2, M2=2),
}


def sha(path):
    return hashlib.sha256(open(path, "rb").read()).hexdigest()


def main():
    if not oracle.reference_transform_available():
        sys.exit("oracle/_ref/ref_mercury is missing: run make -C oracle ref where the reference tree exists")
    for name, c in CASES.items():
        with tempfile.TemporaryDirectory() as tmp:
            s = jn.generate(tmp, Z=c["Z"], N=c["N"], nmax=c["nmax"], M2=c["M2"], nbody=2, antoine=True)
            out = os.path.join(tmp, "ref_me")
            secs = oracle.reference_transform(os.path.join(tmp, "comb.txt"), os.path.join(tmp, "anicr"), out, c["Z"],
                                              c["N"], s["emax_single"], s["emax_pair"],
                                              os.path.join(tmp, "antoine_2nf.bin"))
            arrays, headers = {}, {}
            for f in sorted(os.listdir(out)):
                nd_n, nd_p, x = oracle.read_me_file(os.path.join(out, f))
                bid = f.split("_")[0]
                arrays[f"b{bid}"] = x
                headers[bid] = [nd_n, nd_p]
            np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
            meta = dict(case=c, emax_single=s["emax_single"], emax_pair=s["emax_pair"],
                        antoine_sha256=sha(os.path.join(tmp, "antoine_2nf.bin")),
                        comb_sha256=sha(os.path.join(tmp, "comb.txt")), headers=headers,
                        reference_seconds=secs, num_blocks=len(arrays),
                        num_elements=int(sum(len(v) for v in arrays.values())))
            json.dump(meta, open(os.path.join(HERE, name + ".json"), "w"), indent=1, sort_keys=True)
            print(name, meta["num_blocks"], "blocks", meta["num_elements"], "elements")


if __name__ == "__main__":
    main()
