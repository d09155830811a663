"""Writes the golden fixtures of the J -> M three-body transform from the REFERENCE itself.

For each small case the generator writes the reference-format inputs (a
combination table with three-body blocks and the Anicre basis files) and a
seeded jjj-coupled three-body interaction in the reference's ASCII format
(jjj/jjj.cnf, jjj/jjj.mat); the reference's own three-body transform
(oracle/_ref/ref_mercury3: the reference's src/Mercury + src/Neptune sources
compiled unchanged, with its ASCII reader) writes the M-scheme three-body
blocks, and the fixture stores every block's elements with the sha256 of
the inputs they were computed from.  Run it where the reference tree exists:

    python tests/golden/make_golden_transform3.py
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
    "transform3_he4_n2": dict(Z=2, N=2, nmax=2, M2=0),
    "transform3_li6_n0": dict(Z=3, N=3, nmax=0, M2=0),
}


def sha(path):
    return hashlib.sha256(open(path, "rb").read()).hexdigest()


def main():
    if not oracle.reference_transform3_available():
        sys.exit("oracle/_ref/ref_mercury3 is missing: run make -C oracle ref where the reference tree exists")
    for name, c in CASES.items():
        with tempfile.TemporaryDirectory() as tmp:
            s = jn.generate(tmp, Z=c["Z"], N=c["N"], nmax=c["nmax"], M2=c["M2"], nbody=3, antoine=True)
            e3 = jn.three_body_energy(os.path.join(tmp, "comb.txt"))
            jn.write_jjj(os.path.join(tmp, "jjj"), s["emax_single"], e3)
            out = os.path.join(tmp, "ref_me3")
            secs = oracle.reference_transform3(os.path.join(tmp, "comb.txt"), os.path.join(tmp, "anicr"), out,
                                               c["Z"], c["N"], s["emax_single"], os.path.join(tmp, "jjj"))
            arrays, headers = {}, {}
            for f in sorted(os.listdir(out)):
                nd_n, nd_p, x = oracle.read_me_file(os.path.join(out, f))
                bid = f.split("_")[0]
                arrays[f"b{bid}"] = x
                headers[bid] = [nd_n, nd_p]
            np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
            meta = dict(case=c, emax_single=s["emax_single"], emax_triple=e3,
                        cnf_sha256=sha(os.path.join(tmp, "jjj", "jjj.cnf")),
                        mat_sha256=sha(os.path.join(tmp, "jjj", "jjj.mat")),
                        comb_sha256=sha(os.path.join(tmp, "comb.txt")), headers=headers,
                        reference_seconds=secs, num_blocks=len(arrays),
                        num_elements=int(sum(len(v) for v in arrays.values())))
            json.dump(meta, open(os.path.join(HERE, name + ".json"), "w"), indent=1, sort_keys=True)
            print(name, meta["num_blocks"], "blocks", meta["num_elements"], "elements")


if __name__ == "__main__":
    main()
