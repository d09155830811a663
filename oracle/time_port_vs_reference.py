"""Times the oracle's OpenMP restatement of the product (oracle/minerva_port.c)
against the reference's own compiled kernels (oracle/_ref/libref_minerva.so,
driven by oracle/ref_harness.c) on the same problem, threads and host, and
reports their agreement.  The restatement stands in for the reference as the
CPU arm where the reference tree is absent; this shows how its speed
compares.  Needs oracle/_ref (built by oracle/Makefile from the reference
sources).

    python oracle/time_port_vs_reference.py <problem dir> <Z> <N> [threads] [repeats]
"""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import oracle  # noqa: E402


def main():
    d, Z, N = sys.argv[1], int(sys.argv[2]), int(sys.argv[3])
    threads = int(sys.argv[4]) if len(sys.argv) > 4 else 0
    reps = int(sys.argv[5]) if len(sys.argv) > 5 else 5
    P = oracle.Port(d)
    R = oracle.Reference(d, Z, N, threads=threads)
    D = P.dimension
    x = np.random.default_rng(0).standard_normal(D)
    y = np.zeros(D)
    P.matvec_omp(x, y, R.threads)
    R.matvec(x)
    tp, tr = [], []
    for _ in range(reps):
        y = np.zeros(D)
        tp.append(P.matvec_omp(x, y, R.threads))
        yr = R.matvec(x)
        tr.append(R.seconds)
    diff = float(np.abs(y - yr).max() / np.abs(yr).max())
    print(f"{d}: D={D} threads={R.threads} port {np.median(tp) * 1e3:.1f} ms, reference {np.median(tr) * 1e3:.1f} ms "
          f"(medians of {reps}); port / reference {np.median(tp) / np.median(tr):.2f}; max relative difference {diff:.1e}")
    P.close()
    R.close()


if __name__ == "__main__":
    main()
