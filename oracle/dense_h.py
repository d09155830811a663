"""Dense-Hamiltonian oracle — TEST INFRASTRUCTURE ONLY (never a product path).

Builds the M-scheme Hamiltonian matrix of a generated problem directly from
second quantisation, independently of any index list: every basis Slater
determinant is acted on by every k-body term a+_{b1}..a+_{bk} a_{ak}..a_{a1}
of the synthetic interaction and the result is located in the basis.  Unit-
vector products through the reference Minerva kernels must reproduce this
matrix, which pins the index-list / matrix-element conventions that the
reference only defines through its consumers:

* vector layout — blocks in comb.txt order, element n + Nn*p inside a block
  (src/Minerva/matrix_vector_multiplication/matrix_vector_multiplication.c:58-63);
* orbital order (e, l, j asc, m desc) (src/Neptune/bases/sp_states.c:7-35);
* Slater determinants inside an (E, M) sub-basis in lexicographic order of
  their sorted orbitals;
* the interaction: for every unordered pair {alpha, beta} of k-particle
  states with the same species content, a seeded N(0, sigma) deviate
  (splitmix64 hash + Box-Muller), plus hw * (number of quanta) on the
  diagonal.

Pure-Python loops: intended for small bases (D up to a few thousand).
"""
import math
import itertools

MASK64 = (1 << 64) - 1


def mix64(z):
    z = (z + 0x9E3779B97F4A7C15) & MASK64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
    return z ^ (z >> 31)


def pair_normal(seed, tag, ka, kb):
    lo, hi = min(ka, kb), max(ka, kb)
    h = mix64(seed ^ mix64(tag ^ mix64(lo ^ mix64(hi))))
    h2 = mix64(h)
    u1 = ((h >> 11) + 1.0) * (1.0 / 9007199254740992.0)
    u2 = (h2 >> 11) * (1.0 / 9007199254740992.0)
    return math.sqrt(-2.0 * math.log(u1)) * math.cos(6.283185307179586 * u2)


def orbitals(emax):
    out = []
    for e in range(emax + 1):
        for l in range(e & 1, e + 1, 2):
            for j in (2 * l - 1, 2 * l + 1):
                if j < 0:
                    continue
                for m in range(j, -j - 1, -2):
                    out.append((e, l, j, m))
    out.sort(key=lambda s: (s[0], s[1], s[2], -s[3]))
    return out


def min_energy(n):
    E, e, left = 0, 0, n
    while left > 0:
        c = (e + 1) * (e + 2)
        t = min(c, left)
        E += t * e
        left -= t
        e += 1
    return E


def top_shell(n):
    e, left = 0, n
    if n == 0:
        return 0
    while True:
        c = (e + 1) * (e + 2)
        if left <= c:
            return e
        left -= c
        e += 1


def read_blocks(comb_path):
    """(Ep, Mp, En, Mn, Np, Nn) per basis block, in id order."""
    blocks = []
    section = None
    with open(comb_path) as f:
        for row in f:
            if "***" in row:
                section = "mp" if "mp-states" in row else None
                continue
            if section == "mp" and "ARRAYMP:" in row:
                w = row.split()
                blocks.append((int(w[9].rstrip("=")), int(w[0]), int(w[1]), int(w[2]), int(w[3]),
                               int(w[4]), int(w[5])))
    blocks.sort()
    return [b[1:] for b in blocks]


def species_subbasis(orbs, npart, E, M):
    """Sorted orbital tuples of npart particles with energy E and 2M = M, lexicographic."""
    out = []
    for t in itertools.combinations(range(len(orbs)), npart):
        if sum(orbs[i][0] for i in t) == E and sum(orbs[i][3] for i in t) == M:
            out.append(t)
    return out


def apply_op(occ, alpha, beta):
    """O(beta,alpha)|occ> for a sorted global occupation tuple -> (sign, new sorted tuple) or (0, None)."""
    cur = list(occ)
    sign = 1
    for a in alpha:                      # a_{a1} first
        if a not in cur:
            return 0, None
        pos = cur.index(a)
        if pos & 1:
            sign = -sign
        cur.pop(pos)
    for b in reversed(beta):             # a+_{bk} first
        if b in cur:
            return 0, None
        pos = sum(1 for c in cur if c < b)
        if pos & 1:
            sign = -sign
        cur.insert(pos, b)
    return sign, tuple(cur)


def state_code(orbs_tuple, nsp):
    c = 0
    for o in orbs_tuple:
        c = c * (nsp + 1) + (o + 1)
    return c


def build_dense_h(problem_dir, Z, N, Nmax, nbody=2, seed=20261203, hbar_omega=20.0, sigma2=1.0, sigma3=0.1,
                  me_seed_offset=True):
    import numpy as np

    blocks = read_blocks(f"{problem_dir}/comb.txt")
    emax = max(top_shell(Z), top_shell(N)) + Nmax
    orbs = orbitals(emax)
    nsp = len(orbs)
    # basis in vector order; global orbital ids: proton s -> s, neutron s -> nsp + s
    basis = []
    for (Ep, Mp, En, Mn, Np, Nn) in blocks:
        P = species_subbasis(orbs, Z, Ep, Mp)
        Nb = species_subbasis(orbs, N, En, Mn)
        assert len(P) == Np and len(Nb) == Nn, "sub-basis size mismatch with comb.txt"
        for p in P:
            for n in Nb:
                basis.append(tuple(p) + tuple(nsp + s for s in n))
    index = {s: i for i, s in enumerate(basis)}
    D = len(basis)
    H = np.zeros((D, D))
    A = Z + N

    def seed_for(k):
        return (seed * 1000003 + k) & MASK64

    # term types: (kp, kn)
    types = [(2, 0), (0, 2), (1, 1)]
    if nbody >= 3:
        types += [(3, 0), (0, 3), (2, 1), (1, 2)]
    # all k-particle states per (kp, kn), keyed by total M
    cache = {}

    def states(kp, kn, M):
        key = (kp, kn, M)
        if key not in cache:
            out = []
            for tp in itertools.combinations(range(nsp), kp):
                mp = sum(orbs[i][3] for i in tp)
                ep = sum(orbs[i][0] for i in tp)
                for tn in itertools.combinations(range(nsp), kn):
                    if mp + sum(orbs[i][3] for i in tn) != M:
                        continue
                    out.append((tp, tn, ep + sum(orbs[i][0] for i in tn)))
            cache[key] = out
        return cache[key]

    Emax_total = min_energy(Z) + min_energy(N) + Nmax
    for col, sd in enumerate(basis):
        prot = [o for o in sd if o < nsp]
        neut = [o - nsp for o in sd if o >= nsp]
        E_sd = sum(orbs[o][0] for o in prot) + sum(orbs[o][0] for o in neut)
        H[col, col] += hbar_omega * E_sd
        for (kp, kn) in types:
            if kp > Z or kn > N:
                continue
            sigma = sigma2 if kp + kn == 2 else sigma3
            sd_seed = seed_for(kp + kn)
            span = (nsp + 1) ** kn
            for ap in itertools.combinations(prot, kp):
                for an in itertools.combinations(neut, kn):
                    Ma = sum(orbs[o][3] for o in ap) + sum(orbs[o][3] for o in an)
                    Ea = sum(orbs[o][0] for o in ap) + sum(orbs[o][0] for o in an)
                    ka = state_code(ap, nsp) * span + state_code(an, nsp)
                    alpha = tuple(ap) + tuple(nsp + s for s in an)
                    for (bp, bn, Eb) in states(kp, kn, Ma):
                        if E_sd - Ea + Eb > Emax_total:
                            continue
                        beta = tuple(bp) + tuple(nsp + s for s in bn)
                        sgn, out = apply_op(sd, alpha, beta)
                        if not sgn:
                            continue
                        row = index.get(out)
                        if row is None:
                            continue
                        kb = state_code(bp, nsp) * span + state_code(bn, nsp)
                        v = sigma * pair_normal(sd_seed, kp * 4 + kn, ka, kb)
                        H[row, col] += sgn * v
    return H
