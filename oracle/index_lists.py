"""Index-list restatement — TEST INFRASTRUCTURE ONLY.

Rebuilds, in plain Python, every index list a combination table names, from
the basis conventions alone, so that the generator's binary
``index_list_<id>`` files can be checked byte for byte:

* Slater determinants of one species in an (E, M) sub-basis in lexicographic
  order of their sorted orbitals; orbitals ordered (e, l, j asc, m desc)
  (src/Neptune/bases/sp_states.c:7-35);
* k-particle states of energy E ordered by M, then lexicographically — the
  ``basis_energy_<E>`` order Mercury walks when it numbers connections
  (src/Mercury/connection_list/connection_list.c:448-498);
* for each determinant (list order), each k-subset alpha of energy `depth`
  (lexicographic), each beta of energy depth+dE and M(alpha)+dM (file order):
  the record {in, out, connection | sign<<31}
  (src/Minerva/index_triple/index_triple.h:6-11, sign bit as in
  src/Aurora/index_list/index_list.c:55-56).
"""
import itertools
import struct

from .dense_h import apply_op, min_energy, orbitals, top_shell


def conn_lists(comb_path):
    out, sec = [], None
    with open(comb_path) as f:
        for row in f:
            if "***" in row:
                sec = "cl" if "Conn lists" in row else None
                continue
            if sec == "cl" and "ARRAY:" in row:
                w = row.split()
                out.append(dict(type=w[0], Ein=int(w[1]), Min=int(w[2]), Eout=int(w[3]), Mout=int(w[4]),
                                depth=int(w[5]), length=int(w[6]), id=int(w[9].rstrip("="))))
    return out


class Builder:
    def __init__(self, Z, N, Nmax):
        self.emax = max(top_shell(Z), top_shell(N)) + Nmax
        self.orbs = orbitals(self.emax)
        self.npart = {"p": Z, "n": N}
        Etot = min_energy(Z) + min_energy(N) + Nmax
        self.kmax_energy = max(Etot - min_energy(N), Etot - min_energy(Z))
        self._sub = {}
        self._kst = {}

    def E(self, t):
        return sum(self.orbs[i][0] for i in t)

    def M(self, t):
        return sum(self.orbs[i][3] for i in t)

    def subbasis(self, npart, E, M):
        key = (npart, E, M)
        if key not in self._sub:
            self._sub[key] = [t for t in itertools.combinations(range(len(self.orbs)), npart)
                              if self.E(t) == E and self.M(t) == M]
        return self._sub[key]

    def kstates(self, k, E):
        """basis_energy_<E> order: sorted by M, then lexicographic."""
        key = (k, E)
        if key not in self._kst:
            st = [t for t in itertools.combinations(range(len(self.orbs)), k) if self.E(t) == E]
            st.sort(key=lambda t: (self.M(t), t))
            self._kst[key] = st
        return self._kst[key]

    def build(self, spec):
        k = len(spec["type"])
        npart = self.npart[spec["type"][0]]
        dE, dM, depth = spec["Eout"] - spec["Ein"], spec["Mout"] - spec["Min"], spec["depth"]
        ins = self.subbasis(npart, spec["Ein"], spec["Min"])
        outs = {t: i for i, t in enumerate(self.subbasis(npart, spec["Eout"], spec["Mout"]))}
        alphas = self.kstates(k, depth)
        betas = self.kstates(k, depth + dE)
        # connection numbering: alpha in file order, then the betas with M(alpha)+dM
        by_m = {}
        for b in betas:
            by_m.setdefault(self.M(b), []).append(b)
        offset, acc = {}, 0
        for a in alphas:
            offset[a] = acc
            acc += len(by_m.get(self.M(a) + dM, []))
        rank = {}
        for lst in by_m.values():
            for r, b in enumerate(lst):
                rank[b] = r
        recs = []
        for i, sd in enumerate(ins):
            for a in itertools.combinations(sd, k):
                if self.E(a) != depth:
                    continue
                for b in by_m.get(self.M(a) + dM, []):
                    sgn, out = apply_op(sd, a, b)
                    if not sgn or out not in outs:
                        continue
                    mi = offset[a] + rank[b]
                    if sgn < 0:
                        mi |= 0x80000000
                    recs.append(struct.pack("<iiI", i, outs[out], mi))
        return b"".join(recs)
