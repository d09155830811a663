"""The oracle — TEST INFRASTRUCTURE ONLY.

CPU restatements of the reference's hot path and a driver for the compiled
reference itself.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg use this package, always as the checker, never as the path
being measured or shipped.

* ``Port``       plain-C restatement of the Minerva kernels (minerva_port.c)
* ``Reference``  the reference's own Minerva code, compiled unchanged into
                 _ref/libref_minerva.so when the reference tree is present
* ``dense_h``    independent second-quantisation dense Hamiltonian
* ``index_lists`` Python restatement of index-list construction
* ``jt_transform`` Python restatement of the coupled basis, exact
                 Clebsch-Gordan coefficients and the Antoine file layout
* ``reference_tool``  the reference's aurora.x, mars.x and vulcan.x, compiled
                 unchanged into _ref/ when the reference tree is present
* ``reference_transform``  the reference's own two-body J -> M transform,
                 compiled unchanged into _ref/ref_mercury (with a stand-in
                 for the absent wigxjpf library) when the reference tree is
                 present
* ``reference_transform3``  the reference's own three-body J -> M transform
                 with its ASCII J-scheme reader (_ref/ref_mercury3)
* ``reference_bacchus``  the reference's own Bacchus eigensolver
                 (_ref/ref_bacchus): its Lanczos, tridiagonal solver and
                 eigensystem output on the same files
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference tree the recipes under oracle/ compile from: JNCSM_REFERENCE, else the Makefile's default
REFERENCE = os.environ.get("JNCSM_REFERENCE", "/root/reference")


def reference_tree_present():
    return os.path.isdir(os.path.join(REFERENCE, "src"))

PORT_LIB = os.path.join(HERE, "_build", "libminerva_port.so")
REF_LIB = os.path.join(HERE, "_ref", "libref_minerva.so")
REF_MERCURY = os.path.join(HERE, "_ref", "ref_mercury")
REF_MERCURY3 = os.path.join(HERE, "_ref", "ref_mercury3")
REF_BACCHUS = os.path.join(HERE, "_ref", "ref_bacchus")


def build():
    subprocess.run(["make", "-s", "-C", HERE, "all", f"REFERENCE={REFERENCE}"], check=True)


REF_TOOLS = {name: os.path.join(HERE, "_ref", name) for name in ("aurora", "mars", "vulcan")}


def reference_tool_available(name):
    return os.path.exists(REF_TOOLS[name])


def reference_tool(name, *args):
    """Run the reference program `name` (aurora, mars or vulcan) with args; returns the completed process.

    The programs write <name>.log into their working directory, so they run in
    a scratch directory; relative paths in args are made absolute first."""
    import tempfile
    args = [os.path.abspath(a) if isinstance(a, str) and os.path.exists(a) else str(a) for a in args]
    with tempfile.TemporaryDirectory() as wd:
        return subprocess.run([REF_TOOLS[name], *args], capture_output=True, text=True, cwd=wd)


def reference_available():
    return os.path.exists(REF_LIB)


def reference_transform_available():
    return os.path.exists(REF_MERCURY)


def reference_transform(comb, index_list_dir, output_dir, Z, N, e1, e2, antoine, include_kinetic=True):
    """Run the reference's two-body transform; returns its wall time in seconds."""
    os.makedirs(output_dir, exist_ok=True)
    r = subprocess.run([REF_MERCURY, comb, index_list_dir, output_dir, str(Z), str(N), str(e1), str(e2), antoine,
                        "0" if include_kinetic else "1"], capture_output=True, text=True, check=True)
    return float(r.stdout.split()[-1])


def reference_transform3_available():
    return os.path.exists(REF_MERCURY3)


def reference_transform3(comb, index_list_dir, output_dir, Z, N, e_single, jscheme_dir):
    """Run the reference's three-body transform (ASCII J-scheme input); returns its wall time in seconds.

    It writes a log file into its working directory, so it runs in a scratch directory."""
    import tempfile
    os.makedirs(output_dir, exist_ok=True)
    args = [os.path.abspath(a) for a in (comb, index_list_dir, output_dir)]
    with tempfile.TemporaryDirectory() as wd:
        r = subprocess.run([REF_MERCURY3, *args, str(Z), str(N), str(e_single), os.path.abspath(jscheme_dir)],
                           capture_output=True, text=True, check=True, cwd=wd)
    return float(r.stdout.split()[-1])


def read_me_file(path):
    """(n_dim, p_dim, elements) of a <id>_matrix_elements file."""
    raw = open(path, "rb").read()
    nd_n, nd_p = np.frombuffer(raw[:16], dtype=np.uint64)
    return int(nd_n), int(nd_p), np.frombuffer(raw[16:], dtype=np.float64).copy()


class Port:
    """Single-threaded (or OpenMP task-farm) restatement of run_matrix_vector_multiplication."""
    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            L = ctypes.CDLL(PORT_LIB)
            L.port_open.restype = ctypes.c_void_p
            L.port_open.argtypes = [ctypes.c_char_p] * 4
            L.port_matvec.argtypes = [ctypes.c_void_p] * 3
            L.port_matvec_omp.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int]
            L.port_matvec_omp.restype = ctypes.c_double
            L.port_dimension.restype = ctypes.c_size_t
            L.port_dimension.argtypes = [ctypes.c_void_p]
            L.port_close.argtypes = [ctypes.c_void_p]
            cls._lib = L
        return cls._lib

    def __init__(self, d, order=None):
        e = lambda s: s.encode()
        order = order or f"{d}/evaluation_order.txt"
        self.h = self.lib().port_open(e(f"{d}/comb.txt"), e(order), e(f"{d}/index_lists"),
                                      e(f"{d}/matrix_elements"))
        if not self.h:
            raise RuntimeError(f"oracle port could not open {d}")
        self.dimension = self.lib().port_dimension(self.h)

    def matvec(self, x, y=None):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.dimension) if y is None else y
        self.lib().port_matvec(self.h, x.ctypes.data, y.ctypes.data)
        return y

    def matvec_omp(self, x, y, threads=0):
        """y += H x with the reference's OpenMP task farm; returns seconds of the kernel region."""
        return self.lib().port_matvec_omp(self.h, x.ctypes.data, y.ctypes.data, int(threads))

    def close(self):
        if self.h:
            self.lib().port_close(self.h)
            self.h = None


class Reference:
    """The compiled reference Minerva (in-memory kernels and the file-level scheduler)."""
    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            L = ctypes.CDLL(REF_LIB)
            L.ref_mem_open.restype = ctypes.c_void_p
            L.ref_mem_open.argtypes = [ctypes.c_char_p] * 5 + [ctypes.c_int] * 3
            L.ref_mem_matvec.restype = ctypes.c_double
            L.ref_mem_matvec.argtypes = [ctypes.c_void_p] * 3
            L.ref_mem_dimension.restype = ctypes.c_size_t
            L.ref_mem_dimension.argtypes = [ctypes.c_void_p]
            L.ref_mem_threads.argtypes = [ctypes.c_void_p]
            L.ref_mem_close.argtypes = [ctypes.c_void_p]
            L.ref_matvec_files.argtypes = [ctypes.c_char_p] * 6 + [ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                                                   ctypes.c_int]
            cls._lib = L
        return cls._lib

    def __init__(self, d, Z, N, threads=0):
        self.d, self.Z, self.N = d, Z, N
        zero = write_zero_vectors(d)
        e = lambda s: s.encode()
        self.h = self.lib().ref_mem_open(e(f"{d}/comb.txt"), e(f"{d}/evaluation_order.txt"), e(f"{d}/index_lists"),
                                         e(f"{d}/matrix_elements"), e(zero), Z, N, int(threads))
        self.dimension = self.lib().ref_mem_dimension(self.h)
        self.threads = self.lib().ref_mem_threads(self.h)

    def matvec(self, x, y=None):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.dimension) if y is None else y
        self.seconds = self.lib().ref_mem_matvec(self.h, x.ctypes.data, y.ctypes.data)
        return y

    def matvec_files(self, out_dir, in_dir, threads=0, max_memory=64e9):
        e = lambda s: s.encode()
        d = self.d
        self.lib().ref_matvec_files(e(f"{d}/comb.txt"), e(f"{d}/evaluation_order.txt"), e(f"{d}/index_lists"),
                                    e(f"{d}/matrix_elements"), e(in_dir), e(out_dir), self.Z, self.N, max_memory,
                                    int(threads))

    def close(self):
        if self.h:
            self.lib().ref_mem_close(self.h)
            self.h = None


def read_blocks(d):
    """[(id, Np, Nn)] of the basis blocks in comb.txt order."""
    out, sec = [], None
    with open(f"{d}/comb.txt") as f:
        for row in f:
            if "***" in row:
                sec = "mp" if "mp-states" in row else None
                continue
            if sec == "mp" and "ARRAYMP:" in row:
                w = row.split()
                out.append((int(w[9].rstrip("=")), int(w[4]), int(w[5])))
    return out


def write_vector_dir(d, blocks, v):
    os.makedirs(d, exist_ok=True)
    off = 0
    for (bid, np_, nn_) in blocks:
        n = np_ * nn_
        np.asarray(v[off:off + n], dtype=np.float64).tofile(f"{d}/vec_{bid}")
        off += n


def read_vector_dir(d, blocks):
    return np.concatenate([np.fromfile(f"{d}/vec_{bid}", dtype=np.float64) for (bid, _, _) in blocks])


def write_zero_vectors(d):
    z = f"{d}/zero_vectors"
    blocks = read_blocks(d)
    if not os.path.isdir(z):
        write_vector_dir(z, blocks, np.zeros(sum(a * b for _, a, b in blocks)))
    return z


def reference_bacchus_available():
    return os.path.exists(REF_BACCHUS)


def reference_bacchus(d, Z, N, max_iterations=200, tolerance=1e-6, converge_eigenvectors=False, target=0):
    """Run the reference's Bacchus on the problem in d; returns {"eigenvalues": the final
    eigensystem block's values, "num_eigenvalues", "eigenvectors": (target + 1, D) array,
    "steps": the eigensystem blocks printed while iterating}."""
    import tempfile
    blocks = read_blocks(d)
    with tempfile.TemporaryDirectory() as wd:
        os.makedirs(os.path.join(wd, "krylov"))
        os.makedirs(os.path.join(wd, "eigen"))
        r = subprocess.run([REF_BACCHUS, f"{d}/comb.txt", f"{d}/evaluation_order.txt", f"{d}/index_lists",
                            f"{d}/matrix_elements", str(Z), str(N), os.path.join(wd, "krylov"), str(max_iterations),
                            repr(float(tolerance)), "1" if converge_eigenvectors else "0", os.path.join(wd, "eigen"),
                            str(target)], capture_output=True, text=True, check=True, cwd=wd)
        out = r.stdout
        blocks_text = out.split("eigensystem:")
        last = blocks_text[-1]
        vals = last[last.index("(") + 1:last.index(")")].split(",")
        ev = np.array([float(v) for v in vals if v.strip()])
        vecs = np.array([read_vector_dir(os.path.join(wd, "eigen", f"eigenvector_{i + 1}"), blocks)
                         for i in range(target + 1)])
    return {"eigenvalues": ev, "num_eigenvalues": len(ev), "eigenvectors": vecs, "steps": len(blocks_text) - 2}
