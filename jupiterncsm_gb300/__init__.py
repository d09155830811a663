"""jupiterncsm_gb300 — GB300-native hot path of JupiterNCSM.

The product is the C ABI in ``include/jncsm.h`` implemented by
``lib/libjncsm_gpu.so`` (sm_103a CUDA kernels).  This module is a thin ctypes
binding used by the tests and the benchmark; it adds no computation of its
own and fails loudly when the native library is missing.

Reference interfaces mirrored (paths relative to the reference src/ tree):
``run_matrix_vector_multiplication`` (Minerva/scheduler/scheduler.c:80-145),
``new_combination_table`` (Utilities/combination_table/combination_table.c:83-137),
``read_evaluation_order`` (Minerva/evaluation_order/evaluation_order.c:43-112).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIBDIR = os.path.join(HERE, "lib")
GPU_LIB = os.path.join(LIBDIR, "libjncsm_gpu.so")
GEN_LIB = os.path.join(LIBDIR, "libjncsm_gen.so")
GEN_CLI = os.path.join(LIBDIR, "jn_gen")
BACCHUS_CLI = os.path.join(LIBDIR, "jn_bacchus")
MERCURY_CLI = os.path.join(LIBDIR, "jn_mercury")

JN_OK = 0
(JN_ERR_INVALID, JN_ERR_IO, JN_ERR_FORMAT, JN_ERR_CUDA, JN_ERR_NOMEM, JN_ERR_NOT_CONVERGED,
 JN_ERR_TIMEOUT) = range(1, 8)
STATUS_NAMES = {0: "JN_OK", 1: "JN_ERR_INVALID", 2: "JN_ERR_IO", 3: "JN_ERR_FORMAT", 4: "JN_ERR_CUDA",
                5: "JN_ERR_NOMEM", 6: "JN_ERR_NOT_CONVERGED", 7: "JN_ERR_TIMEOUT"}


class JnError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def build(jobs=8):
    """Compile the native libraries in-tree (nvcc for sm_103a, gcc for host C)."""
    subprocess.run(["make", "-s", f"-j{jobs}", "-C", os.path.join(HERE, "csrc")], check=True)


class PlanStats(ctypes.Structure):
    _fields_ = [("dimension", ctypes.c_size_t), ("num_blocks", ctypes.c_int), ("num_instructions", ctypes.c_int),
                ("list_entries", ctypes.c_size_t), ("me_elements", ctypes.c_size_t),
                ("me_referenced", ctypes.c_size_t), ("multiply_adds", ctypes.c_double), ("algorithmic_bytes", ctypes.c_double),
                ("num_work_units", ctypes.c_int), ("num_tiles", ctypes.c_int)]


MAX_REPORTED = 64
LANCZOS_FULL, LANCZOS_REFERENCE = 0, 1


class BatchOptions(ctypes.Structure):
    _fields_ = [("num_instances", ctypes.c_int), ("matrix_elements", ctypes.c_void_p),
                ("start_vectors", ctypes.c_void_p), ("max_iterations", ctypes.c_int),
                ("num_eigenvalues", ctypes.c_int), ("tolerance", ctypes.c_double), ("precision", ctypes.c_int),
                ("check_every", ctypes.c_int), ("use_graph", ctypes.c_int), ("refine_extra", ctypes.c_int),
                ("num_eigenvectors", ctypes.c_int), ("eigenvectors", ctypes.c_void_p)]


class BatchResult(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("converged", ctypes.c_int), ("num_eigenvalues", ctypes.c_int),
                ("eigenvalues", ctypes.c_double * MAX_REPORTED), ("ritz_values", ctypes.c_double * MAX_REPORTED),
                ("residual_norms", ctypes.c_double * MAX_REPORTED)]


class TransformStats(ctypes.Structure):
    _fields_ = [("num_two_body_blocks", ctypes.c_int), ("num_one_body_blocks", ctypes.c_int),
                ("num_elements", ctypes.c_size_t), ("num_pair_states", ctypes.c_size_t),
                ("num_configurations", ctypes.c_size_t), ("dense_flops", ctypes.c_double),
                ("algorithmic_bytes", ctypes.c_double), ("plan_seconds", ctypes.c_double)]


class Transform3Stats(ctypes.Structure):
    _fields_ = [("num_three_body_blocks", ctypes.c_int), ("num_elements", ctypes.c_size_t),
                ("num_states", ctypes.c_size_t), ("num_terms", ctypes.c_size_t),
                ("num_coupled_states", ctypes.c_size_t), ("num_m_blocks", ctypes.c_size_t),
                ("file_states", ctypes.c_size_t), ("file_elements", ctypes.c_size_t), ("v_entries", ctypes.c_size_t),
                ("dense_flops", ctypes.c_double), ("algorithmic_bytes", ctypes.c_double),
                ("plan_seconds", ctypes.c_double)]


class Tuning(ctypes.Structure):
    _fields_ = [("engine", ctypes.c_int), ("rows_per_lane", ctypes.c_int), ("ctas_per_sm", ctypes.c_int),
                ("ms", ctypes.c_float), ("candidates", ctypes.c_int)]


class WarmStartOptions(ctypes.Structure):
    _fields_ = [("hidden", ctypes.c_int), ("basis_size", ctypes.c_int), ("train_steps", ctypes.c_int),
                ("learning_rate", ctypes.c_float), ("seed", ctypes.c_uint64), ("noise", ctypes.c_double)]


class LanczosOptions(ctypes.Structure):
    _fields_ = [("max_iterations", ctypes.c_int), ("num_eigenvalues", ctypes.c_int), ("tolerance", ctypes.c_double),
                ("mode", ctypes.c_int), ("check_every", ctypes.c_int), ("start_vector", ctypes.c_void_p),
                ("verbose", ctypes.c_int), ("criterion", ctypes.c_int)]


class LanczosResult(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("converged", ctypes.c_int), ("num_ritz_values", ctypes.c_int),
                ("num_eigenvalues", ctypes.c_int), ("eigenvalues", ctypes.c_double * MAX_REPORTED),
                ("ritz_values", ctypes.c_double * MAX_REPORTED), ("residual_norms", ctypes.c_double * MAX_REPORTED),
                ("iteration_seconds", ctypes.c_double), ("refinement_seconds", ctypes.c_double)]


_gpu = None


def gpu_lib():
    """Load libjncsm_gpu.so with the prototypes of include/jncsm.h."""
    global _gpu
    if _gpu is not None:
        return _gpu
    if not os.path.exists(GPU_LIB):
        raise JnError(4, f"native library {GPU_LIB} is missing: run jupiterncsm_gb300.build()")
    L = ctypes.CDLL(GPU_LIB)
    vp, cp, ci, csz = ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_size_t
    L.jn_last_error.restype = cp
    L.jn_version.restype = cp
    L.jn_open.argtypes = [cp, ctypes.POINTER(vp)]
    L.jn_open_files.argtypes = [cp, cp, cp, cp, ci, ci, ctypes.POINTER(vp)]
    L.jn_close.argtypes = [vp]
    L.jn_close.restype = None
    L.jn_dimension.argtypes = [vp]
    L.jn_dimension.restype = csz
    L.jn_num_blocks.argtypes = [vp]
    L.jn_block_info.argtypes = [vp, ci, ctypes.POINTER(ci), ctypes.POINTER(csz), ctypes.POINTER(csz)]
    L.jn_matvec.argtypes = [vp, vp, vp]
    L.jn_matvec_device.argtypes = [vp, vp, vp, ci, vp]
    L.jn_matvec_files.argtypes = [vp, cp, cp]
    L.jn_synchronize.argtypes = [vp]
    L.jn_matvec_profile.argtypes = [vp, vp, vp, ci, ctypes.POINTER(ctypes.c_float)]
    L.jn_get_plan_stats.argtypes = [vp, ctypes.POINTER(PlanStats)]
    L.jn_inspect_files.argtypes = [cp, cp, cp, cp, ci, ci, ctypes.POINTER(PlanStats)]
    L.jn_set_precision.argtypes = [vp, ci]
    L.jn_set_engine.argtypes = [vp, ci]
    L.jn_lanczos.argtypes = [vp, ctypes.POINTER(LanczosOptions), ctypes.POINTER(LanczosResult)]
    L.jn_lanczos_ritz_values.argtypes = [vp, ctypes.POINTER(ctypes.c_double), ci, ctypes.POINTER(ci)]
    L.jn_lanczos_eigenvector.argtypes = [vp, ci, vp]
    L.jn_lanczos_save_eigenvectors.argtypes = [vp, cp, ci]
    L.jn_print_eigensystem.argtypes = [ctypes.POINTER(ctypes.c_double), ci]
    L.jn_print_eigensystem.restype = None
    L.jn_me_count.argtypes = [vp]
    L.jn_me_count.restype = ctypes.c_size_t
    L.jn_read_matrix_elements.argtypes = [vp, cp, vp]
    L.jn_set_matrix_elements.argtypes = [vp, vp]
    L.jn_lanczos_batch.argtypes = [vp, ctypes.POINTER(BatchOptions), vp]
    L.jn_lanczos_batch_bases.argtypes = [vp, ci, ctypes.POINTER(BatchOptions), vp]
    L.jn_transform_open.argtypes = [cp, cp, ci, ci, ci, ci, cp, ci, ctypes.POINTER(vp)]
    L.jn_transform_run.argtypes = [vp, vp]
    L.jn_transform_profile.argtypes = [vp, ctypes.POINTER(ctypes.c_float)]
    L.jn_transform_elements.argtypes = [vp, ci, vp, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]
    L.jn_transform_write.argtypes = [vp, cp]
    L.jn_transform_get_stats.argtypes = [vp, ctypes.POINTER(TransformStats)]
    L.jn_transform_close.argtypes = [vp]
    L.jn_transform_close.restype = None
    L.jn_transform_2nf.argtypes = [cp, cp, cp, ci, ci, ci, ci, cp, ci]
    L.jn_transform3_open.argtypes = [cp, cp, ci, ci, ci, cp, ctypes.POINTER(vp)]
    L.jn_transform3_run.argtypes = [vp, vp]
    L.jn_transform3_profile.argtypes = [vp, ctypes.POINTER(ctypes.c_float)]
    L.jn_transform3_elements.argtypes = [vp, ci, vp, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]
    L.jn_transform3_write.argtypes = [vp, cp]
    L.jn_transform3_get_stats.argtypes = [vp, ctypes.POINTER(Transform3Stats)]
    L.jn_transform3_close.argtypes = [vp]
    L.jn_transform3_close.restype = None
    L.jn_transform_3nf.argtypes = [cp, cp, cp, ci, ci, ci, cp]
    L.jn_clebsch_gordan.argtypes = [ci] * 6
    L.jn_clebsch_gordan.restype = ctypes.c_double
    L.jn_autotune.argtypes = [vp, ci, ci, ctypes.POINTER(Tuning)]
    L.jn_autotune.restype = ci
    L.jn_set_panel_schedule.argtypes = [vp, ci, ci]
    L.jn_set_panel_schedule.restype = ci
    L.jn_active_engine.argtypes = [vp]
    L.jn_active_engine.restype = ci
    L.jn_set_walk_arithmetic.argtypes = [vp, ci]
    L.jn_set_walk_arithmetic.restype = ci
    L.jn_walk_stats.argtypes = [vp, ctypes.POINTER(ctypes.c_double)]
    L.jn_walk_stats.restype = ci
    fp = ctypes.POINTER(ctypes.c_float)
    L.jn_mlp_create.argtypes = [ci, ci, ci, ctypes.c_uint64, ctypes.POINTER(vp)]
    L.jn_mlp_destroy.argtypes = [vp]
    L.jn_mlp_destroy.restype = None
    L.jn_mlp_num_params.argtypes = [vp]
    L.jn_mlp_num_params.restype = csz
    L.jn_mlp_get_params.argtypes = [vp, vp]
    L.jn_mlp_set_params.argtypes = [vp, vp]
    L.jn_mlp_loss_and_gradient.argtypes = [vp, vp, vp, ci, fp, vp]
    L.jn_mlp_train.argtypes = [vp, vp, vp, ci, ci, ctypes.c_float, fp]
    L.jn_mlp_predict.argtypes = [vp, vp, ci, vp]
    L.jn_warm_start_fit.argtypes = [ctypes.POINTER(WarmStartOptions), ctypes.c_int64, ci, ci, vp, ci, vp,
                                    ctypes.POINTER(vp), fp]
    L.jn_warm_start_vectors.argtypes = [vp, ci, vp, vp]
    L.jn_warm_start_basis.argtypes = [vp, vp]
    L.jn_warm_start_basis_size.argtypes = [vp]
    L.jn_warm_start_destroy.argtypes = [vp]
    L.jn_warm_start_destroy.restype = None
    L.jn_default_start_vector.argtypes = [ctypes.c_int64, vp]
    L.jn_default_start_vector.restype = None
    for name in ("jn_mlp_create", "jn_mlp_get_params", "jn_mlp_set_params", "jn_mlp_loss_and_gradient",
                 "jn_mlp_train", "jn_mlp_predict", "jn_warm_start_fit", "jn_warm_start_vectors",
                 "jn_warm_start_basis"):
        getattr(L, name).restype = ci
    L.jn_subspace_matrices.argtypes = [vp, ci, vp, vp, vp]
    L.jn_subspace_matrices.restype = ci
    L.jn_ceres_files.argtypes = [vp, ci, vp, cp, cp]
    L.jn_ceres_files.restype = ci
    L.jn_aurora.argtypes = [cp, cp, cp, ci, ci, ci, ci, ctypes.POINTER(ci)]
    L.jn_mars.argtypes = [cp, ci, ci, cp, ci, ctypes.POINTER(ci)]
    L.jn_vulcan.argtypes = [cp, ci, ci, ci, vp, vp, cp]
    for name in ("jn_aurora", "jn_mars", "jn_vulcan"):
        getattr(L, name).restype = ci
    for name in ("jn_open", "jn_open_files", "jn_block_info", "jn_matvec", "jn_matvec_device", "jn_matvec_files",
                 "jn_synchronize", "jn_get_plan_stats", "jn_matvec_profile", "jn_inspect_files", "jn_set_precision", "jn_set_engine", "jn_lanczos",
                 "jn_lanczos_ritz_values", "jn_lanczos_eigenvector", "jn_lanczos_save_eigenvectors",
                 "jn_transform_open", "jn_transform_run", "jn_transform_profile", "jn_transform_elements",
                 "jn_transform_write", "jn_transform_get_stats", "jn_transform_2nf", "jn_read_matrix_elements",
                 "jn_set_matrix_elements", "jn_lanczos_batch", "jn_lanczos_batch_bases", "jn_transform3_open",
                 "jn_transform3_run",
                 "jn_transform3_profile", "jn_transform3_elements", "jn_transform3_write", "jn_transform3_get_stats",
                 "jn_transform_3nf"):
        getattr(L, name).restype = ci
    _gpu = L
    return L


def _check(status):
    if status != JN_OK:
        raise JnError(status, gpu_lib().jn_last_error().decode(errors="replace"))


class Hamiltonian:
    """An opened Hamiltonian: index lists and matrix elements resident in HBM."""

    def __init__(self, conf=None, *, comb=None, order=None, lists=None, mes=None, Z=None, N=None):
        L = gpu_lib()
        h = ctypes.c_void_p()
        if conf is not None:
            _check(L.jn_open(conf.encode(), ctypes.byref(h)))
        else:
            _check(L.jn_open_files(comb.encode(), order.encode(), lists.encode(), mes.encode(), int(Z), int(N),
                                   ctypes.byref(h)))
        self._h = h
        self.dimension = L.jn_dimension(h)

    @classmethod
    def from_dir(cls, d, Z, N):
        return cls(comb=f"{d}/comb.txt", order=f"{d}/evaluation_order.txt", lists=f"{d}/index_lists",
                   mes=f"{d}/matrix_elements", Z=Z, N=N)

    def close(self):
        if self._h:
            gpu_lib().jn_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def matvec(self, x, y=None):
        """y += H x on host arrays (y = H x when y is None).  Raises JnError for an x outside
        the fixed-point products' range (max|x| >= 2^127, or the row-sum bound times max|x|
        outside [2^-47, 2^121)); engine 2 at precision 64 takes any x."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        if x.shape != (self.dimension,):
            raise ValueError("x has the wrong dimension")
        y = np.zeros(self.dimension) if y is None else y
        if y.dtype != np.float64 or not y.flags.c_contiguous or y.shape != x.shape:
            raise ValueError("y must be a contiguous float64 vector of the same dimension")
        _check(gpu_lib().jn_matvec(self._h, x.ctypes.data, y.ctypes.data))
        return y

    def matvec_device(self, d_x, d_y, accumulate=False, stream=0):
        _check(gpu_lib().jn_matvec_device(self._h, ctypes.c_void_p(d_x), ctypes.c_void_p(d_y), int(accumulate),
                                          ctypes.c_void_p(stream)))

    def matvec_profile(self, d_x, d_y, accumulate=False):
        """Device product on the context stream; returns (ms of the gather-multiply kernel, ms of the rest)."""
        ms = (ctypes.c_float * 2)()
        _check(gpu_lib().jn_matvec_profile(self._h, ctypes.c_void_p(d_x), ctypes.c_void_p(d_y), int(accumulate), ms))
        return ms[0], ms[1]

    def set_precision(self, bits):
        """64: FP64 products (default); 32: FP32 matrix elements and x with compensated sums."""
        _check(gpu_lib().jn_set_precision(self._h, int(bits)))

    def lanczos(self, max_iterations=200, num_eigenvalues=10, tolerance=1e-6, mode=LANCZOS_FULL, check_every=1,
                start_vector=None, verbose=False, allow_unconverged=False, converge_eigenvectors=False):
        """Run Lanczos on the GPU; returns a dict with eigenvalues (refined), Ritz values, residuals.
        converge_eigenvectors (reference mode): converge the lowest eigenvector of the tridiagonal matrix
        instead of the lowest Ritz value, as the run file's lanczos.converge_eigenvectors does."""
        o = LanczosOptions(max_iterations, num_eigenvalues, tolerance, mode, check_every, None, int(verbose),
                           int(bool(converge_eigenvectors)))
        sv = None
        if start_vector is not None:
            sv = np.ascontiguousarray(start_vector, dtype=np.float64)
            o.start_vector = sv.ctypes.data
        r = LanczosResult()
        st = gpu_lib().jn_lanczos(self._h, ctypes.byref(o), ctypes.byref(r))
        if st != JN_OK and not (allow_unconverged and st == 6):
            _check(st)
        n = r.num_eigenvalues
        return {"iterations": r.iterations, "converged": bool(r.converged), "num_ritz_values": r.num_ritz_values,
                "eigenvalues": np.array(r.eigenvalues[:n]), "ritz_values": np.array(r.ritz_values[:n]),
                "residual_norms": np.array(r.residual_norms[:n]), "status": st,
                "iteration_seconds": r.iteration_seconds, "refinement_seconds": r.refinement_seconds}

    def me_count(self):
        return int(gpu_lib().jn_me_count(self._h))

    def read_matrix_elements(self, directory):
        """Matrix elements of another directory with the same combination table (host array)."""
        out = np.zeros(self.me_count())
        _check(gpu_lib().jn_read_matrix_elements(self._h, directory.encode(), out.ctypes.data))
        return out

    def set_matrix_elements(self, me):
        me = np.ascontiguousarray(me, dtype=np.float64)
        assert me.shape == (self.me_count(),)
        _check(gpu_lib().jn_set_matrix_elements(self._h, me.ctypes.data))

    def lanczos_batch(self, matrix_elements, start_vectors=None, max_iterations=200, num_eigenvalues=10,
                      tolerance=1e-6, precision=32, check_every=10, use_graph=True, refine_extra=4,
                      eigenvectors=0):
        """Solve len(matrix_elements) Hamiltonians on these lists together; returns a list of dicts, and
        with eigenvectors=k also, per instance, the k lowest refined eigenvectors as a (k, D) array."""
        B = len(matrix_elements)
        mes = [np.ascontiguousarray(m, dtype=np.float64) for m in matrix_elements]
        me_ptrs = (ctypes.c_void_p * B)(*[m.ctypes.data for m in mes])
        o = BatchOptions(B, ctypes.cast(me_ptrs, ctypes.c_void_p), None, max_iterations, num_eigenvalues, tolerance,
                         precision, check_every, int(use_graph), refine_extra, int(eigenvectors), None)
        svs = None
        if start_vectors is not None:
            svs = [None if v is None else np.ascontiguousarray(v, dtype=np.float64) for v in start_vectors]
            sv_ptrs = (ctypes.c_void_p * B)(*[None if v is None else v.ctypes.data for v in svs])
            o.start_vectors = ctypes.cast(sv_ptrs, ctypes.c_void_p)
        gs = None
        if eigenvectors:
            gs = [np.zeros((eigenvectors, self.dimension)) for _ in range(B)]
            gs_ptrs = (ctypes.c_void_p * B)(*[g.ctypes.data for g in gs])
            o.eigenvectors = ctypes.cast(gs_ptrs, ctypes.c_void_p)
        res = (BatchResult * B)()
        _check(gpu_lib().jn_lanczos_batch(self._h, ctypes.byref(o), res))
        out = _batch_results(res)
        return (out, gs) if eigenvectors else out

    def ritz_values(self):
        cap = 4096
        out = (ctypes.c_double * cap)()
        cnt = ctypes.c_int()
        _check(gpu_lib().jn_lanczos_ritz_values(self._h, out, cap, ctypes.byref(cnt)))
        return np.array(out[:min(cnt.value, cap)])

    def eigenvector(self, i):
        v = np.zeros(self.dimension)
        _check(gpu_lib().jn_lanczos_eigenvector(self._h, int(i), v.ctypes.data))
        return v

    def save_eigenvectors(self, directory, count):
        _check(gpu_lib().jn_lanczos_save_eigenvectors(self._h, directory.encode(), int(count)))

    def autotune(self, trials=5, tune_engine=False):
        """Time candidate product schedules on this problem, L2 flushed before each, at both
        precisions; install the fastest for the current one (set_precision installs the
        other's) and report it (jn_autotune)."""
        t = Tuning()
        _check(gpu_lib().jn_autotune(self._h, int(trials), int(tune_engine), ctypes.byref(t)))
        return {k: getattr(t, k) for k, _ in Tuning._fields_}

    def set_panel_schedule(self, rows_per_lane, ctas_per_sm):
        _check(gpu_lib().jn_set_panel_schedule(self._h, int(rows_per_lane), int(ctas_per_sm)))

    def subspace_matrices(self, vectors):
        """(norm, op): <v_i|v_j> and <v_j|H v_i> of the given vectors, computed on the GPU (jn_subspace_matrices)."""
        vs = [np.ascontiguousarray(v, dtype=np.float64) for v in vectors]
        n = len(vs)
        ptrs = (ctypes.c_void_p * n)(*[v.ctypes.data for v in vs])
        N, O = np.zeros((n, n)), np.zeros((n, n))
        _check(gpu_lib().jn_subspace_matrices(self._h, n, ctypes.cast(ptrs, ctypes.c_void_p), N.ctypes.data,
                                              O.ctypes.data))
        return N, O

    def ceres_files(self, vector_dirs, norm_matrix_path, subspace_operator_path):
        """The Ceres drop-in: .npy norm and subspace-operator matrices from vec_<block> directories."""
        dirs = (ctypes.c_char_p * len(vector_dirs))(*[d.encode() for d in vector_dirs])
        _check(gpu_lib().jn_ceres_files(self._h, len(vector_dirs), ctypes.cast(dirs, ctypes.c_void_p),
                                        norm_matrix_path.encode() if norm_matrix_path else None,
                                        subspace_operator_path.encode() if subspace_operator_path else None))

    def set_walk_arithmetic(self, fp64_fma):
        """Precision-64 products of the walk engine: exact integers (False, the default) or FP64 FMAs (True)."""
        _check(gpu_lib().jn_set_walk_arithmetic(self._h, 1 if fp64_fma else 0))

    def walk_stats(self):
        """The walk engine's plan: tasks, pieces, row groups, multiply-adds with padding (and with idle lanes), the
        walk element array's length, and the persistent grid."""
        out = (ctypes.c_double * 7)()
        _check(gpu_lib().jn_walk_stats(self._h, out))
        return dict(zip(("tasks", "pieces", "groups", "padded_multiply_adds", "lane_slots", "walk_elements", "grid"),
                        list(out)))

    def active_engine(self):
        """The engine the next product runs (4 panels, 3 block tiles, 2 warp pieces)."""
        return gpu_lib().jn_active_engine(self._h)

    def set_engine(self, engine):
        """4: panels (default where the accumulator fits in shared memory); 5: walks (default above that);
        3: block tiles; 2: warp pieces."""
        _check(gpu_lib().jn_set_engine(self._h, int(engine)))

    def matvec_files(self, out_dir, in_dir):
        _check(gpu_lib().jn_matvec_files(self._h, out_dir.encode(), in_dir.encode()))

    def synchronize(self):
        _check(gpu_lib().jn_synchronize(self._h))

    def stats(self):
        s = PlanStats()
        _check(gpu_lib().jn_get_plan_stats(self._h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in PlanStats._fields_}

    def blocks(self):
        L = gpu_lib()
        out = []
        for b in range(L.jn_num_blocks(self._h)):
            i, o, n = ctypes.c_int(), ctypes.c_size_t(), ctypes.c_size_t()
            _check(L.jn_block_info(self._h, b, ctypes.byref(i), ctypes.byref(o), ctypes.byref(n)))
            out.append((i.value, o.value, n.value))
        return out


def _batch_results(res):
    out = []
    for r in res:
        n = r.num_eigenvalues
        out.append({"iterations": r.iterations, "converged": bool(r.converged),
                    "eigenvalues": np.array(r.eigenvalues[:n]), "ritz_values": np.array(r.ritz_values[:n]),
                    "residual_norms": np.array(r.residual_norms[:n])})
    return out


def lanczos_batch_bases(bases, max_iterations=200, num_eigenvalues=10, tolerance=1e-6, precision=32, check_every=10,
                        use_graph=True, refine_extra=4, eigenvectors=0):
    """Solve the Hamiltonians of several bases together (jn_lanczos_batch_bases): bases is a list of
    (Hamiltonian, [matrix-element arrays], start vectors or None).  Every Lanczos step is one graph with
    one product launch for all instances of all bases.  Returns, per basis, a list of dicts (and with
    eigenvectors=k, per basis, the k lowest refined eigenvectors of each instance as (k, D) arrays)."""
    nb = len(bases)
    opts = (BatchOptions * nb)()
    keep, results, gs_all = [], [], []
    for b, entry in enumerate(bases):
        H, mes = entry[0], [np.ascontiguousarray(m, dtype=np.float64) for m in entry[1]]
        svs = entry[2] if len(entry) > 2 else None
        B = len(mes)
        me_ptrs = (ctypes.c_void_p * B)(*[m.ctypes.data for m in mes])
        o = opts[b]
        o.num_instances, o.matrix_elements = B, ctypes.cast(me_ptrs, ctypes.c_void_p)
        o.max_iterations, o.num_eigenvalues, o.tolerance, o.precision = max_iterations, num_eigenvalues, tolerance, precision
        o.check_every, o.use_graph, o.refine_extra, o.num_eigenvectors = check_every, int(use_graph), refine_extra, int(eigenvectors)
        keep += [mes, me_ptrs]
        if svs is not None:
            svs = [None if v is None else np.ascontiguousarray(v, dtype=np.float64) for v in svs]
            sv_ptrs = (ctypes.c_void_p * B)(*[None if v is None else v.ctypes.data for v in svs])
            o.start_vectors = ctypes.cast(sv_ptrs, ctypes.c_void_p)
            keep += [svs, sv_ptrs]
        if eigenvectors:
            gs = [np.zeros((eigenvectors, H.dimension)) for _ in range(B)]
            gs_ptrs = (ctypes.c_void_p * B)(*[g.ctypes.data for g in gs])
            o.eigenvectors = ctypes.cast(gs_ptrs, ctypes.c_void_p)
            keep += [gs_ptrs]
            gs_all.append(gs)
        results.append((BatchResult * B)())
    ctxs = (ctypes.c_void_p * nb)(*[entry[0]._h for entry in bases])
    res_ptrs = (ctypes.c_void_p * nb)(*[ctypes.addressof(r) for r in results])
    _check(gpu_lib().jn_lanczos_batch_bases(ctxs, nb, opts, res_ptrs))
    out = [_batch_results(r) for r in results]
    return (out, gs_all) if eigenvectors else out


def _f32(a, cols):
    a = np.ascontiguousarray(a, dtype=np.float32)
    if a.ndim == 1:
        a = a.reshape(1, -1)
    assert a.shape[1] == cols, (a.shape, cols)
    return a


class MLP:
    """The warm start's perceptron, trained and evaluated by the library's CUDA kernels (jn_mlp_*)."""

    def __init__(self, num_inputs, hidden, num_outputs, seed=0):
        self.shape = (num_inputs, hidden, num_outputs)
        self._h = ctypes.c_void_p()
        _check(gpu_lib().jn_mlp_create(num_inputs, hidden, num_outputs, seed, ctypes.byref(self._h)))

    def close(self):
        if self._h:
            gpu_lib().jn_mlp_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_params(self):
        return gpu_lib().jn_mlp_num_params(self._h)

    def params(self):
        p = np.zeros(self.num_params, dtype=np.float32)
        _check(gpu_lib().jn_mlp_get_params(self._h, p.ctypes.data))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.shape == (self.num_params,)
        _check(gpu_lib().jn_mlp_set_params(self._h, p.ctypes.data))

    def loss_and_gradient(self, x, t):
        x, t = _f32(x, self.shape[0]), _f32(t, self.shape[2])
        loss = ctypes.c_float()
        g = np.zeros(self.num_params, dtype=np.float32)
        _check(gpu_lib().jn_mlp_loss_and_gradient(self._h, x.ctypes.data, t.ctypes.data, len(x), ctypes.byref(loss),
                                                  g.ctypes.data))
        return loss.value, g

    def train(self, x, t, steps, learning_rate=1e-3):
        x, t = _f32(x, self.shape[0]), _f32(t, self.shape[2])
        loss = ctypes.c_float()
        _check(gpu_lib().jn_mlp_train(self._h, x.ctypes.data, t.ctypes.data, len(x), int(steps),
                                      ctypes.c_float(learning_rate), ctypes.byref(loss)))
        return loss.value

    def predict(self, x):
        x = _f32(x, self.shape[0])
        y = np.zeros((len(x), self.shape[2]), dtype=np.float32)
        _check(gpu_lib().jn_mlp_predict(self._h, x.ctypes.data, len(x), y.ctypes.data))
        return y


def aurora(comb, anicre_dir, output_dir, Z, N, human_readable=False, skip_three_body=False):
    """Anicre index lists -> index_list_<id> (jn_aurora, the aurora.x drop-in); returns the lists written."""
    n = ctypes.c_int()
    _check(gpu_lib().jn_aurora(comb.encode(), anicre_dir.encode(), output_dir.encode(), Z, N, int(human_readable),
                               int(skip_three_body), ctypes.byref(n)))
    return n.value


def mars(comb, Z, N, output_file, two_body_only=False):
    """Evaluation order from the combination table's CALCBLOCK rows (jn_mars, the mars.x drop-in)."""
    n = ctypes.c_int()
    _check(gpu_lib().jn_mars(comb.encode(), Z, N, output_file.encode(), int(two_body_only), ctypes.byref(n)))
    return n.value


def vulcan(comb, Z, N, operators, output_dir):
    """sum_i c_i * operator_i over every matrix-element block (jn_vulcan, the vulcan.x drop-in);
    operators: [(directory, coefficient), ...]."""
    dirs = [d.encode() for d, _ in operators]
    dp = (ctypes.c_char_p * max(1, len(dirs)))(*dirs)
    cf = (ctypes.c_double * max(1, len(dirs)))(*[c for _, c in operators])
    _check(gpu_lib().jn_vulcan(comb.encode(), Z, N, len(dirs), ctypes.cast(dp, ctypes.c_void_p),
                               ctypes.cast(cf, ctypes.c_void_p), output_dir.encode()))


def default_start_vector(dim):
    """The batched solver's default start vector (jn_default_start_vector)."""
    v = np.zeros(dim)
    gpu_lib().jn_default_start_vector(int(dim), v.ctypes.data)
    return v


class WarmStart:
    """Learned warm start for Hamiltonian.lanczos_batch (jn_warm_start_*): fitted on couplings and the
    eigenvectors the solver returned for them; gives start vectors for new couplings."""

    def __init__(self, couplings, eigenvectors, hidden=128, basis_size=32, train_steps=3000, learning_rate=1e-3,
                 seed=0, noise=0.01):
        c = np.ascontiguousarray(couplings, dtype=np.float64)
        S, nc = c.shape
        ev = [np.ascontiguousarray(v, dtype=np.float64) for v in eigenvectors]
        assert len(ev) == S and all(v.shape == ev[0].shape for v in ev)
        nv, dim = ev[0].shape
        ptrs = (ctypes.c_void_p * S)(*[v.ctypes.data for v in ev])
        o = WarmStartOptions(hidden, basis_size, train_steps, learning_rate, seed, noise)
        self._h = ctypes.c_void_p()
        loss = ctypes.c_float()
        _check(gpu_lib().jn_warm_start_fit(ctypes.byref(o), dim, nc, S, c.ctypes.data, nv,
                                           ctypes.cast(ptrs, ctypes.c_void_p), ctypes.byref(self._h),
                                           ctypes.byref(loss)))
        self.final_loss = loss.value
        self.dim, self.num_couplings = dim, nc

    def close(self):
        if self._h:
            gpu_lib().jn_warm_start_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def basis_size(self):
        return gpu_lib().jn_warm_start_basis_size(self._h)

    def basis(self):
        b = np.zeros((self.basis_size, self.dim))
        _check(gpu_lib().jn_warm_start_basis(self._h, b.ctypes.data))
        return b

    def start_vectors(self, couplings):
        c = np.ascontiguousarray(couplings, dtype=np.float64).reshape(-1, self.num_couplings)
        out = [np.zeros(self.dim) for _ in range(len(c))]
        ptrs = (ctypes.c_void_p * len(c))(*[v.ctypes.data for v in out])
        _check(gpu_lib().jn_warm_start_vectors(self._h, len(c), c.ctypes.data, ctypes.cast(ptrs, ctypes.c_void_p)))
        return out


class Transform:
    """J-scheme -> M-scheme two-body transform on the GPU (Mercury's two-body part)."""

    def __init__(self, comb, index_list_dir, Z, N, single_particle_energy, two_particle_energy, antoine_file,
                 include_kinetic=True):
        L = gpu_lib()
        h = ctypes.c_void_p()
        _check(L.jn_transform_open(comb.encode(), index_list_dir.encode(), Z, N, single_particle_energy,
                                   two_particle_energy, antoine_file.encode(), int(include_kinetic), ctypes.byref(h)))
        self._h = h

    @classmethod
    def from_dir(cls, d, Z, N, single_particle_energy, two_particle_energy, include_kinetic=True):
        """A generator output directory: comb.txt, anicr/ and antoine_2nf.bin."""
        return cls(os.path.join(d, "comb.txt"), os.path.join(d, "anicr"), Z, N, single_particle_energy,
                   two_particle_energy, os.path.join(d, "antoine_2nf.bin"), include_kinetic)

    def run(self, stream=None):
        _check(gpu_lib().jn_transform_run(self._h, ctypes.c_void_p(stream)))

    def profile(self):
        ms = ctypes.c_float()
        _check(gpu_lib().jn_transform_profile(self._h, ctypes.byref(ms)))
        return ms.value

    def block(self, block_id):
        import numpy as np
        L = gpu_lib()
        n = ctypes.c_size_t()
        _check(L.jn_transform_elements(self._h, block_id, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value)
        _check(L.jn_transform_elements(self._h, block_id, out.ctypes.data_as(ctypes.c_void_p), n.value, ctypes.byref(n)))
        return out

    def write(self, output_dir):
        _check(gpu_lib().jn_transform_write(self._h, output_dir.encode()))

    def stats(self):
        s = TransformStats()
        _check(gpu_lib().jn_transform_get_stats(self._h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in TransformStats._fields_}

    def close(self):
        if self._h:
            gpu_lib().jn_transform_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def transform_2nf(comb, index_list_dir, output_dir, Z, N, single_particle_energy, two_particle_energy, antoine_file,
                  include_kinetic=True):
    """The two-body part of mercury_J_scheme_to_internal.x: writes <output_dir>/<id>_matrix_elements."""
    _check(gpu_lib().jn_transform_2nf(comb.encode(), index_list_dir.encode(), output_dir.encode(), Z, N,
                                      single_particle_energy, two_particle_energy, antoine_file.encode(),
                                      int(include_kinetic)))


class Transform3:
    """J-scheme -> M-scheme three-body transform on the GPU (Mercury's three-body
    part, J-scheme elements in the reference's ASCII format)."""

    def __init__(self, comb, index_list_dir, Z, N, single_particle_energy, jscheme_dir):
        h = ctypes.c_void_p()
        _check(gpu_lib().jn_transform3_open(comb.encode(), index_list_dir.encode(), Z, N, single_particle_energy,
                                            jscheme_dir.encode(), ctypes.byref(h)))
        self._h = h

    @classmethod
    def from_dir(cls, d, Z, N, single_particle_energy, jscheme_subdir="jjj"):
        """A generator output directory: comb.txt, anicr/ and the J-scheme directory."""
        return cls(os.path.join(d, "comb.txt"), os.path.join(d, "anicr"), Z, N, single_particle_energy,
                   os.path.join(d, jscheme_subdir))

    def run(self, stream=None):
        _check(gpu_lib().jn_transform3_run(self._h, ctypes.c_void_p(stream)))

    def profile(self):
        ms = ctypes.c_float()
        _check(gpu_lib().jn_transform3_profile(self._h, ctypes.byref(ms)))
        return ms.value

    def block(self, block_id):
        import numpy as np
        L = gpu_lib()
        n = ctypes.c_size_t()
        _check(L.jn_transform3_elements(self._h, block_id, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value)
        _check(L.jn_transform3_elements(self._h, block_id, out.ctypes.data_as(ctypes.c_void_p), n.value,
                                        ctypes.byref(n)))
        return out

    def write(self, output_dir):
        _check(gpu_lib().jn_transform3_write(self._h, output_dir.encode()))

    def stats(self):
        s = Transform3Stats()
        _check(gpu_lib().jn_transform3_get_stats(self._h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in Transform3Stats._fields_}

    def close(self):
        if self._h:
            gpu_lib().jn_transform3_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def transform_3nf(comb, index_list_dir, output_dir, Z, N, single_particle_energy, jscheme_dir):
    """The three-body part of mercury_J_scheme_to_internal.x: writes <output_dir>/<id>_matrix_elements."""
    _check(gpu_lib().jn_transform_3nf(comb.encode(), index_list_dir.encode(), output_dir.encode(), Z, N,
                                      single_particle_energy, jscheme_dir.encode()))


def transform3_status(comb, index_list_dir, Z, N, single_particle_energy, jscheme_dir):
    """(status, message) of jn_transform3_open without raising: the host plan
    validates its inputs before any device is touched."""
    L = gpu_lib()
    h = ctypes.c_void_p()
    st = L.jn_transform3_open(comb.encode(), index_list_dir.encode(), Z, N, single_particle_energy,
                              jscheme_dir.encode(), ctypes.byref(h))
    msg = L.jn_last_error().decode(errors="replace") if st else ""
    if h.value:
        L.jn_transform3_close(h)
    return st, msg


def transform_status(comb, index_list_dir, Z, N, single_particle_energy, two_particle_energy, antoine_file,
                     include_kinetic=True):
    """(status, message) of jn_transform_open without raising: host-side validation is
    reported before any device is touched."""
    L = gpu_lib()
    h = ctypes.c_void_p()
    st = L.jn_transform_open(comb.encode(), index_list_dir.encode(), Z, N, single_particle_energy,
                             two_particle_energy, antoine_file.encode(), int(include_kinetic), ctypes.byref(h))
    msg = L.jn_last_error().decode(errors="replace") if st else ""
    if h.value:
        L.jn_transform_close(h)
    return st, msg


def clebsch_gordan(j1, j2, j3, m1, m2, m3):
    """<j1 m1 j2 m2 | j3 m3>, arguments doubled (host computation, no GPU)."""
    return gpu_lib().jn_clebsch_gordan(j1, j2, j3, m1, m2, m3)


def inspect(d, Z, N):
    """Plan statistics of a problem directory, computed on the host (no GPU)."""
    s = PlanStats()
    e = lambda t: t.encode()
    _check(gpu_lib().jn_inspect_files(e(f"{d}/comb.txt"), e(f"{d}/evaluation_order.txt"), e(f"{d}/index_lists"),
                                      e(f"{d}/matrix_elements"), int(Z), int(N), ctypes.byref(s)))
    return {k: getattr(s, k) for k, _ in PlanStats._fields_}


# ---------------------------------------------------------------- generator
class GenConfig(ctypes.Structure):
    _fields_ = [("Z", ctypes.c_int), ("N", ctypes.c_int), ("Nmax", ctypes.c_int), ("M2", ctypes.c_int),
                ("parity", ctypes.c_int), ("nbody", ctypes.c_int), ("seed", ctypes.c_uint64),
                ("hbar_omega", ctypes.c_double), ("sigma2", ctypes.c_double), ("sigma3", ctypes.c_double),
                ("me_only", ctypes.c_int), ("me_subdir", ctypes.c_char_p), ("write_basis_files", ctypes.c_int),
                ("lanczos_iterations", ctypes.c_int), ("antoine", ctypes.c_int), ("anicre_lists", ctypes.c_int)]


class GenSummary(ctypes.Structure):
    _fields_ = [("dimension", ctypes.c_size_t), ("num_basis_blocks", ctypes.c_int), ("num_lists", ctypes.c_size_t),
                ("list_entries", ctypes.c_size_t), ("num_me_blocks", ctypes.c_size_t),
                ("me_elements", ctypes.c_size_t), ("num_calc_blocks", ctypes.c_size_t),
                ("multiplications", ctypes.c_ulonglong), ("num_orbitals", ctypes.c_int),
                ("num_proton_sds", ctypes.c_int), ("num_neutron_sds", ctypes.c_int),
                ("emax_single", ctypes.c_int), ("emax_pair", ctypes.c_int)]


_gen = None


def gen_lib():
    global _gen
    if _gen is None:
        if not os.path.exists(GEN_LIB):
            raise JnError(2, f"{GEN_LIB} is missing: run jupiterncsm_gb300.build()")
        _gen = ctypes.CDLL(GEN_LIB)
        _gen.jn_generate.argtypes = [ctypes.POINTER(GenConfig), ctypes.c_char_p, ctypes.POINTER(GenSummary)]
        _gen.jn_gen_last_error.restype = ctypes.c_char_p
        _gen.jn_gen_default_config.argtypes = [ctypes.POINTER(GenConfig)]
        _gen.jn_gen_pair_normal.restype = ctypes.c_double
        _gen.jn_gen_pair_normal.argtypes = [ctypes.c_uint64] * 4
        _gen.jn_gen_antoine.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                        ctypes.c_uint64, ctypes.c_double]
        _gen.jn_gen_jjj_ascii.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_uint64, ctypes.c_double,
                                          ctypes.c_void_p, ctypes.c_void_p]
    return _gen


def generate(outdir, Z=2, N=2, nmax=4, M2=0, parity=0, nbody=2, seed=20261203, hbar_omega=20.0, sigma2=1.0,
             sigma3=0.1, me_only_subdir=None, basis_files=True, lanczos_iterations=200, antoine=False,
             anicre_lists=0):
    """Write a synthetic problem in the reference formats; returns the generator summary.

    With antoine=True the two-body interaction is written as a J-scheme
    Antoine file (antoine_2nf.bin) and its M-scheme blocks are left to the
    J->M transform.  anicre_lists=1 (raw) or 2 (text rows) also writes the
    index lists under the names Anicre gives them (anicr_lists/), the input
    of aurora.x / jn_aurora."""
    G = gen_lib()
    c = GenConfig()
    G.jn_gen_default_config(ctypes.byref(c))
    c.Z, c.N, c.Nmax, c.M2, c.parity, c.nbody = Z, N, nmax, M2, parity, nbody
    c.seed, c.hbar_omega, c.sigma2, c.sigma3 = seed, hbar_omega, sigma2, sigma3
    c.write_basis_files = int(basis_files)
    c.lanczos_iterations = lanczos_iterations
    c.antoine = int(antoine)
    c.anicre_lists = int(anicre_lists)
    if me_only_subdir:
        c.me_only = 1
        c.me_subdir = me_only_subdir.encode()
    s = GenSummary()
    rc = G.jn_generate(ctypes.byref(c), outdir.encode(), ctypes.byref(s))
    if rc != 0:
        raise JnError(rc, G.jn_gen_last_error().decode())
    return {k: getattr(s, k) for k, _ in GenSummary._fields_}


def three_body_energy(comb):
    """Largest three-particle energy (ket or bra side) among the three-body
    matrix-element blocks of a combination table (0 when there are none)."""
    e3, sec = 0, 0
    with open(comb) as f:
        for row in f:
            if "***" in row:
                sec = 1 if "Matrix-elements V (cross p-n)" in row else 2 if "Matrix-elements V (same p/n)" in row else 0
                continue
            if not sec or "ARRAY:" not in row:
                continue
            w = row.split()
            if sec == 1:
                k = w[0].count("p") + w[4].count("n")
                dEp, dp, dEn, dn = int(w[1]), int(w[3]), int(w[5]), int(w[7])
                lo, hi = dp + dn, dp + dEp + dn + dEn
            else:
                k = len(w[0])
                dE, d = int(w[1]), int(w[3])
                lo, hi = d, d + dE
            if k == 3:
                e3 = max(e3, lo, hi)
    return e3


def write_jjj(dirname, emax, e3max, seed=20261203, sigma=0.1):
    """Write a seeded jjj-coupled three-body interaction in the reference's
    ASCII format (dirname/jjj.cnf, dirname/jjj.mat); returns (states, elements)."""
    G = gen_lib()
    ns, ne = ctypes.c_int64(), ctypes.c_int64()
    rc = G.jn_gen_jjj_ascii(dirname.encode(), emax, e3max, seed, sigma, ctypes.byref(ns), ctypes.byref(ne))
    if rc != 0:
        raise JnError(rc, G.jn_gen_last_error().decode())
    return ns.value, ne.value


def write_antoine(path, emax1, emax2, num_particles, hbar_omega=20.0, seed=20261203, sigma=1.0):
    """Write a seeded J-scheme two-body interaction in the Antoine format."""
    G = gen_lib()
    rc = G.jn_gen_antoine(path.encode(), emax1, emax2, num_particles, hbar_omega, seed, sigma)
    if rc != 0:
        raise JnError(rc, G.jn_gen_last_error().decode())
