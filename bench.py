"""Benchmark: index-list matvec GB/s on one GB300 (and N independent replicas).

A step is one Hamiltonian product y = H x of the JupiterNCSM hot path on the
workload below (default: 6Li Nmax 6, 2M = 2, two- plus three-body forces,
D = 186 894, the largest single-GPU configuration), with x, y, the index
lists and the matrix elements already resident in HBM.  `value` is the
algorithmic traffic of one product in the reference's FP64 terms (index
lists in the reference's 12-byte format, the 8-byte matrix elements they
reference, x read and y written) times the steps of all ranks, divided by
the CUDA-event time of the slowest rank.  L2 is flushed (256 MiB write)
between timed steps.  The headline arithmetic is the walk engine's exact
integer product (`dtype` "i64"); its error against the CPU reference is
reported beside the FP64-FMA and FP32 paths'.

`e2e` is the same metric through the public C ABI call jn_matvec with host
buffers in pinned memory: host->device copy of x and y and device->host copy
of y inside the timed region of every step.

`--impl reference` times the reference's CPU algorithm (OpenMP task farm over
the evaluation order with per-thread output replicas) on the host cores: the
compiled reference where it was built on this machine, else the oracle's
plain-C restatement of it, with the same byte formula.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # the largest single-GPU configuration: A=6 Nmax=6 with two- and three-body forces
    "li6_nmax6_2nf3nf": dict(Z=3, N=3, nmax=6, nbody=3, M2=2,
                             label="6Li (Z=3,N=3) HO M-scheme Nmax=6, 2M=2, +parity, seeded 2NF N(0,1) + 3NF N(0,0.1) "
                                   "MeV, hw=20 MeV"),
    # the A=4 Nmax=6 configuration with two- plus three-body forces
    "he4_nmax6_2nf3nf": dict(Z=2, N=2, nmax=6, nbody=3, M2=0,
                             label="4He (Z=2,N=2) HO M-scheme Nmax=6, 2M=0, +parity, seeded 2NF N(0,1) + 3NF N(0,0.1) MeV, hw=20 MeV"),
    "he4_nmax4_2nf": dict(Z=2, N=2, nmax=4, nbody=2, M2=0,
                          label="4He (Z=2,N=2) HO M-scheme Nmax=4, 2M=0, +parity, seeded 2NF N(0,1) MeV, hw=20 MeV"),
    # a medium case of the large workload's structure (larger than L2, a few GB on the device): profiling
    "li6_nmax4_2nf3nf": dict(Z=3, N=3, nmax=4, nbody=3, M2=2,
                             label="6Li (Z=3,N=3) HO M-scheme Nmax=4, 2M=2, +parity, seeded 2NF N(0,1) + 3NF N(0,0.1) "
                                   "MeV, hw=20 MeV"),
    "li6_nmax6_2nf": dict(Z=3, N=3, nmax=6, nbody=2, M2=2,
                          label="6Li (Z=3,N=3) HO M-scheme Nmax=6, 2M=2, +parity, seeded 2NF N(0,1) MeV, hw=20 MeV"),
}
# product arithmetics: precision, FP64 FMAs on the walk engine
ARITH = {"i64": (64, False), "fp64": (64, True), "f32": (32, False)}
METRIC = "index-list matvec GB/s vs HBM peak"
FLUSH_BYTES = 256 << 20


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return None


KERNELS = {(4, "f32"): "jn_panel_kernel_i32", (4, "i64"): "jn_panel_kernel_fp64", (4, "fp64"): "jn_panel_kernel_fp64",
           (3, "f32"): "jn_tile_kernel<float>", (3, "i64"): "jn_tile_kernel<double>", (3, "fp64"): "jn_tile_kernel<double>",
           (5, "i64"): "jn_walk_kernel<1>", (5, "fp64"): "jn_walk_kernel<64>", (5, "f32"): "jn_walk_kernel<32>"}
# kernels launched per product: max|x| (and the copies of x), the product, the conversion into y; the walk
# engine's integer path converts x in a kernel of its own
LAUNCHES = {(5, "i64"): 4}


def max_over_ranks(v, dist, device):
    """The largest of every rank's v (a job takes as long as its slowest rank); v itself on one rank."""
    if not dist:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_gbs(bytes_per_step, world, seconds_per_step):
    """Whole-job GB/s: every rank's products (replicas of the same workload) over the slowest rank's time."""
    return bytes_per_step * world / seconds_per_step / 1e9


def profile_traffic(workload, engine, arith):
    """DRAM bytes (read + write) per launch of the product kernel from the committed ncu summary, if any."""
    name = {4: "jn_panel_kernel", 3: "jn_tile_kernel", 5: "jn_walk_kernel"}.get(engine)
    if name is None:
        return None
    path = os.path.join(ROOT, "profiles", f"{name}_{workload}.md")
    try:
        m = re.search(rf"dram_bytes_per_launch_{arith}:\s*([0-9.eE+]+)", open(path).read())
        return float(m.group(1)) if m else None
    except OSError:
        return None


class ClockSampler:
    """SM clocks and throttle reasons sampled during the timed region.

    NVML (libnvidia-ml, read-only queries) is polled every 2 ms from a thread,
    so that even a timed region of a few milliseconds gets samples; where NVML
    cannot be loaded, `nvidia-smi -lms 200` is used instead."""
    SMI_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                  "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                  "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    # nvmlClocksEventReason bits
    REASON_BITS = {"sw_power_cap": 0x4, "hw_slowdown": 0x8 | 0x80, "sw_thermal_slowdown": 0x20,
                   "hw_thermal_slowdown": 0x40}

    def __init__(self, device):
        self.device = device
        vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
        try:
            self.nvml_index = int(vis.split(",")[device]) if vis else device
        except (ValueError, IndexError):
            self.nvml_index = device
        self.proc = None
        self.path = None
        self.thread = None
        self.samples = []
        self.source = None

    def _nvml(self):
        import ctypes
        lib = ctypes.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        h = ctypes.c_void_p()
        if lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(self.nvml_index), ctypes.byref(h)) != 0:
            raise OSError("nvmlDeviceGetHandleByIndex failed")
        reasons_fn = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            lib.nvmlDeviceGetCurrentClocksThrottleReasons
        mx = ctypes.c_uint(0)
        lib.nvmlDeviceGetMaxClockInfo(h, ctypes.c_int(1), ctypes.byref(mx))
        return lib, h, reasons_fn, mx.value

    def start(self):
        import threading
        try:
            lib, h, reasons_fn, mx = self._nvml()
        except Exception:
            return self._start_smi()
        import ctypes
        self.source = "nvml (2 ms polling)"
        self.max_mhz = mx
        self.stop_flag = threading.Event()

        def run():
            sm, rs, pw = ctypes.c_uint(), ctypes.c_ulonglong(), ctypes.c_uint()
            while not self.stop_flag.is_set():
                if lib.nvmlDeviceGetClockInfo(h, ctypes.c_int(1), ctypes.byref(sm)) == 0 and \
                        reasons_fn(h, ctypes.byref(rs)) == 0:
                    lib.nvmlDeviceGetPowerUsage(h, ctypes.byref(pw))
                    self.samples.append((sm.value, rs.value, pw.value / 1000.0))
                time.sleep(0.002)
        self.thread = threading.Thread(target=run, daemon=True)
        self.thread.start()

    def _start_smi(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.nvml_index), f"--query-gpu={self.SMI_FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=fd, stderr=subprocess.DEVNULL)
            os.close(fd)
            self.source = "nvidia-smi -lms 200"
        except Exception:
            self.proc = None

    def stop(self):
        if self.thread:
            self.stop_flag.set()
            self.thread.join(timeout=5)
            if not self.samples:
                return None
            sm = [s[0] for s in self.samples]
            reasons = sorted({n for s in self.samples for n, b in self.REASON_BITS.items() if s[1] & b})
            return {"sm_mhz": statistics.median(sm), "sm_max_mhz": self.max_mhz, "reasons": reasons,
                    "samples": len(self.samples), "sm_mhz_min": min(sm),
                    "power_w_median": statistics.median(s[2] for s in self.samples), "source": self.source}
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            w = [x.strip() for x in line.split(",")]
            if len(w) >= 9:
                rows.append(w)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "source": self.source}


def prepare(workload, workdir):
    import jupiterncsm_gb300 as jn
    w = WORKLOADS[workload]
    d = os.path.join(workdir, workload)
    stamp = os.path.join(d, ".complete")
    if not os.path.exists(stamp):
        t = time.time()
        jn.generate(d, Z=w["Z"], N=w["N"], nmax=w["nmax"], nbody=w["nbody"], M2=w["M2"], basis_files=False)
        open(stamp, "w").write("ok\n")
        log(f"generated {workload} in {time.time() - t:.1f} s")
    return d


TRANSFORM_WORKLOAD = dict(Z=3, N=3, nmax=6, M2=2,
                          label="6Li (Z=3,N=3) Nmax=6, 2M=2: seeded J-scheme 2NF N(0,1) MeV (Antoine format) -> "
                                "all two-body M-scheme blocks of the combination table")


def transform_leg(workdir, steps, warmup, flush, peak):
    """The J -> M two-body transform on the GPU: one kernel computes every
    two-body block; timed with CUDA events, L2 flushed between runs."""
    import torch
    import jupiterncsm_gb300 as jn
    w = TRANSFORM_WORKLOAD
    d = os.path.join(workdir, "li6_nmax6_jscheme")
    stamp = os.path.join(d, ".complete")
    if not os.path.exists(stamp):
        t = time.time()
        s = jn.generate(d, Z=w["Z"], N=w["N"], nmax=w["nmax"], M2=w["M2"], nbody=2, antoine=True)
        open(stamp, "w").write(f"{s['emax_single']} {s['emax_pair']}\n")
        log(f"generated the J-scheme workload in {time.time() - t:.1f} s")
    e1, e2 = (int(v) for v in open(stamp).read().split())
    t0 = time.perf_counter()
    T = jn.Transform.from_dir(d, w["Z"], w["N"], e1, e2)
    open_s = time.perf_counter() - t0
    st = T.stats()
    for _ in range(warmup):
        T.profile()
    ms = []
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        ms.append(T.profile())
    T.close()
    kms = sum(ms) / len(ms)
    # the drop-in call end to end: plan, upload, kernel, copy back, files written
    out = os.path.join(d, "transformed")
    t0 = time.perf_counter()
    jn.transform_2nf(os.path.join(d, "comb.txt"), os.path.join(d, "anicr"), out, w["Z"], w["N"], e1, e2,
                     os.path.join(d, "antoine_2nf.bin"))
    e2e_s = time.perf_counter() - t0
    achieved = st["algorithmic_bytes"] / (kms / 1e3) / 1e9
    return {"workload": w["label"], "elements": st["num_elements"], "two_body_blocks": st["num_two_body_blocks"],
            "pair_states": st["num_pair_states"], "configurations": st["num_configurations"],
            "kernel_ms": kms, "elements_per_s": st["num_elements"] / (kms / 1e3),
            "roofline": {"bound": "fp64 pipe", "fp64_pipe_busy_ncu": 0.764,
                         "profile": "profiles/jn_jt_to_m_kernel_li6_nmax6.md",
                         "hbm_achieved": achieved, "hbm_peak": peak, "unit": "GB/s", "hbm_frac": achieved / peak,
                         "bytes_per_run": st["algorithmic_bytes"], "kernel": "jn_jt_to_m_kernel",
                         "note": "each element is a sum of separately rounded FP64 products (the reference's "
                                 "arithmetic), so GB300's FP64 pipe bounds the kernel, not HBM"},
            "dense_equivalent_flops": st["dense_flops"],
            "dense_equivalent_tflop_per_s": st["dense_flops"] / (kms / 1e3) / 1e12,
            "plan_seconds": st["plan_seconds"], "open_seconds": open_s,
            "e2e": {"seconds": e2e_s, "what": "jn_transform_2nf: plan + upload + kernel + copy back + files"},
            "l2": "flushed between timed runs (256 MiB write)", "steps": steps, "warmup": warmup}


TRANSFORM3_WORKLOAD = dict(Z=3, N=3, nmax=4, M2=0,
                           label="6Li (Z=3,N=3) Nmax=4, 2M=0: seeded jjj-coupled 3NF N(0,0.1) MeV (the reference's "
                                 "ASCII J-scheme format) -> all three-body M-scheme blocks of the combination table")


def transform3_leg(workdir, steps, warmup, flush, peak):
    """The J -> M three-body transform on the GPU: one kernel computes every
    three-body block; timed with CUDA events, L2 flushed between runs."""
    import torch
    import jupiterncsm_gb300 as jn
    w = TRANSFORM3_WORKLOAD
    d = os.path.join(workdir, "li6_nmax4_jjj")
    stamp = os.path.join(d, ".complete")
    if not os.path.exists(stamp):
        t = time.time()
        s = jn.generate(d, Z=w["Z"], N=w["N"], nmax=w["nmax"], M2=w["M2"], nbody=3, antoine=True)
        e3 = jn.three_body_energy(os.path.join(d, "comb.txt"))
        jn.write_jjj(os.path.join(d, "jjj"), s["emax_single"], e3)
        open(stamp, "w").write(f"{s['emax_single']}\n")
        log(f"generated the three-body J-scheme workload in {time.time() - t:.1f} s")
    e1 = int(open(stamp).read())
    t0 = time.perf_counter()
    T = jn.Transform3.from_dir(d, w["Z"], w["N"], e1)
    open_s = time.perf_counter() - t0
    st = T.stats()
    for _ in range(warmup):
        T.profile()
    ms = []
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        ms.append(T.profile())
    T.close()
    kms = sum(ms) / len(ms)
    out = os.path.join(d, "transformed3")
    t0 = time.perf_counter()
    jn.transform_3nf(os.path.join(d, "comb.txt"), os.path.join(d, "anicr"), out, w["Z"], w["N"], e1,
                     os.path.join(d, "jjj"))
    e2e_s = time.perf_counter() - t0
    achieved = st["algorithmic_bytes"] / (kms / 1e3) / 1e9
    return {"workload": w["label"], "elements": st["num_elements"], "three_body_blocks": st["num_three_body_blocks"],
            "m_scheme_states": st["num_states"], "coupled_terms": st["num_terms"],
            "file_states": st["file_states"], "file_elements": st["file_elements"],
            "kernel_ms": kms, "elements_per_s": st["num_elements"] / (kms / 1e3),
            "roofline": {"bound": "fp64 pipe", "fp64_pipe_busy_ncu": 0.791,
                         "profile": "profiles/jn_jjj_to_m_kernel_li6_nmax4.md",
                         "hbm_achieved": achieved, "hbm_peak": peak, "unit": "GB/s", "hbm_frac": achieved / peak,
                         "bytes_per_run": st["algorithmic_bytes"],
                         "kernel": "jn_jjj_inner_kernel + jn_jjj_to_m_kernel"},
            "dense_equivalent_flops": st["dense_flops"],
            "dense_equivalent_tflop_per_s": st["dense_flops"] / (kms / 1e3) / 1e12,
            "plan_seconds": st["plan_seconds"], "open_seconds": open_s,
            "e2e": {"seconds": e2e_s, "what": "jn_transform_3nf: plan + upload + kernel + copy back + files"},
            "l2": "flushed between timed runs (256 MiB write)", "steps": steps, "warmup": warmup}


LARGE_SOLVE_WORKLOAD = dict(Z=3, N=3, nmax=6, M2=2,
                            label="6Li (Z=3,N=3) Nmax=6, 2M=2: two-body elements from the GPU J->M transform of a "
                                  "seeded J-scheme file (Antoine format, N(0,1) MeV), seeded three-body M-scheme "
                                  "elements N(0,0.1) MeV")


def large_solve_leg(workdir, steps, warmup, flush, max_iterations=300, check_every=10):
    """The largest single-GPU configuration end to end: the J-scheme two-body
    interaction goes through the GPU J->M transform into M-scheme blocks,
    joined by the seeded three-body blocks, and feeds the product; Lanczos
    finds the 10 lowest eigenvalues to 1e-6 MeV in at most 300 iterations,
    plain FP64-grade (exact-integer products) and mixed precision (FP32
    products, FP64 recurrence, full reorthogonalisation and an FP64-grade
    Rayleigh-Ritz refinement), both checking convergence every 10 steps.
    The time per step beside the product kernel's shows what the rest of a
    step costs."""
    import numpy as np
    import torch
    import jupiterncsm_gb300 as jn
    w = LARGE_SOLVE_WORKLOAD
    d = os.path.join(workdir, "li6_nmax6_jscheme_3nf")
    stamp = os.path.join(d, ".complete")
    if not os.path.exists(stamp):
        g = jn.generate(d, Z=w["Z"], N=w["N"], nmax=w["nmax"], M2=w["M2"], nbody=3, antoine=True)
        open(stamp, "w").write(f"{g['emax_single']} {g['emax_pair']}\n")
    e1, e2 = (int(v) for v in open(stamp).read().split())
    mes = os.path.join(d, "transformed")
    t0 = time.perf_counter()
    jn.transform_2nf(os.path.join(d, "comb.txt"), os.path.join(d, "anicr"), mes, w["Z"], w["N"], e1, e2,
                     os.path.join(d, "antoine_2nf.bin"))
    transform_s = time.perf_counter() - t0
    # the three-body blocks (written by the generator) beside the transform's one- and two-body blocks
    for f in os.listdir(os.path.join(d, "matrix_elements")):
        if not os.path.exists(os.path.join(mes, f)):
            os.symlink(os.path.join(d, "matrix_elements", f), os.path.join(mes, f))
    H = jn.Hamiltonian(comb=f"{d}/comb.txt", order=f"{d}/evaluation_order.txt", lists=f"{d}/index_lists", mes=mes,
                       Z=w["Z"], N=w["N"])
    out = {"workload": w["label"], "dimension": H.dimension, "transform_e2e_seconds": transform_s,
           "check_every": check_every, "max_iterations": max_iterations}
    try:
        D = H.dimension
        x = torch.randn(D, dtype=torch.float64, device="cuda", generator=torch.Generator(device="cuda").manual_seed(3))
        y = torch.zeros_like(x)
        for name, prec in (("plain_fp64_grade", 64), ("mixed_fp32_products", 32)):
            H.set_precision(prec)
            H.set_walk_arithmetic(False)
            for _ in range(warmup):
                H.matvec_profile(x.data_ptr(), y.data_ptr())
            ks = []
            for _ in range(steps):
                flush.zero_()
                torch.cuda.synchronize()
                ks.append(H.matvec_profile(x.data_ptr(), y.data_ptr())[0])
            t0 = time.perf_counter()
            r = H.lanczos(max_iterations=max_iterations, num_eigenvalues=10, tolerance=1e-6, check_every=check_every,
                          allow_unconverged=True)
            sec = time.perf_counter() - t0
            out[name] = {"seconds": sec, "iterations": r["iterations"], "converged": r["converged"],
                         "ms_per_step": 1e3 * sec / max(r["iterations"], 1),
                         "loop_ms_per_step": 1e3 * r["iteration_seconds"] / max(r["iterations"], 1),
                         "refinement_seconds": r["refinement_seconds"],
                         "product_kernel_ms": sum(ks) / len(ks),
                         "eigenvalues_MeV": [float(v) for v in r["eigenvalues"]],
                         "residual_norms": [float(v) for v in r["residual_norms"]]}
    finally:
        H.close()
    a = np.array(out["plain_fp64_grade"]["eigenvalues_MeV"])
    b = np.array(out["mixed_fp32_products"]["eigenvalues_MeV"])
    n = min(len(a), len(b))
    out["per_state_diff_mixed_vs_plain_MeV"] = [float(v) for v in np.abs(a[:n] - b[:n])]
    out["max_eigenvalue_diff_MeV"] = float(np.abs(a[:n] - b[:n]).max()) if n else None
    return out


def per_state_leg(workdir, tol=1e-6):
    """4He Nmax 6, two- plus three-body (D = 7 916): each of the 10 lowest
    eigenvalues from the plain FP64 solver and the mixed-precision solvers
    (FP32 products with FP64 recurrence and refinement: the single solver
    and the batched one) against dense eigenvalues of the same Hamiltonian,
    assembled column by column from FP64-grade GPU products (the tests pin
    that product to the CPU reference within 1e-12)."""
    import numpy as np
    import torch
    from scipy.linalg import eigh
    import jupiterncsm_gb300 as jn
    w = WORKLOADS["he4_nmax6_2nf3nf"]
    d = prepare("he4_nmax6_2nf3nf", workdir)
    H = jn.Hamiltonian.from_dir(d, w["Z"], w["N"])
    try:
        D = H.dimension
        H.set_precision(64)
        t0 = time.perf_counter()
        e = torch.zeros(D, dtype=torch.float64, device="cuda")
        cols = torch.zeros((D, D), dtype=torch.float64, device="cuda")
        st = torch.cuda.Stream()        # the unit vectors and the products on one stream, in order
        with torch.cuda.stream(st):
            for j in range(D):
                e.zero_()
                e[j] = 1.0
                H.matvec_device(e.data_ptr(), cols[j].data_ptr(), False, st.cuda_stream)
        torch.cuda.synchronize()
        Hd = cols.cpu().numpy().T
        del cols
        dense = eigh(0.5 * (Hd + Hd.T), eigvals_only=True, subset_by_index=[0, 9])
        dense_s = time.perf_counter() - t0
        me = H.read_matrix_elements(os.path.join(d, "matrix_elements"))
        rows = {}
        H.set_precision(64)
        rows["plain_fp64"] = H.lanczos(max_iterations=400, num_eigenvalues=10, tolerance=tol)["eigenvalues"]
        H.set_precision(32)
        rows["mixed_single"] = H.lanczos(max_iterations=400, num_eigenvalues=10, tolerance=tol)["eigenvalues"]
        rows["mixed_batched"] = H.lanczos_batch([me], max_iterations=400, num_eigenvalues=10, tolerance=tol,
                                                precision=32)[0]["eigenvalues"]
    finally:
        H.close()
    table = [{"state": i, "dense_MeV": float(dense[i]),
              **{f"{k}_error_MeV": float(abs(v[i] - dense[i])) for k, v in rows.items()}} for i in range(10)]
    return {"workload": w["label"], "dimension": int(D), "tolerance_MeV": tol, "dense_seconds": dense_s,
            "max_error_MeV": {k: float(np.abs(np.asarray(v[:10]) - dense).max()) for k, v in rows.items()},
            "per_state": table,
            "dense": "eigenvalues of the matrix assembled from FP64-grade GPU products of every unit vector"}


SOLVE_FAMILY = [  # (label, Z, N, Nmax, 2M): the bases of the batched-Hamiltonian workload
    ("4He Nmax=2", 2, 2, 2, 0), ("4He Nmax=4", 2, 2, 4, 0), ("4He Nmax=6", 2, 2, 6, 0), ("6Li Nmax=4", 3, 3, 4, 2)]
SOLVE_INSTANCES = 64
SOLVE_COUPLINGS = 4


def solves_leg(workdir, seed=20261203):
    """Lanczos solves/s: 64 Hamiltonians H(c) = H0 + sum_{i=1..4} c_i H_i, c_i ~ U(-1,1),
    16 on each of four bases, to 1e-6 MeV on the 10 lowest eigenvalues.
    Plain: FP64 Lanczos (full reorthogonalisation, FP64 products) one
    Hamiltonian after another, with the same convergence-check interval (10
    steps) and the same captured-graph step as the batched solver (a batch of
    one at precision 64); the plain solver that synchronises with the host
    every step is timed beside it.  Batched: one call for all 64 instances
    of the four bases (jn_lanczos_batch_bases: every step one graph with one
    product launch for all of them), FP32 products, FP64 recurrence and FP64
    Rayleigh-Ritz refinement; one call per basis is timed beside it.  All
    start from the same vector per basis; the error of every batched
    eigenvalue is measured against the plain FP64 solve."""
    import numpy as np
    import jupiterncsm_gb300 as jn
    rng = np.random.default_rng(seed)
    per = SOLVE_INSTANCES // len(SOLVE_FAMILY)
    plain_s = sync_s = percall_s = 0.0
    opts = dict(max_iterations=300, num_eigenvalues=10, tolerance=1e-6, check_every=10, use_graph=True)
    bases, plains, details = [], [], []
    try:
        for bi, (label, Z, N, nmax, M2) in enumerate(SOLVE_FAMILY):
            d = family_dir(workdir, Z, N, nmax, M2, seed)
            H = jn.Hamiltonian.from_dir(os.path.join(d, "h0"), Z, N)
            comps = [H.read_matrix_elements(os.path.join(d, f"h{i}", "matrix_elements"))
                     for i in range(SOLVE_COUPLINGS + 1)]
            cs = rng.uniform(-1.0, 1.0, size=(per, SOLVE_COUPLINGS))
            mes = [comps[0] + sum(c[i] * comps[i + 1] for i in range(SOLVE_COUPLINGS)) for c in cs]
            start = np.random.default_rng(seed + bi).standard_normal(H.dimension)
            bases.append((H, mes, [start] * per))
            # plain FP64, sequential, graph-replayed steps, convergence checked every 10 steps
            H.lanczos_batch(mes[:1], start_vectors=[start], precision=64, **opts)     # warm-up: graph and buffers
            plain = []
            t0 = time.perf_counter()
            for me in mes:
                plain += H.lanczos_batch([me], start_vectors=[start], precision=64, **opts)
            t1 = time.perf_counter()
            # plain FP64 solver that checks (and synchronises with the host) every step, for reference
            for me in mes[:4]:
                H.set_matrix_elements(me)
                H.lanczos(max_iterations=300, num_eigenvalues=10, tolerance=1e-6, start_vector=start,
                          allow_unconverged=True)
            t2 = time.perf_counter()
            # batched mixed precision, one call for this basis alone
            H.lanczos_batch(mes, start_vectors=[start] * per, precision=32, **opts)
            t3 = time.perf_counter()
            plain_s += t1 - t0
            sync_s += (t2 - t1) * per / 4
            percall_s += t3 - t2
            plains.append(plain)
            details.append({"basis": label, "dimension": int(len(start)), "instances": per, "plain_s": t1 - t0,
                            "batched_alone_s": t3 - t2})
        # all four bases in one call; the first call (walk plans, graph) is a warm-up
        jn.lanczos_batch_bases([(H, mes[:1], sv[:1]) for H, mes, sv in bases], precision=32, **opts)
        t0 = time.perf_counter()
        res = jn.lanczos_batch_bases(bases, precision=32, **opts)
        batch_s = time.perf_counter() - t0
    finally:
        for H, _, _ in bases:
            H.close()
    worst = 0.0
    iters_plain, iters_batch = [], []
    for det, rs, plain in zip(details, res, plains):
        err = max(float(np.abs(r["eigenvalues"] - p["eigenvalues"]).max()) for r, p in zip(rs, plain))
        worst = max(worst, err)
        iters_plain += [p["iterations"] for p in plain]
        iters_batch += [r["iterations"] for r in rs]
        det["max_eigenvalue_diff_MeV"] = err
        det["all_converged"] = all(r["converged"] for r in rs) and all(p["converged"] for p in plain)
    return {"metric": "Lanczos solves/s at 1e-6 MeV (10 lowest) vs plain FP64",
            "workload": f"{SOLVE_INSTANCES} H(c)=H0+sum_{{i=1..{SOLVE_COUPLINGS}}} c_i H_i, c~U(-1,1), "
                        f"{per} on each of " + ", ".join(f[0] for f in SOLVE_FAMILY) + " (two-body, seeded)",
            "batched_solves_per_s": SOLVE_INSTANCES / batch_s, "plain_fp64_solves_per_s": SOLVE_INSTANCES / plain_s,
            "speedup": plain_s / batch_s, "batched_seconds": batch_s, "plain_seconds": plain_s,
            "batched_one_call_per_basis_solves_per_s": SOLVE_INSTANCES / percall_s,
            "plain_fp64_per_step_sync_solves_per_s": SOLVE_INSTANCES / sync_s,
            "max_eigenvalue_diff_vs_plain_fp64_MeV": worst,
            "mean_iterations": {"plain": float(np.mean(iters_plain)), "batched": float(np.mean(iters_batch))},
            "batched": "one call for all 64 instances of the four bases: FP32 products (one persistent walk-engine "
                       "launch per step for every instance), FP64 recurrence + full reorthogonalisation + "
                       "Rayleigh-Ritz refinement, CUDA graph per step, convergence checked every 10 steps",
            "plain": "FP64 products and recurrence, one Hamiltonian at a time, CUDA graph per step, convergence "
                     "checked every 10 steps (a batch of one at precision 64)",
            "per_basis": details}


WARM_BASIS = ("6Li Nmax=4", 3, 3, 4, 2)
WARM_TRAIN, WARM_TEST, WARM_PLAIN = 256, 64, 16


def family_dir(workdir, Z, N, nmax, M2, seed=20261203):
    """H0 and the couplings' operators H_1..H_4 of one basis (generated once)."""
    import jupiterncsm_gb300 as jn
    d = os.path.join(workdir, f"family_{Z}_{N}_{nmax}_{M2}")
    stamp = os.path.join(d, ".complete")
    if not os.path.exists(stamp):
        jn.generate(os.path.join(d, "h0"), Z=Z, N=N, nmax=nmax, M2=M2, nbody=2, basis_files=False)
        for i in range(1, SOLVE_COUPLINGS + 1):
            jn.generate(os.path.join(d, f"h{i}"), Z=Z, N=N, nmax=nmax, M2=M2, nbody=2, seed=seed + 1000 * i,
                        hbar_omega=0.0, basis_files=False)
        open(stamp, "w").write("ok\n")
    return d


def warm_start_leg(workdir, seed=20261203, check_every=5):
    """The learned warm start (6Li Nmax=4, 4 couplings): 256 training solves by
    the batched solver give the snapshots; the MLP is trained on the GPU; 64
    held-out Hamiltonians are solved from the default start and from the
    network's start vectors.  Plain FP64 Lanczos on 16 of the held-out ones
    gives the per-solve time of the plain method and the eigenvalue oracle."""
    import numpy as np
    import jupiterncsm_gb300 as jn
    label, Z, N, nmax, M2 = WARM_BASIS
    d = family_dir(workdir, Z, N, nmax, M2, seed)
    rng = np.random.default_rng(seed + 77)
    cs = rng.uniform(-1.0, 1.0, size=(WARM_TRAIN + WARM_TEST, SOLVE_COUPLINGS))
    H = jn.Hamiltonian.from_dir(os.path.join(d, "h0"), Z, N)
    try:
        comps = [H.read_matrix_elements(os.path.join(d, f"h{i}", "matrix_elements"))
                 for i in range(SOLVE_COUPLINGS + 1)]
        mes = [comps[0] + sum(c[i] * comps[i + 1] for i in range(SOLVE_COUPLINGS)) for c in cs]
        t0 = time.perf_counter()
        _, vecs = H.lanczos_batch(mes[:WARM_TRAIN], max_iterations=300, num_eigenvalues=10, tolerance=1e-6,
                                  eigenvectors=10, check_every=check_every)
        t1 = time.perf_counter()
        ws = jn.WarmStart(cs[:WARM_TRAIN], vecs, hidden=128, basis_size=32, train_steps=3000, seed=0)
        t2 = time.perf_counter()
        del vecs
        test = mes[WARM_TRAIN:]
        starts = ws.start_vectors(cs[WARM_TRAIN:])
        t3 = time.perf_counter()
        cold = H.lanczos_batch(test, max_iterations=300, num_eigenvalues=10, tolerance=1e-6, check_every=check_every)
        t4 = time.perf_counter()
        warm = H.lanczos_batch(test, start_vectors=starts, max_iterations=300, num_eigenvalues=10, tolerance=1e-6,
                               check_every=check_every)
        t5 = time.perf_counter()
        # plain FP64, one Hamiltonian at a time, with the same check interval and graph replay
        H.lanczos_batch(test[:1], max_iterations=300, num_eigenvalues=10, tolerance=1e-6, precision=64,
                        check_every=check_every, use_graph=True)
        t5 = time.perf_counter()
        plain = []
        for me in test[:WARM_PLAIN]:
            plain += H.lanczos_batch([me], max_iterations=300, num_eigenvalues=10, tolerance=1e-6, precision=64,
                                     check_every=check_every, use_graph=True)
        t6 = time.perf_counter()
        ws.close()
    finally:
        H.close()
    err_w = max(float(np.abs(w["eigenvalues"] - p["eigenvalues"]).max()) for w, p in zip(warm, plain))
    err_c = max(float(np.abs(c["eigenvalues"] - p["eigenvalues"]).max()) for c, p in zip(cold, plain))
    plain_per = (t6 - t5) / WARM_PLAIN
    return {"workload": f"{label}: H(c)=H0+sum_{{i=1..{SOLVE_COUPLINGS}}} c_i H_i, c~U(-1,1); MLP "
                        f"{SOLVE_COUPLINGS}->128->128->32 (GELU) trained on {WARM_TRAIN} solves, {WARM_TEST} held out",
            "dimension": int(len(starts[0])),
            "snapshot_solves_seconds": t1 - t0, "fit_seconds": t2 - t1, "start_vectors_seconds": t3 - t2,
            "final_training_loss": ws.final_loss,
            "cold_batched_solves_per_s": WARM_TEST / (t4 - t3),
            "warm_batched_solves_per_s": WARM_TEST / (t5 - t4 + t3 - t2),
            "plain_fp64_solves_per_s": 1.0 / plain_per,
            "warm_batched_vs_plain_fp64": plain_per * WARM_TEST / (t5 - t4 + t3 - t2),
            "mean_iterations": {"cold": float(np.mean([c["iterations"] for c in cold])),
                                "warm": float(np.mean([w["iterations"] for w in warm])),
                                "plain_fp64": float(np.mean([p["iterations"] for p in plain]))},
            "max_eigenvalue_diff_vs_plain_fp64_MeV": {"warm": err_w, "cold": err_c},
            "all_converged": all(r["converged"] for r in cold + warm),
            "check_every": check_every,
            "note": "warm time includes computing the start vectors; plain FP64 (one Hamiltonian at a time, "
                    f"graph-replayed steps, convergence checked every {check_every} steps) timed on "
                    f"{WARM_PLAIN} of the held-out Hamiltonians"}


def cpu_baseline(d, w, bytes_per_step, seconds=10.0, min_steps=3, x=None):
    """The reference's CPU algorithm on all host threads over a time-bounded
    sample; with x, also its y = H x (the reference for the GPU paths' errors)."""
    import numpy as np
    import oracle
    threads = os.cpu_count() or 1
    kind = "port"
    impl = None
    if oracle.reference_available():
        try:
            impl = oracle.Reference(d, w["Z"], w["N"], threads=threads)
            kind = "reference"
        except OSError:
            impl = None
    if impl is None:
        impl = oracle.Port(d)
    D = impl.dimension
    x = np.random.default_rng(1).standard_normal(D) if x is None else x
    y = np.zeros(D)
    times = []
    t_end = time.perf_counter() + seconds
    while len(times) < min_steps or time.perf_counter() < t_end:
        y[:] = 0.0
        if kind == "reference":
            impl.matvec(x, y)
            times.append(impl.seconds)
        else:
            times.append(impl.matvec_omp(x, y, threads))
    impl.close()
    per = sum(times) / len(times)
    return {"value": bytes_per_step / per / 1e9, "unit": "GB/s", "cores": threads, "kind": kind,
            "sample": f"{len(times)} full products of the workload ({sum(times):.1f} s of CPU work), "
                      f"OpenMP task farm with per-thread replicas, {threads} threads",
            "ms_per_step": per * 1e3}, y


def product_leg(args):
    """Diagnostic: --steps products y = H x of --workload with the chosen engine
    and arithmetic, each after the L2 flush, with the product kernel's
    CUDA-event time (the target of the ncu captures under profiles/)."""
    import numpy as np
    import torch
    import jupiterncsm_gb300 as jn
    w = WORKLOADS[args.workload]
    d = prepare(args.workload, args.workdir)
    H = jn.Hamiltonian.from_dir(d, w["Z"], w["N"])
    try:
        if args.engine:
            H.set_engine(args.engine)
        prec, fma = ARITH[args.arith]
        H.set_precision(prec)
        if H.active_engine() == 5:
            H.set_walk_arithmetic(fma)
        D = H.dimension
        x = torch.from_numpy(np.random.default_rng(3).standard_normal(D)).cuda()
        y = torch.zeros(D, dtype=torch.float64, device="cuda")
        flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
        ms = []
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            ms.append(H.matvec_profile(x.data_ptr(), y.data_ptr())[0])
        return {"workload": w["label"], "dimension": D, "engine": H.active_engine(), "arith": args.arith,
                "kernel_ms": ms}
    finally:
        H.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="li6_nmax6_2nf3nf", choices=sorted(WORKLOADS))
    ap.add_argument("--workdir", default=os.environ.get("JNCSM_BENCH_DIR", os.path.join(tempfile.gettempdir(), "jncsm_bench")))
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--arith", default="i64", choices=sorted(ARITH),
                    help="the headline product: i64 exact integers (FP64-grade), fp64 FP64 FMAs, f32 FP32")
    ap.add_argument("--no-transform", action="store_true", help="skip the J->M transform legs")
    ap.add_argument("--no-solves", action="store_true", help="skip the Lanczos solve legs")
    ap.add_argument("--schedule", metavar="ROWS,CTAS",
                    help="fix the panel schedule (rows per lane, CTAs per SM) instead of autotuning it "
                         "(panel-engine workloads)")
    ap.add_argument("--leg", choices=["transform", "transform3", "product", "large_solve"],
                    help="run only this leg and print its JSON (a diagnostic run, e.g. under ncu; not the bench line); "
                         "product: --steps products of --workload on --engine in --arith, timed with CUDA events; "
                         "large_solve: the 6Li Nmax 6 2+3NF solves, --max-iterations steps at most")
    ap.add_argument("--max-iterations", type=int, default=300, help="Lanczos steps at most (--leg large_solve)")
    ap.add_argument("--engine", type=int, choices=[2, 3, 4, 5], help="the product engine (--leg product)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.leg == "product":
        print(json.dumps({"product": product_leg(args)}), flush=True)
        return
    if args.leg:
        import torch
        flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
        if args.leg == "large_solve":
            print(json.dumps({"large_solve": large_solve_leg(args.workdir, args.steps, args.warmup, flush,
                                                             max_iterations=args.max_iterations)}), flush=True)
            return
        peaks = measured_peaks()
        leg = transform_leg if args.leg == "transform" else transform3_leg
        print(json.dumps({args.leg: leg(args.workdir, args.steps, args.warmup, flush,
                                         peaks["hbm_gbs"] if peaks else 6800.0)}), flush=True)
        return

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    w = WORKLOADS[args.workload]

    if args.impl == "reference":
        if rank != 0:
            return
        import jupiterncsm_gb300 as jn
        d = prepare(args.workload, args.workdir)
        stats = algorithmic_stats(d, w)
        cb, _ = cpu_baseline(d, w, stats["bytes"], seconds=args.cpu_seconds)
        line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": "GB/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": cb["ms_per_step"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": w["label"], "dimension": stats["dimension"], "threads": cb["cores"],
                           "bytes_per_step": stats["bytes"]},
                "cpu_baseline": cb,
                "e2e": {"value": cb["value"], "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    import torch
    import numpy as np
    import jupiterncsm_gb300 as jn

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as tdist
        tdist.init_process_group("nccl")
        dist = tdist
    wd = os.path.join(args.workdir, f"rank{rank}") if world > 1 else args.workdir
    d = prepare(args.workload, wd)
    t0 = time.perf_counter()
    H = jn.Hamiltonian.from_dir(d, w["Z"], w["N"])
    open_s = time.perf_counter() - t0
    st = H.stats()
    D = H.dimension
    dev = torch.device("cuda", local)
    x = torch.randn(D, dtype=torch.float64, device=dev, generator=torch.Generator(device=dev).manual_seed(7))
    y = torch.zeros(D, dtype=torch.float64, device=dev)
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    engine = H.active_engine()

    # bytes of one product in the reference's FP64 terms: lists (12 B/entry), referenced matrix elements
    # (8 B), x and y (FP64); the FP32 path moves 4-byte elements
    def bytes_for(arith):
        return 12.0 * st["list_entries"] + (4 if arith == "f32" else 8) * st["me_referenced"] + 16.0 * D

    def set_arith(arith):
        prec, fma = ARITH[arith]
        H.set_precision(prec)
        if engine == 5:
            H.set_walk_arithmetic(fma)

    def timed(arith):
        """K products, each preceded by the L2 flush, all enqueued on one stream
        without host synchronisation; each product is bracketed by CUDA events
        on that stream, so a step is the device time of one product (its
        kernels and the gaps between them).  Then K profiled products give the
        product kernel's own duration."""
        set_arith(arith)
        s = torch.cuda.Stream(device=dev)

        def run_steps(k):
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(k)]
            with torch.cuda.stream(s):
                for a, b in ev:
                    flush.zero_()
                    a.record(s)
                    H.matvec_device(x.data_ptr(), y.data_ptr(), False, s.cuda_stream)
                    b.record(s)
            return ev

        torch.cuda.synchronize()
        t0 = time.perf_counter()
        run_steps(1)            # builds the arithmetic's element arrays on first use
        torch.cuda.synchronize()
        setup_s = time.perf_counter() - t0
        run_steps(args.warmup)
        torch.cuda.synchronize()
        sampler = ClockSampler(local)
        sampler.start()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        wall0 = time.perf_counter()
        ev = run_steps(args.steps)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        wall = time.perf_counter() - wall0
        clocks = sampler.stop()
        total_ms = sum(a.elapsed_time(b) for a, b in ev)
        kern_ms, prof_total = 0.0, 0.0
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            k, r = H.matvec_profile(x.data_ptr(), y.data_ptr(), accumulate=False)
            kern_ms += k
            prof_total += k + r
        t_max = max_over_ranks(total_ms, dist, dev)
        return {"ms_per_step": t_max / args.steps, "kernel_ms": kern_ms / args.steps, "wall_s": wall,
                "profiled_ms_per_step": prof_total / args.steps, "clocks": clocks, "setup_s": setup_s,
                "y": y.cpu().numpy().copy()}

    tuning = None
    if engine == 4:
        set_arith(args.arith)
        if args.schedule:
            rows, ctas = (int(v) for v in args.schedule.split(","))
            H.set_panel_schedule(rows, ctas)
            tuning = {"engine": 4, "rows_per_lane": rows, "ctas_per_sm": ctas, "fixed": True}
        else:
            tuning = H.autotune(trials=5)
    order = [args.arith] + [a for a in ("i64", "fp64", "f32") if a != args.arith and (engine == 5 or a != "fp64")]
    runs = {a: timed(a) for a in order}
    main_r = runs[args.arith]
    bytes_step = bytes_for("i64")                      # the reference's FP64 bytes, whatever the arithmetic
    value = job_gbs(bytes_step, world, main_r["ms_per_step"] / 1e3)

    # end to end through the public host-pointer call, pinned host buffers
    set_arith(args.arith)
    hx = torch.randn(D, dtype=torch.float64).pin_memory().numpy()
    hy = torch.zeros(D, dtype=torch.float64).pin_memory().numpy()
    for _ in range(args.warmup):
        H.matvec(hx, hy)
    e2e_s = 0.0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        H.matvec(hx, hy)
        e2e_s += time.perf_counter() - t0
    e2e_value = job_gbs(bytes_step, world, max_over_ranks(e2e_s, dist, dev) / args.steps)

    peaks = measured_peaks()
    peak = peaks["hbm_gbs"] if peaks else 6800.0
    achieved = bytes_step / (main_r["kernel_ms"] / 1e3) / 1e9
    traffic = profile_traffic(args.workload, engine, args.arith)
    wstats = H.walk_stats() if engine == 5 else None

    def path_summary(r, a):
        return {"ms_per_step": r["ms_per_step"], "GB_per_s_fp64_bytes": bytes_step / (r["ms_per_step"] / 1e3) / 1e9,
                "own_bytes_per_step": bytes_for(a), "product_kernel_ms": r["kernel_ms"],
                "profiled_ms_per_step": r["profiled_ms_per_step"],
                "hbm_frac_fp64_bytes": bytes_step / (r["kernel_ms"] / 1e3) / 1e9 / peak,
                "multiply_adds_per_s": st["multiply_adds"] / (r["kernel_ms"] / 1e3),
                "first_product_setup_s": r["setup_s"]}

    line = {"metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": main_r["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": {"i64": "i64", "fp64": "f64", "f32": "f32"}[args.arith],
            "arithmetic": {"i64": "exact integers: FP64 matrix elements (each block at its own exponent) and x as "
                                  "52-bit fixed-point integers split 28+24 bits, three 32x32->64-bit integer "
                                  "multiply-adds per contribution, exact sums, one rounding per row sum; FP64 x and "
                                  "y at the interface; error against the CPU reference in paths",
                           "fp64": "FP64 fused multiply-adds, one rounding per row sum into exact 64-bit sums",
                           "f32": "FP32 matrix elements and x, FP32 fused multiply-adds, exact 64-bit sums"}[args.arith],
            "data": "synthetic",
            "config": {"workload": w["label"], "dimension": D, "instructions": st["num_instructions"],
                       "list_entries": st["list_entries"], "me_elements": st["me_elements"],
                       "me_elements_referenced": st["me_referenced"],
                       "multiply_adds": st["multiply_adds"], "bytes_per_step": bytes_step,
                       "bytes_formula": "12 x list entries + 8 x referenced matrix elements + 16 x D (the reference arm's)",
                       "l2": "flushed between timed steps (256 MiB write)", "parallelism": f"replicas x{world}",
                       "timing": "CUDA events on the product's stream around each product; flush and products "
                                 "enqueued without host synchronisation; the product kernel's duration from a "
                                 "second pass with events around the kernel",
                       "engine": engine, "open_seconds": open_s, "schedule": tuning, "walk_plan": wstats},
            "paths": {a: path_summary(runs[a], a) for a in order},
            "e2e": {"value": e2e_value, "unit": "GB/s", "h2d_bytes_per_step": 16 * D, "d2h_bytes_per_step": 8 * D},
            "gpu_launches": LAUNCHES.get((engine, args.arith), 3) * args.steps,
            "engine": engine,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (burst copy)" if peaks else "fallback 6.8 TB/s",
                         "kernel": KERNELS.get((engine, args.arith))},
            "clocks": main_r["clocks"]}
    if rank == 0:
        try:
            cb, y_ref = cpu_baseline(d, w, bytes_step, seconds=args.cpu_seconds, x=x.cpu().numpy())
            line["cpu_baseline"] = cb
            scale = float(np.abs(y_ref).max())
            for a in order:
                line["paths"][a]["max_rel_err_vs_cpu_reference"] = float(np.abs(runs[a]["y"] - y_ref).max()) / scale
        except Exception as e:  # the baseline must never hide the GPU line
            line["cpu_baseline"] = {"error": str(e)}
    H.close()
    if rank == 0 and not args.no_solves:
        try:
            line["large_solve"] = large_solve_leg(wd, min(args.steps, 10), args.warmup, flush)
        except Exception as e:
            line["large_solve"] = {"error": str(e)}
    if rank == 0 and not args.no_transform:
        try:
            line["transform"] = transform_leg(wd, args.steps, args.warmup, flush, peak)
        except Exception as e:  # the transform leg must never hide the matvec line
            line["transform"] = {"error": str(e)}
        try:
            line["transform3"] = transform3_leg(wd, min(args.steps, 10), args.warmup, flush, peak)
        except Exception as e:
            line["transform3"] = {"error": str(e)}
    if rank == 0 and not args.no_solves:
        try:
            line["per_state"] = per_state_leg(wd)
        except Exception as e:
            line["per_state"] = {"error": str(e)}
        try:
            line["solves"] = solves_leg(wd)
        except Exception as e:  # the solves leg must never hide the matvec line
            line["solves"] = {"error": str(e)}
        try:
            line["warm_start"] = warm_start_leg(wd)
        except Exception as e:
            line["warm_start"] = {"error": str(e)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def algorithmic_stats(d, w):
    """Bytes per product from the plan statistics, computed on the host (no GPU needed)."""
    import jupiterncsm_gb300 as jn
    st = jn.inspect(d, w["Z"], w["N"])
    return {"bytes": st["algorithmic_bytes"], "dimension": st["dimension"]}


if __name__ == "__main__":
    main()
