"""Benchmark: verified resonances per second of the plain sweep.

Workload (one step): the plain resonance search on the circular scatterer of
the reference's CPU-runnable configuration -- radius 0.25, N = 50 circular-arc
panels, c_i = 23.4, c_o = 1, Gauss order 11, continuous P1 spaces (T(k) is
100 x 100 complex128) -- over k in [0.5, 10] on 200 grid points: sigma_min
by dense SVD at every grid point, 3-point local minima, sigma' at both bracket
ends and validation sigma'(left) < 0 < sigma'(right), quartic/Brent guess,
safeguarded Newton on sigma' with sigma'' to |dk| <= 1e-8, then every root
verified by a sign change of sigma' across [root - 1e-8, root + 1e-8].

  value : verified roots / s with the mesh resident on the device (builder and
          solutions operator created once, outside the timed region)
  e2e   : the same through the public C ABI from host data: builder + operator
          creation (mesh upload), the search and the root read-back, per step

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl {gb300,reference}]
"""
import argparse
import math
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
# 32 hardware work queues for the search's many streams (the package sets the same
# default on import; here it must precede torch's CUDA initialisation)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

CFG = dict(radius=0.25, N=50, c_i=23.4, c_o=1.0, order=11, k_min=0.5, k_max=10.0, npoints=200, tol=1e-8)
WORKLOAD = ("plain sweep: circle r=0.25, N=50 arc panels, c_i=23.4, c_o=1, Gauss order 11, P1/P1 "
            "(T 100x100 c128), k in [0.5,10] x 200, dense sigma on the grid, sigma' at bracket ends, "
            "Newton on sigma' with sigma'' to |dk|<=1e-8")
METRIC = "verified resonances/sec at |dk|<=1e-8 (plain sweep)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--skip-cpu", action="store_true", help="omit the CPU-baseline leg")
    ap.add_argument("--profile-search", action="store_true",
                    help="no timing: one plain search of the workload (for launch-list captures)")
    ap.add_argument("--profile-dense-tail", action="store_true",
                    help="no timing: FP64 and complex-FP32 LU + rSVD of 4 matrices of order 1600 (for captures)")
    ap.add_argument("--profile-case", action="store_true",
                    help="no timing: three sigma sweeps over 16 wavenumbers of the workload (for ncu captures)")
    ap.add_argument("--full-configs", action="store_true",
                    help="one run of the batching configuration at its full size (8 scatterers x 256 k) and "
                         "of the precision configuration at all eight wavenumbers 40..47; prints one JSON line")
    ap.add_argument("--profile-lu", action="store_true",
                    help="one complex-FP32 LU of order 8000 (for ncu captures of the tensor-core update)")
    ap.add_argument("--profile-field", action="store_true",
                    help="no timing: the field-at-scale scatterer lifted on a 160 x 160 grid (for ncu captures)")
    return ap.parse_args()


def run_profile_field():
    """The field_at_scale scatterer and wave, traces solved once, total field on a
    160 x 160 grid over [-1.6, 1.6]^2 with 16 Gauss points per panel."""
    from helmholtzbem_gb300 import api, geometry
    x, y = geometry.star_polygon(24, seed=2)
    so = api.SolutionsOperator(api.BuilderData(geometry.polygon_graded(x, y, 400, 0.5), order=11), proj=False)
    w = api.wave("Plane", 1.0, angle=math.pi / 3)
    tr = api.tp_solve(so, w, 10.0, 1.0, 4.0)
    S, _, _ = api.tp_field_grid(so, w, 10.0, 1.0, 4.0, 16, (-1.6, -1.6), (1.6, 1.6), 160, 160, total_field=True,
                                traces=tr)
    print("profile field done, max |u| = %.6e" % float(np.max(np.abs(S))))


def run_profile_case():
    """Small fixed case for profiler captures: 3 x hbem_sweep_sigma over 16 k of the
    workload's scatterer (each sweep: assembly, T gather, projection, dense SVD)."""
    from helmholtzbem_gb300 import api, geometry
    data = api.BuilderData(geometry.circle(CFG["radius"], CFG["N"]), order=CFG["order"])
    so = api.SolutionsOperator(data)
    ks = np.linspace(CFG["k_min"], CFG["k_max"], 16)
    for _ in range(3):
        out = so.sweep_sigma(ks, CFG["c_o"], CFG["c_i"], d=2)
    print("profile case done, sigma_min(k0) = %.6e" % out[0, 0])


def run_profile_search():
    """One step of the workload: the plain search with every root checked (grid, bracket-end
    sigma', Newton runs and the roots' sign-change checks, as the timed step)."""
    from helmholtzbem_gb300 import api, geometry
    data = api.BuilderData(geometry.circle(CFG["radius"], CFG["N"]), order=CFG["order"])
    so = api.SolutionsOperator(data)
    roots, grid, nev, chk = so.find_resonances_plain_verified(CFG["k_min"], CFG["k_max"], CFG["npoints"], CFG["c_o"],
                                                              CFG["c_i"], tol=CFG["tol"])
    print("profile search done: %d roots, %d T(k) evaluations" % (roots.size, nev))


def run_profile_dense_tail():
    """Batched LU (complex128 and complex64) and randomized SVD (FP64 and mixed) of
    four matrices of order 1600 from the star polygon N = 800 at k = 3, 7.5, 12.25, 19."""
    import ctypes
    import torch
    from helmholtzbem_gb300 import _capi as C, api, geometry
    data = api.BuilderData(geometry.polygon(*geometry.star_polygon(24, seed=2), 800), order=11)
    so = api.SolutionsOperator(data)
    n, nk = 1600, 4
    ks = np.array([3.0, 7.5, 12.25, 19.0])
    T = torch.empty((nk, n, n), dtype=torch.complex128, device="cuda")
    L = C.lib()
    C.check(L.hbem_gen_sol_op_batch_device(so._h, C.dptr(ks), nk, 1.0, 9.0, 0, ctypes.c_void_p(T.data_ptr())))
    R = torch.from_numpy(np.ascontiguousarray(api.randGaussian(n, 12, seed=1).T)).cuda()
    out = np.zeros(nk)
    for prec in (0, 1):
        C.check(L.hbem_rsvd_sv_batch_device_ex(n, nk, 0, ctypes.c_void_p(T.data_ptr()), n * n, n * n,
                                               ctypes.c_void_p(R.data_ptr()), 12, 2, prec, 3, C.dptr(out)))
    print("profile dense tail done, sigma = %s" % out)


def run_profile_lu():
    """The complex-FP32 LU of one matrix of order 8000 (the precision configuration's
    size; a random complex matrix with a dominant diagonal stands in for T(k)): 62
    depth-128 tensor-core trailing updates, each preceded by four panel
    factorisations and a block triangular solve."""
    import ctypes
    import torch
    from helmholtzbem_gb300 import _capi as C
    n = 8000
    g = torch.Generator(device="cuda").manual_seed(8000)
    A = torch.randn((n, n), dtype=torch.complex64, device="cuda", generator=g)
    A += 3.0 * math.sqrt(n) * torch.eye(n, dtype=torch.complex64, device="cuda")
    piv = torch.zeros(n, dtype=torch.int32, device="cuda")
    C.check(C.lib().hbem_lu_factor_batch_device_f32(n, 1, ctypes.c_void_p(A.data_ptr()), n * n,
                                                    ctypes.c_void_p(piv.data_ptr()), None))
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    A2 = torch.randn((n, n), dtype=torch.complex64, device="cuda", generator=g)
    A2 += 3.0 * math.sqrt(n) * torch.eye(n, dtype=torch.complex64, device="cuda")
    ev[0].record()
    C.check(C.lib().hbem_lu_factor_batch_device_f32(n, 1, ctypes.c_void_p(A2.data_ptr()), n * n,
                                                    ctypes.c_void_p(piv.data_ptr()), None))
    ev[1].record()
    torch.cuda.synchronize()
    print("profile lu done: n = %d, %.2f ms" % (n, ev[0].elapsed_time(ev[1])))


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


# ------------------------------------------------------------------ clocks

class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ CPU leg (oracle port)

L2_NOTE = "GPU arm: a 256 MB buffer (> 129 MB L2) is written between timed steps; CPU arm: not applicable"
CONFIG = {"workload": WORKLOAD, "l2": L2_NOTE}


def grid_ks():
    h = (CFG["k_max"] - CFG["k_min"]) / (CFG["npoints"] - 1)
    return CFG["k_min"] + h * np.arange(CFG["npoints"])


def sweep_pool():
    """The oracle port of the reference's plain search with the reference driver's
    parallel structure (grid, bracket ends and Newton searches over all host cores)."""
    from oracle import oracle as O
    kinds, par = O.circle_panels(CFG["radius"], CFG["N"])
    return O.SweepPool(kinds, par, CFG["order"], CFG["c_o"], CFG["c_i"])


def cpu_search(pool):
    """One step of the workload on the host cores: the plain search over all 200 grid
    points plus the verification of its roots.  Returns (verified, seconds, roots, grid
    sigma, evaluations)."""
    t0 = time.perf_counter()
    roots, sig, nev = pool.plain_sweep(grid_ks(), tol=CFG["tol"])
    ok = pool.verify(roots, tol=CFG["tol"])
    return int(ok.sum()), time.perf_counter() - t0, roots, sig, nev + 2 * roots.size


CPU_SAMPLE = "the whole workload per step: all 200 grid points, bracket ends, Newton searches and verification"


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    pool = sweep_pool()   # worker processes start outside the timed region
    try:
        for _ in range(max(0, args.warmup)):
            pool.evald(list(grid_ks()[:pool.workers]), 0)   # bounded warm-up: one grid point per worker
        tot_v, tot_t = 0, 0.0
        for _ in range(args.steps):
            v, t, _, _, _ = cpu_search(pool)
            tot_v += v
            tot_t += t
    finally:
        pool.close()
    val = tot_v / tot_t if tot_t > 0 else 0.0
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": "resonances/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_t / max(1, args.steps),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": CONFIG,
        "workload_stats": {"roots_per_step": tot_v / max(1, args.steps)},
        "cpu_baseline": {"value": val, "unit": "resonances/s", "cores": pool.workers, "kind": "port",
                         "sample": CPU_SAMPLE},
        "e2e": {"value": val, "unit": "resonances/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


# ------------------------------------------------------------------ GPU leg

def nominal_fp64_tflops(sm_mhz=2070.0, sms=152):
    """2 DFMA (4 flops) per cycle per SM."""
    return 4.0 * sms * sm_mhz * 1e6 / 1e12


def fp64_peak_tflops():
    """Measured FP64 peak: cuBLAS DGEMM 8192^3 through torch (best of 5)."""
    import torch
    n = 8192
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = max(best, 2.0 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    del a, b
    return best


def assembly_at_scale(torch, C, api, geometry, lib, peak):
    """Assembly-at-scale configuration: seeded star polygon (24 vertices, r = 1 + 0.3 u),
    N = 1000 line panels, Gauss order 16, c_i = 4, c_o = 1, k = 20: T, T', T'' (2000 x
    2000 complex128, both media, projected) on the device.  Reports T-sets/s and the
    assembly kernels' algorithmic FP64 rate (CUDA events on their stream)."""
    N, order, k = 1000, 16, 20.0
    data = api.BuilderData(geometry.polygon(*geometry.star_polygon(24, seed=2), N), order=order)
    so = api.SolutionsOperator(data)
    n = 2 * N
    T = torch.empty((3, n, n), dtype=torch.complex128, device="cuda")
    ks = np.array([k])

    def one():
        C.check(lib.hbem_gen_sol_op_batch_device(so._h, C.dptr(ks), 1, 1.0, 4.0, 2, C.ctypes.c_void_p(T.data_ptr())))

    one()
    torch.cuda.synchronize()
    lib.hbem_stats_reset()
    lib.hbem_stats_enable_timing(1)
    reps = 2
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        one()
    e1.record()
    torch.cuda.synchronize()
    lib.hbem_stats_enable_timing(0)
    ms = e0.elapsed_time(e1) / reps
    launches, asm_ms, asm_l, asm_pts = (C.ctypes.c_longlong(), C.ctypes.c_double(), C.ctypes.c_longlong(),
                                        C.ctypes.c_longlong())
    lib.hbem_stats_read(C.ctypes.byref(launches), C.ctypes.byref(asm_ms), C.ctypes.byref(asm_l),
                        C.ctypes.byref(asm_pts))
    achieved = assembly_flops(C, lib) / (asm_ms.value * 1e-3) / 1e12 if asm_ms.value > 0 else 0.0
    del T
    return {"workload": "star polygon 24 vertices (seed 2), N=1000 lines, order 16, k=20, c_i=4, c_o=1, "
                        "T/T'/T'' 2000x2000 c128 projected",
            "ms_per_T_set": ms, "T_sets_per_s": 1e3 / ms,
            "quad_points_per_T_set": asm_pts.value // reps,
            "assembly_ms_per_T_set": asm_ms.value / reps,
            "assembly_fp64_tflops": achieved, "assembly_frac_of_measured_fp64": achieved / peak if peak else None,
            "assembly_frac_of_nominal_fp64": achieved / nominal_fp64_tflops(),
            "note": "algorithmic flops (the reference's per-point work); a fraction above 1 means this build "
                    "executes fewer FP64 instructions per point than that count credits, not a rate above the pipe's"}


def assembly_flops(C, lib):
    """Algorithmic FP64 flops of the timed assembly launches: per quadrature point and
    medium F(d) = 130 (Hankel pair) + 50 (geometry and weights) + 100 (d + 1) (kernel
    values and moment updates of orders 0..d); singular-pair points whose geometry
    comes from the builder's k-independent table do not repeat the 50."""
    split = (C.ctypes.c_longlong * 9)()
    lib.hbem_stats_read_points(split)
    f = 0.0
    for d in range(3):
        f += split[d] * (180.0 + 100.0 * (d + 1))
        f += split[3 + d] * (130.0 + 100.0 * (d + 1))
        f += split[6 + d] * (180.0 + 100.0 * (d + 1))
    return f


def dense_tail_at_scale(torch, C, api, geometry, lib, peak, nk=16):
    """Largest scatterer of the batching configuration: star polygon (24 vertices,
    seed 2), N = 800 line panels (T of order 1600), order 11, c_i = 9, c_o = 1; nk
    wavenumbers uniform on [1, 30] assembled in one batch, then randomized_svd::sv
    (sketch 12, 2 subspace steps) on all of them.  Reports T(k)/s for assembly and
    for the rSVD, and the batched LU's algorithmic FP64 rate ((8/3) n^3 real flops
    per matrix, CUDA events on the launching stream)."""
    N, order = 800, 11
    n = 2 * N
    data = api.BuilderData(geometry.polygon(*geometry.star_polygon(24, seed=2), N), order=order)
    so = api.SolutionsOperator(data)
    ks = np.random.default_rng(3000).uniform(1.0, 30.0, nk)
    T = torch.empty((nk, n, n), dtype=torch.complex128, device="cuda")
    R = torch.from_numpy(np.ascontiguousarray(api.randGaussian(n, 12, seed=3000).T)).cuda()
    A = torch.empty_like(T)
    piv = torch.empty(nk * n, dtype=torch.int32, device="cuda")
    out = np.zeros(nk)
    ev = lambda: torch.cuda.Event(enable_timing=True)   # noqa: E731

    def assemble():
        C.check(lib.hbem_gen_sol_op_batch_device(so._h, C.dptr(ks), nk, 1.0, 9.0, 0, C.ctypes.c_void_p(T.data_ptr())))

    def lu():
        A.copy_(T)
        C.check(lib.hbem_lu_factor_batch_device(n, nk, C.ctypes.c_void_p(A.data_ptr()), n * n,
                                                C.ctypes.c_void_p(piv.data_ptr()), None))

    def rsvd():
        C.check(lib.hbem_rsvd_sv_batch_device(n, nk, 0, C.ctypes.c_void_p(T.data_ptr()), n * n, n * n,
                                              C.ctypes.c_void_p(R.data_ptr()), 12, 2, C.dptr(out)))

    out32 = np.zeros(nk)

    def rsvd_mixed():
        C.check(lib.hbem_rsvd_sv_batch_device_ex(n, nk, 0, C.ctypes.c_void_p(T.data_ptr()), n * n, n * n,
                                                 C.ctypes.c_void_p(R.data_ptr()), 12, 2, 1, 3, C.dptr(out32)))

    def rsvd_mixed_fma():
        C.check(lib.hbem_set_option(b"lu_tensor_cores", 0))
        try:
            rsvd_mixed()
        finally:
            C.check(lib.hbem_set_option(b"lu_tensor_cores", 1))

    res = {}
    for name, fn in (("assembly", assemble), ("lu", lu), ("rsvd", rsvd), ("rsvd_mixed", rsvd_mixed),
                     ("rsvd_mixed_fma", rsvd_mixed_fma)):
        fn()
        torch.cuda.synchronize()
        e0, e1 = ev(), ev()
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        res[name] = e0.elapsed_time(e1)
    A.copy_(T)
    torch.cuda.synchronize()
    e0, e1 = ev(), ev()
    e0.record()
    C.check(lib.hbem_lu_factor_batch_device(n, nk, C.ctypes.c_void_p(A.data_ptr()), n * n,
                                            C.ctypes.c_void_p(piv.data_ptr()), None))
    e1.record()
    torch.cuda.synchronize()
    lu_ms = e0.elapsed_time(e1)
    lu_tf = nk * (8.0 / 3.0) * n ** 3 / (lu_ms * 1e-3) / 1e12
    del T, A
    return {"workload": "star polygon 24 vertices (seed 2), N=800 lines (T 1600x1600 c128), order 11, c_i=9, "
                        "%d k in [1,30]; rSVD sketch 12, q=2" % nk,
            "assembly_ms_per_T": res["assembly"] / nk, "rsvd_ms_per_T": res["rsvd"] / nk,
            "lu_ms_per_T": lu_ms / nk, "lu_fp64_tflops": lu_tf,
            "lu_frac_of_measured_fp64": lu_tf / peak if peak else None,
            "T_per_s_assembly_plus_rsvd": 1e3 * nk / (res["assembly"] + res["rsvd"]),
            "rsvd_mixed_ms_per_T": res["rsvd_mixed"] / nk,
            "rsvd_mixed_lu_fp32_fma_ms_per_T": res["rsvd_mixed_fma"] / nk,
            "T_per_s_assembly_plus_rsvd_mixed": 1e3 * nk / (res["assembly"] + res["rsvd_mixed"]),
            "rsvd_mixed_max_rel_err_vs_fp64": float(np.max(np.abs(out32 - out) / out)),
            "sigma_min": [float(x) for x in out[:4]]}


def precision_at_scale(torch, C, api, geometry, lib, ks=(40.0, 41.0)):
    """Precision configuration: seeded Fourier-sum scatterer (seed 4000, 8 modes,
    a_m, b_m ~ N(0, 0.05/m)), N = 4000 line panels (T 8000 x 8000), order 11, c_i = 9,
    c_o = 1, sketch 16, q = 2.  sigma_min by the mixed path (complex-FP32 LU with
    tensor-core trailing updates, FP64 refinement) and by the FP64 path on the same
    sketch, each against sigma_min of T itself from the FP64 Arnoldi path at a
    residual of 1e-12 (a dense FP64 SVD of order 8000 is out of reach of a benchmark
    run; the Arnoldi path agrees with dense SVD and ARPACK in the tests)."""
    import ctypes
    N, n = 4000, 8000
    a, b = geometry.random_fourier_coeffs(4000)
    data = api.BuilderData(geometry.fourier_curve(a, b, N), order=11)
    so = api.SolutionsOperator(data)
    kk = np.array(ks, float)
    nk = kk.size
    T = torch.empty((nk, n, n), dtype=torch.complex128, device="cuda")
    R = torch.from_numpy(np.ascontiguousarray(api.randGaussian(n, 16, seed=4000).T)).cuda()
    ev = lambda: torch.cuda.Event(enable_timing=True)   # noqa: E731
    out = {0: np.zeros(nk), 1: np.zeros(nk)}

    def timed(fn):
        torch.cuda.synchronize()
        e0, e1 = ev(), ev()
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    asm_ms = timed(lambda: C.check(lib.hbem_gen_sol_op_batch_device(so._h, C.dptr(kk), nk, 1.0, 9.0, 0,
                                                                    ctypes.c_void_p(T.data_ptr()))))

    def rsvd(prec):
        C.check(lib.hbem_rsvd_sv_batch_device_ex(n, nk, 0, ctypes.c_void_p(T.data_ptr()), n * n, n * n,
                                                 ctypes.c_void_p(R.data_ptr()), 16, 2, prec, 3, C.dptr(out[prec])))

    rsvd(1)
    mixed_ms = timed(lambda: rsvd(1))
    fp64_ms = timed(lambda: rsvd(0))
    err = np.abs(out[1] - out[0]) / out[0]
    # the complex-FP32 LU alone (tensor-core 128-column blocks, and FP32 FMA with
    # 32-column panels for comparison), on a complex64 copy of the first T
    lu = {}
    T32 = torch.empty((n, n), dtype=torch.complex64, device="cuda")
    piv = torch.zeros(n, dtype=torch.int32, device="cuda")
    for tc in (1, 0):
        C.check(lib.hbem_set_option(b"lu_tensor_cores", tc))
        try:
            T32.copy_(T[0])
            ms = timed(lambda: C.check(lib.hbem_lu_factor_batch_device_f32(n, 1, ctypes.c_void_p(T32.data_ptr()), n * n,
                                                                           ctypes.c_void_p(piv.data_ptr()), None)))
        finally:
            C.check(lib.hbem_set_option(b"lu_tensor_cores", 1))
        lu["tensor_cores" if tc else "fp32_fma"] = {"ms": ms, "tflops": 8.0 / 3.0 * n ** 3 / (ms * 1e-3) / 1e12}
    del T32
    # sigma_min of T itself in FP64: the Arnoldi path (block iteration on T^-1 T^-H
    # with an FP64 LU, ARPACK's residual test at 1e-12; checked against dense SVD and
    # against ARPACK in the tests) -- the dense FP64 reference at this order
    arn = np.zeros(nk)
    st = (ctypes.c_int * nk)()
    it = (ctypes.c_int * nk)()
    arn_ms = timed(lambda: C.check(lib.hbem_arnoldi_sv_batch_device(n, nk, 0, 1, 1e-12, ctypes.c_void_p(T.data_ptr()),
                                                                    n * n, n * n, C.dptr(arn), st, it)))
    del T
    return {"workload": "Fourier-sum scatterer (seed 4000), N=4000 lines (T 8000x8000 c128), order 11, c_i=9, "
                        "k in %s; rSVD sketch 16, q=2" % list(ks),
            "assembly_ms_per_T": asm_ms / nk, "rsvd_mixed_ms_per_T": mixed_ms / nk, "rsvd_fp64_ms_per_T": fp64_ms / nk,
            "sigma_min_mixed": [float(x) for x in out[1]], "sigma_min_fp64": [float(x) for x in out[0]],
            "rel_err_mixed_vs_fp64": [float(x) for x in err],
            "sigma_min_dense_fp64": [float(x) for x in arn],
            "dense_fp64_method": "Arnoldi on T^-1 T^-H, FP64 LU, residual <= 1e-12 sigma (iterations %s)" % list(it),
            "arnoldi_ms_per_T": arn_ms / nk,
            "lu_complex64_n8000": lu,
            "rel_err_vs_dense_fp64": {"mixed": [float(x) for x in np.abs(out[1] - arn) / arn],
                                      "fp64_rsvd": [float(x) for x in np.abs(out[0] - arn) / arn]}}


def batching_scatterers(geometry, api, nk):
    """The 8 seeded scatterers of the batching configuration with their c_i and k."""
    out = []
    for sidx in range(8):
        seed = 3000 + sidx
        rng = np.random.default_rng(seed)
        N = 100 * (sidx + 1)
        if sidx < 4:
            nv = int(rng.integers(8, 41))
            mesh = geometry.polygon(*geometry.star_polygon(nv, seed=seed), N)
        else:
            a, b = geometry.random_fourier_coeffs(seed)
            mesh = geometry.fourier_curve(a, b, N)
        c_i = float(rng.uniform(2.0, 25.0))
        ks = np.sort(rng.uniform(1.0, 30.0, nk))
        out.append((seed, N, mesh, c_i, ks, api.SolutionsOperator(api.BuilderData(mesh, order=11))))
    return out


def batching_sample(torch, C, api, geometry, lib, nk=16, peak=None):
    """Batching configuration on a bounded sample: 8 seeded scatterers (s = 0..3 star
    polygons with 8..40 vertices, s = 4..7 Fourier-sum curves, seed 3000 + s), N =
    100, 200, ..., 800 line panels, c_i ~ U[2, 25], c_o = 1, order 11, nk wavenumbers
    per scatterer uniform on [1, 30] (the configuration's 256 per scatterer, 2048 T(k)
    in all, run under --full-configs); sigma_min by the mixed-precision rSVD (sketch 12,
    q = 2).  Two ways: one batched assembly per scatterer, and every scatterer's
    panel pairs in one assembly launch (hbem_gen_sol_op_multi_device).  Reports T(k)/s
    and the assembly's FP64 rate."""
    import ctypes
    ev = lambda: torch.cuda.Event(enable_timing=True)   # noqa: E731
    scat = batching_scatterers(geometry, api, nk)
    sketches = [torch.from_numpy(np.ascontiguousarray(api.randGaussian(2 * N, 12, seed=seed).T)).cuda()
                for (seed, N, _, _, _, _) in scat]

    def rsvd_all(Ts):
        outs = []
        for (seed, N, _, _, ks, _), T, R in zip(scat, Ts, sketches):
            n = 2 * N
            out = np.zeros(len(ks))
            C.check(lib.hbem_rsvd_sv_batch_device_ex(n, len(ks), 0, ctypes.c_void_p(T.data_ptr()), n * n, n * n,
                                                     ctypes.c_void_p(R.data_ptr()), 12, 2, 1, 3, C.dptr(out)))
            outs.append(out)
        return outs

    # (a) one batched assembly per scatterer
    tot_ms, asm_ms_all, rs_ms_all, per = 0.0, 0.0, 0.0, []
    for (seed, N, _, c_i, ks, so), R in zip(scat, sketches):
        n = 2 * N
        T = torch.empty((nk, n, n), dtype=torch.complex128, device="cuda")
        out = np.zeros(nk)
        torch.cuda.synchronize()
        e0, e1, e2 = ev(), ev(), ev()
        e0.record()
        C.check(lib.hbem_gen_sol_op_batch_device(so._h, C.dptr(ks), nk, 1.0, c_i, 0, ctypes.c_void_p(T.data_ptr())))
        e1.record()
        C.check(lib.hbem_rsvd_sv_batch_device_ex(n, nk, 0, ctypes.c_void_p(T.data_ptr()), n * n, n * n,
                                                 ctypes.c_void_p(R.data_ptr()), 12, 2, 1, 3, C.dptr(out)))
        e2.record()
        torch.cuda.synchronize()
        a_ms, r_ms = e0.elapsed_time(e1), e1.elapsed_time(e2)
        asm_ms_all += a_ms
        rs_ms_all += r_ms
        tot_ms += a_ms + r_ms
        per.append({"N": N, "c_i": round(c_i, 3), "ms_per_T": (a_ms + r_ms) / nk, "sigma_min_min": float(out.min())})
        del T
    tot_T = 8 * nk
    # (b) every scatterer in one assembly launch, then the rSVDs
    ops = [x[5] for x in scat]
    kss = [x[4] for x in scat]
    cis = [x[3] for x in scat]
    Ts = [torch.empty((nk, 1, 2 * N, 2 * N), dtype=torch.complex128, device="cuda") for (_, N, _, _, _, _) in scat]
    api.gen_sol_op_multi_device(ops, kss, 1.0, cis, d=0, out=Ts)   # warm-up
    torch.cuda.synchronize()
    lib.hbem_stats_reset()
    lib.hbem_stats_enable_timing(1)
    e0, e1, e2 = ev(), ev(), ev()
    e0.record()
    api.gen_sol_op_multi_device(ops, kss, 1.0, cis, d=0, out=Ts)
    e1.record()
    outs = rsvd_all(Ts)
    e2.record()
    torch.cuda.synchronize()
    lib.hbem_stats_enable_timing(0)
    launches, a_ms, a_l, a_pts = (C.ctypes.c_longlong(), C.ctypes.c_double(), C.ctypes.c_longlong(),
                                  C.ctypes.c_longlong())
    lib.hbem_stats_read(C.ctypes.byref(launches), C.ctypes.byref(a_ms), C.ctypes.byref(a_l), C.ctypes.byref(a_pts))
    flops = assembly_flops(C, lib)
    m_asm, m_rs = e0.elapsed_time(e1), e1.elapsed_time(e2)
    tf = flops / (a_ms.value * 1e-3) / 1e12 if a_ms.value > 0 else None
    diff = max(abs(float(o.min()) - p["sigma_min_min"]) / p["sigma_min_min"] for o, p in zip(outs, per))
    del Ts
    return {"workload": "8 scatterers (4 star polygons, 4 Fourier curves), N=100..800, order 11, %d k each in "
                        "[1,30]; mixed rSVD sketch 12, q=2" % nk,
            "T_per_s": 1e3 * tot_T / tot_ms, "assembly_share": asm_ms_all / tot_ms, "rsvd_share": rs_ms_all / tot_ms,
            "per_scatterer": per,
            "one_launch": {"T_per_s": 1e3 * tot_T / (m_asm + m_rs), "assembly_ms": m_asm, "rsvd_ms": m_rs,
                           "assembly_launches": int(a_l.value), "assembly_fp64_tflops": tf,
                           "assembly_frac_of_measured_fp64": (tf / peak) if (tf and peak) else None,
                           "assembly_frac_of_nominal_fp64": (tf / nominal_fp64_tflops()) if tf else None,
                           "sigma_min_min_max_rel_diff_vs_per_scatterer": diff}}


def combine_ranks(tot_ms, tot_v, world):
    """Replicas meet on the host only: the slowest rank's time and the verified roots
    of all ranks (a gloo all-reduce when world > 1)."""
    if world <= 1:
        return float(tot_ms), float(tot_v)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(tot_ms)], dtype=torch.float64)
    v = torch.tensor([float(tot_v)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(v)
    return t.item(), v.item()


def arnoldi_at_scale(torch, C, api, geometry, lib):
    """arnoldi::sv / sv_2nd_der on the GPU (block iteration on T^-1 T^-H, ARPACK's
    residual test).  Small: the bench scatterer (circle N=50, T 100x100), 64 k on
    [0.5, 10], count 1, acc 1e-12, with and without derivatives (one CTA per
    matrix).  Large: the dense-tail scatterer (star polygon N=800, T 1600x1600),
    16 k, count 1, acc 1e-10 (batched global-memory LU), beside the randomized
    sigma on the same matrices.  Returns the timings and the matrices the CPU
    ARPACK comparison uses."""
    import ctypes
    ev = lambda: torch.cuda.Event(enable_timing=True)   # noqa: E731

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        e0, e1 = ev(), ev()
        e0.record()
        r = fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), r

    def arn(T, n, nmat, d, count, acc, ms, ds):
        out = np.zeros((nmat, count, d + 1))
        st = (ctypes.c_int * nmat)()
        it = (ctypes.c_int * nmat)()
        C.check(lib.hbem_arnoldi_sv_batch_device(n, nmat, d, count, acc, ctypes.c_void_p(T.data_ptr()), ms, ds,
                                                 C.dptr(out), st, it))
        return out, list(it)

    res = {}
    so = api.SolutionsOperator(api.BuilderData(geometry.circle(CFG["radius"], CFG["N"]), order=CFG["order"]))
    ks = np.linspace(0.5, 10.0, 64)
    n = 2 * CFG["N"]
    T3 = torch.empty((64, 3, n, n), dtype=torch.complex128, device="cuda")
    C.check(lib.hbem_gen_sol_op_batch_device(so._h, C.dptr(ks), 64, CFG["c_o"], CFG["c_i"], 2,
                                             ctypes.c_void_p(T3.data_ptr())))
    ms0, (o0, it0) = timed(lambda: arn(T3, n, 64, 0, 1, 1e-12, 3 * n * n, n * n))
    ms2, (o2, _) = timed(lambda: arn(T3, n, 64, 2, 1, 1e-12, 3 * n * n, n * n))
    res["small"] = {"workload": "circle N=50 (T 100x100), 64 k in [0.5,10], count 1, acc 1e-12",
                    "ms_per_T_sv": ms0 / 64, "ms_per_T_sv_2nd_der": ms2 / 64,
                    "iterations_mean": float(np.mean(it0)), "iterations_max": int(np.max(it0))}
    small_host = [T3[i, 0].cpu().numpy().T.copy() for i in range(4)]
    small_sig = o0[:4, 0, 0].copy()
    del T3
    N = 800
    n = 2 * N
    so = api.SolutionsOperator(api.BuilderData(geometry.polygon(*geometry.star_polygon(24, seed=2), N), order=11))
    ks = np.random.default_rng(3000).uniform(1.0, 30.0, 16)
    T = torch.empty((16, n, n), dtype=torch.complex128, device="cuda")
    C.check(lib.hbem_gen_sol_op_batch_device(so._h, C.dptr(ks), 16, 1.0, 9.0, 0, ctypes.c_void_p(T.data_ptr())))
    msl, (ol, itl) = timed(lambda: arn(T, n, 16, 0, 1, 1e-10, n * n, n * n))
    R = torch.from_numpy(np.ascontiguousarray(api.randGaussian(n, 12, seed=3000).T)).cuda()
    rs = np.zeros(16)
    msr, _ = timed(lambda: C.check(lib.hbem_rsvd_sv_batch_device(n, 16, 0, ctypes.c_void_p(T.data_ptr()), n * n,
                                                                 n * n, ctypes.c_void_p(R.data_ptr()), 12, 2,
                                                                 C.dptr(rs))))
    res["large"] = {"workload": "star polygon 24 vertices (seed 2), N=800 (T 1600x1600), 16 k in [1,30], count 1, "
                                "acc 1e-10",
                    "ms_per_T_sv": msl / 16, "iterations_mean": float(np.mean(itl)), "iterations_max": int(np.max(itl)),
                    "rsvd_ms_per_T (sketch 12, q 2)": msr / 16,
                    "rsvd_rel_excess_over_arnoldi_max": float(np.max((rs - ol[:, 0, 0]) / ol[:, 0, 0]))}
    large_host = [T[0].cpu().numpy().T.copy()]
    large_sig = ol[:1, 0, 0].copy()
    del T, R
    return res, (small_host, small_sig, large_host, large_sig)


FIELD_FLOPS_PER_PAIR = 200.0   # per (grid point, boundary node): Hankel pair ~170, geometry + terms ~30


def field_at_scale(torch, C, api, geometry, lib, peak):
    """tp::direct_second_kind::solve_in_rectangle at a plot-sized workload: star
    polygon (24 vertices, seed 2) with 400 corner-graded panels, c_i = 4, c_o = 1,
    k = 10, plane wave at 60 degrees; traces by the transmission solve, then the total
    field on a 400 x 400 grid over [-1.6, 1.6]^2 with 16 Gauss points per panel.
    Reports the solve and lifting times (host to host, through the C ABI) and the
    grid kernel's CUDA-event time and FP64 rate."""
    import ctypes
    import time
    x, y = geometry.star_polygon(24, seed=2)
    kinds, par = geometry.polygon_graded(x, y, 400, 0.5)
    so = api.SolutionsOperator(api.BuilderData((kinds, par), order=11), proj=False)
    w = api.wave("Plane", 1.0, angle=math.pi / 3)
    k, c_o, c_i, order, n = 10.0, 1.0, 4.0, 16, 400
    api.tp_solve(so, w, k, c_o, c_i)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    tr = api.tp_solve(so, w, k, c_o, c_i)
    t1 = time.perf_counter()
    api.tp_field_grid(so, w, k, c_o, c_i, order, (-1.6, -1.6), (1.6, 1.6), n, n, total_field=True, traces=tr)
    t2 = time.perf_counter()
    S, gx, gy = api.tp_field_grid(so, w, k, c_o, c_i, order, (-1.6, -1.6), (1.6, 1.6), n, n, total_field=True,
                                  traces=tr)
    t3 = time.perf_counter()
    ms, units, near = ctypes.c_double(), ctypes.c_longlong(), ctypes.c_longlong()
    lib.hbem_field_stats(ctypes.byref(ms), ctypes.byref(units), ctypes.byref(near))
    tf = units.value * FIELD_FLOPS_PER_PAIR / (ms.value * 1e-3) / 1e12 if ms.value > 0 else None
    sample = {"kinds": kinds, "par": par, "traces": tr, "wave": w, "k": k, "c_o": c_o, "c_i": c_i, "order": order,
              "pts": np.c_[gx.ravel()[::1597], gy.ravel()[::1597]], "gpu": S.ravel()[::1597]}
    return {"workload": "star polygon 24 vertices (seed 2), 400 graded panels (rf 0.5), c_i=4, c_o=1, k=10, plane "
                        "wave; total field on a 400x400 grid over [-1.6,1.6]^2, 16 Gauss points per panel",
            "tp_solve_ms": 1e3 * (t1 - t0), "field_grid_ms_e2e": 1e3 * (t3 - t2),
            "grid_kernel_ms": ms.value, "point_node_pairs": units.value, "near_pairs": near.value,
            "grid_kernel_fp64_tflops": tf, "grid_kernel_frac_of_measured_fp64": (tf / peak) if (tf and peak) else None,
            "points_per_s_e2e": n * n / (t3 - t2)}, sample


def field_cpu(sample):
    """The same Green sum on the host for a sample of grid points (every 1597th):
    numpy/scipy, the oracle's restatement of the lifting; seconds per point and the
    largest relative difference from the GPU values."""
    import time
    from oracle import oracle as O
    pts = [tuple(p) for p in sample["pts"]]
    t0 = time.perf_counter()
    ref = O.field_points(sample["kinds"], sample["par"], sample["traces"], sample["wave"], sample["k"], sample["c_o"],
                         sample["c_i"], sample["order"], pts, total_field=True)
    dt = time.perf_counter() - t0
    return {"points": len(pts), "ms_per_point": 1e3 * dt / len(pts), "cores": 1, "kind": "port",
            "max_rel_diff_gpu_vs_oracle": float(np.max(np.abs(sample["gpu"] - ref)) / np.max(np.abs(ref)))}


def learned_vs_plain(torch, api, windows=40):
    """The learned proposal (network shipped with the package) against the plain search
    on held-out scatterer windows (seeds 20000..), every root confirmed by Newton on
    sigma'; and the same network on the benchmark circle, windows of width 2 from 0.5."""
    from helmholtzbem_gb300 import learned as L
    net = L.default_network()
    res = L.evaluate(net, list(range(20000, 20000 + windows)))
    # the bench circle (arcs; the network was trained on line panels of the same family)
    so = api.SolutionsOperator(api.BuilderData(geometry_circle(), order=CFG["order"]))
    plain, _, _ = so.find_resonances_plain(CFG["k_min"], CFG["k_max"], CFG["npoints"], CFG["c_o"], CFG["c_i"],
                                           tol=CFG["tol"])
    k0s = np.arange(CFG["k_min"], CFG["k_max"], L.FAMILY["width"])
    cases = [(np.zeros(8), np.zeros(8), CFG["c_i"], float(k)) for k in k0s]
    mins, _ = L.propose(net, cases)
    h = L.FAMILY["width"] / (L.FAMILY["npts"] - 1)
    lo = np.concatenate([L.window(c[3])[m] - 2 * h for c, m in zip(cases, mins)])
    hi = np.concatenate([L.window(c[3])[m] + 2 * h for c, m in zip(cases, mins)])
    keep = (lo < CFG["k_max"]) & (hi > CFG["k_min"])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    roots, ev = so.refine_brackets(lo[keep], hi[keep], CFG["c_o"], CFG["c_i"], tol=CFG["tol"])
    torch.cuda.synchronize()
    t = time.perf_counter() - t0
    hit = int(sum(np.min(np.abs(roots - p)) <= 1e-6 for p in plain)) if roots.size else 0
    res["bench_circle"] = {"plain_roots": int(plain.size), "learned_roots": int(roots.size), "found_plain_roots": hit,
                           "learned_seconds": t, "learned_evals": ev}
    res["workload"] = ("held-out Fourier scatterers (scale 0.25, N=50 lines, c_i ~ U[2,25]), one width-2 window "
                       "each; plain = 210-point grid + Newton per window")
    return res


def geometry_circle():
    from helmholtzbem_gb300 import geometry
    return geometry.circle(CFG["radius"], CFG["N"])


def arnoldi_cpu(mats):
    """The reference's arnoldi::sv call (ARPACK on [0 T^-H; T^-1 0] through one LU)
    made through scipy's ARPACK on the host: ms per matrix and the largest relative
    difference from the GPU result."""
    import time
    from oracle import oracle as O
    small_host, small_sig, large_host, large_sig = mats
    out = {}
    for name, Ts, sig, acc in (("small", small_host, small_sig, 1e-12), ("large", large_host, large_sig, 1e-10)):
        t0 = time.perf_counter()
        ref = np.array([O.arnoldi_sv_arpack(T, 1, acc)[0] for T in Ts])
        dt = time.perf_counter() - t0
        out[name] = {"arpack_ms_per_T": 1e3 * dt / len(Ts), "matrices": len(Ts),
                     "max_rel_diff_gpu_vs_arpack": float(np.max(np.abs(sig - ref) / ref))}
    return out


def adaptive_search(torch, so, plain_roots):
    """The reference's find_resonances search (opt_subdiv sampling with randomized
    sigma on a 2-wide sketch, q = 2, batches of 64; rational-interpolation guess;
    Brent on the dense sigma to relative interval 1e-9) on the bench workload, one run
    after a warm-up, and how many of its minima coincide with the plain search's
    roots (within 1e-6)."""
    import time
    kw = dict(batch_size=64, limit=10, tol=1e-9, seed=1, sketch=2, q=2)
    so.find_resonances_adaptive(CFG["k_min"], CFG["k_max"], CFG["c_o"], CFG["c_i"], **kw)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    roots, ns, ne = so.find_resonances_adaptive(CFG["k_min"], CFG["k_max"], CFG["c_o"], CFG["c_i"], **kw)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    match = sum(1 for r in roots if plain_roots.size and np.min(np.abs(plain_roots - r)) <= 1e-6)
    return {"workload": "adaptive search (opt_subdiv, batch 64, limit 10, sketch 2, q 2; Brent on dense sigma, "
                        "relative interval 1e-9), same scatterer and k range as the bench line",
            "seconds": dt, "minima": int(roots.size), "samples": ns, "T_evals": ne,
            "minima_matching_plain_roots": int(match), "plain_roots": int(plain_roots.size)}


def roots_parity(roots, grid_sigma, oroots, osig, source):
    """The GPU search's roots and grid sigma against the oracle's on the same workload:
    the oracle port run in this process (oroots, osig), else the committed fixture."""
    if oroots is None:
        with open(os.path.join(ROOT, "tests", "golden", "plain_search_circle_N50.json")) as f:
            gold = json.load(f)
        oroots, osig = np.array(gold["roots"]), np.array(gold["grid_sigma"])
    roots, oroots = np.sort(np.asarray(roots)), np.sort(np.asarray(oroots))
    same = roots.size == oroots.size
    dk = float(np.max(np.abs(roots - oroots))) if same and roots.size else None
    ds = float(np.max(np.abs(grid_sigma - osig) / osig)) if grid_sigma is not None else None
    return {"oracle": source, "gpu_roots": int(roots.size), "oracle_roots": int(oroots.size),
            "max_abs_dk": dk, "grid_sigma_max_rel_diff": ds,
            "roots_match_oracle": bool(same and dk is not None and dk <= CFG["tol"])}


def run_gpu(args):
    rank, world, local = dist_env()
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        # independent replicas: the ranks meet only on the host (barrier, max time)
        import torch.distributed as dist
        dist.init_process_group("gloo")
    from helmholtzbem_gb300 import _capi as C, api, geometry

    C.check(C.lib().hbem_set_device(local))
    mesh = geometry.circle(CFG["radius"], CFG["N"])
    data = api.BuilderData(mesh, order=CFG["order"])
    so = api.SolutionsOperator(data)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")   # > L2 (129 MB)
    last_grid = [None]

    def step(solop):
        # the search with every root checked: sigma' at root - tol and root + tol, each
        # root's two points evaluated as soon as it has converged
        roots, grid, nev, chk = solop.find_resonances_plain_verified(CFG["k_min"], CFG["k_max"], CFG["npoints"],
                                                                     CFG["c_o"], CFG["c_i"], tol=CFG["tol"])
        last_grid[0] = grid[:, 0].copy()
        ver = int(np.sum((chk[:, 0] <= 0.0) & (chk[:, 1] >= 0.0)))
        return ver, roots, nev

    for _ in range(max(3, args.warmup)):
        step(so)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()

    lib = C.lib()
    lib.hbem_stats_reset()
    tot_ms, tot_v, nev_tot = 0.0, 0, 0
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            v, roots, nev = step(so)
            e1.record()
            torch.cuda.synchronize()
            tot_ms += e0.elapsed_time(e1)
            tot_v += v
            nev_tot += nev
    launches, asm_ms, asm_l, asm_pts = (C.ctypes.c_longlong(), C.ctypes.c_double(), C.ctypes.c_longlong(),
                                        C.ctypes.c_longlong())
    lib.hbem_stats_read(C.ctypes.byref(launches), None, None, None)
    ms, tot_v_all = combine_ranks(tot_ms, tot_v, world)
    value = tot_v_all / (ms * 1e-3)

    # end to end from host data through the C ABI: mesh upload, operator set-up,
    # search and root read-back inside the timed region
    kinds, par = mesh
    h2d = kinds.nbytes + par.nbytes
    e2e_ms, e2e_v = 0.0, 0
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        d2 = api.BuilderData((kinds.copy(), par.copy()), order=CFG["order"])
        s2 = api.SolutionsOperator(d2)
        v, roots, _ = step(s2)
        e1.record()
        torch.cuda.synchronize()
        e2e_ms += e0.elapsed_time(e1)
        e2e_v += v
        del s2, d2
    d2h = int(roots.nbytes + CFG["npoints"] * 3 * 8 + 2 * roots.size * 8)   # roots, grid, the roots' checks

    # roofline of the dominant kernel (panel-pair assembly, FP64 CUDA-core bound):
    # algorithmic work of the timed launches by derivative order and point kind, on one
    # search of the workload with the Newton candidates in lock step, so that the timed
    # assembly launches do not overlap (on per-candidate streams a launch's event
    # interval would also cover other candidates' kernels)
    C.check(lib.hbem_set_option(b"plain_async", 0))
    try:
        lib.hbem_stats_reset()
        lib.hbem_stats_enable_timing(1)
        step(so)
        torch.cuda.synchronize()
        lib.hbem_stats_enable_timing(0)
        lib.hbem_stats_read(None, C.ctypes.byref(asm_ms), C.ctypes.byref(asm_l), C.ctypes.byref(asm_pts))
    finally:
        C.check(lib.hbem_set_option(b"plain_async", 1))
    flops = assembly_flops(C, lib)
    achieved = flops / (asm_ms.value * 1e-3) / 1e12 if asm_ms.value > 0 else 0.0
    peak = fp64_peak_tflops()
    roofline = {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak if peak else None,
                # DRAM bytes (read + write) per assembly launch, averaged over the 24
                # k_singular / k_general(_w) launches of one plain search of this workload
                # (ncu dram__bytes_read.sum + dram__bytes_write.sum, caches flushed
                # between launches): the singular launches read the 68 MB point table,
                # the grid's general launch writes 63 MB of pair blocks
                "traffic": 3.0e7, "traffic_unit": "bytes per launch",
                "peak_source": "measured: cuBLAS DGEMM 8192^3 on this GPU (MEASURED_PEAKS.json has no FP64 entry)",
                "kernel": "k_general + k_singular (panel-pair assembly)", "launches": asm_l.value,
                "measured_on": "one search of the workload, Newton candidates in lock step (non-overlapping launches)",
                "avg_launch_ms": asm_ms.value / max(1, asm_l.value),
                # nominal FP64 peak: 2 DFMA per cycle per SM x 152 SMs at the sampled SM clock
                "peak_nominal": nominal_fp64_tflops(), "frac_of_nominal": achieved / nominal_fp64_tflops(),
                # FP64 instructions the kernels execute (ncu: DFMA x 2 + DMUL + DADD per cycle
                # x SM clock), from profiles/assembly_kernels_circle_N50_p11_d2.md; the
                # algorithmic count above uses the reference's per-point work, which this
                # build's Hankel pair undercuts, so the algorithmic rate reads above these
                "ncu_executed_fp64_tflops": {"k_general<0> grid": 0.79, "k_singular<0> grid": 0.66,
                                             "k_singular<2> Newton": 0.77}}

    scale = assembly_at_scale(torch, C, api, geometry, lib, peak)
    tail = dense_tail_at_scale(torch, C, api, geometry, lib, peak)
    prec = precision_at_scale(torch, C, api, geometry, lib)
    batch = batching_sample(torch, C, api, geometry, lib, peak=peak)
    adapt = adaptive_search(torch, so, step(so)[1])
    arnoldi, arn_mats = arnoldi_at_scale(torch, C, api, geometry, lib)
    field, field_sample = field_at_scale(torch, C, api, geometry, lib, peak)
    learned = learned_vs_plain(torch, api)

    cpu = None
    parity = roots_parity(roots, last_grid[0], None, None, "committed fixture tests/golden/plain_search_circle_N50.json")
    if rank == 0 and not args.skip_cpu:
        try:
            pool = sweep_pool()
            try:
                v, tsec, oroots, osig, _ = cpu_search(pool)
            finally:
                pool.close()
            cpu = {"value": v / tsec if tsec > 0 else None, "unit": "resonances/s", "cores": pool.workers,
                   "kind": "port", "sample": CPU_SAMPLE + " (one step)"}
            parity = roots_parity(roots, last_grid[0], oroots, osig, "oracle port, same run")
        except Exception as ex:   # the baseline must not hide the GPU line
            cpu = {"value": None, "unit": "resonances/s", "cores": os.cpu_count(), "kind": "port",
                   "error": str(ex)[:200]}
        try:
            arnoldi["cpu_arpack"] = arnoldi_cpu(arn_mats)
        except Exception as ex:
            arnoldi["cpu_arpack"] = {"error": str(ex)[:200]}
        try:
            field["cpu_port"] = field_cpu(field_sample)
        except Exception as ex:
            field["cpu_port"] = {"error": str(ex)[:200]}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "resonances/s", "n_gpus": world, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": CONFIG,
            "workload_stats": {"roots_per_step": tot_v / args.steps, "T_evals_per_step": nev_tot / args.steps},
            "parity": parity,
            "e2e": {"value": e2e_v / (e2e_ms * 1e-3), "unit": "resonances/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": int(launches.value),
            "roofline": roofline,
            "assembly_at_scale": scale,
            "dense_tail_at_scale": tail,
            "precision_at_scale": prec,
            "batching_sample": batch,
            "adaptive_search": adapt,
            "arnoldi_at_scale": arnoldi,
            "field_at_scale": field,
            "learned_vs_plain": learned,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def run_full_configs():
    """The batching configuration with all 256 wavenumbers per scatterer (2048 T(k))
    and the precision configuration at k = 40, ..., 47, each once (a few tens of
    seconds of GPU time, so not part of the default run)."""
    import torch
    from helmholtzbem_gb300 import _capi as C, api, geometry
    lib = C.lib()
    torch.cuda.set_device(0)
    batch = batching_sample(torch, C, api, geometry, lib, nk=256, peak=fp64_peak_tflops())
    prec = precision_at_scale(torch, C, api, geometry, lib, ks=tuple(float(k) for k in range(40, 48)))
    print(json.dumps({"batching_full": batch, "precision_full": prec}))


def main():
    args = parse()
    if args.full_configs:
        run_full_configs()
    elif args.profile_search:
        run_profile_search()
    elif args.profile_dense_tail:
        run_profile_dense_tail()
    elif args.profile_case:
        run_profile_case()
    elif args.profile_field:
        run_profile_field()
    elif args.profile_lu:
        run_profile_lu()
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
