"""Benchmark: time-to-solution of the DDA solve on the 128^3 sphere (N = 1,099,136, grid 256^3) on one GB300.

One step = one complete solve of both incident polarisations (2 right-hand sides) of the 128^3 sphere (1,099,136
dipoles, FFT grid 256^3, m = 1.33+0.01i, 15 dipoles per wavelength) with QMR_CS to relative residual 1e-5 in the
mixed-precision mode (FP32 Krylov + FFT matvec, FP64 residual refinement), inputs resident in HBM. The line also
reports the plain-FP64 GPU time-to-solution on the same workload, the FP32 matvec's HBM roofline, the end-to-end
time through the host-pointer C ABI, and a CPU baseline (the oracle port on this machine's host cores).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--method qmr|bicgstab]

--impl reference times the reference's CPU algorithm (the oracle restatement; the reference binary itself is built
only where its sources are) on the host cores, on the same metric.
Multi-GPU: the path does not shard one solve; N GPUs run N independent replicas (weak scaling).
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "a-dda_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "time-to-solution @res 1e-5, 128^3 sphere (both polarisations), mixed FP32/FP64 on GB300"
# MIXED here = FP32 matvec (FFTs, D, expanded grid) with double-float Krylov vectors (float pairs, ~48 bits, FP32
# pipes), FP64 recurrence scalars and FP64 residual refinement; the variants with FP64 ("mixed_f64vec") and FP32
# ("mixed_f32vec") Krylov vectors are reported beside it
GRID, M_REF, DPL, EPS = 128, 1.33 + 0.01j, 15.0, 1e-5
WORKLOAD = ("sphere 128^3 box, N=1099136 dipoles, FFT grid 256^3, m=1.33+0.01i, dpl=15, LDR, %s to 1e-5, "
            "2 RHS (both polarisations)")
# iteration counts of the reference build (ADDA 1.3b6 seq + FFTW-subset shim) on this workload, per polarisation
# (Y, X), from a full run of '-grid 128 -dpl 15 -m 1.33 0.01 -iter <m> -eps 5 -sym no'; used only to extrapolate
# the bounded CPU samples to a time-to-solution
# (tests/golden/reference_c2.json: 623 + 648 QMR_CS iterations in 6956 s, 311 + 314 BiCGStab iterations in 6726 s
# of one x86 core)
REF_ITERS = {"qmr": (623, 648), "bicgstab": (311, 314)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p.get("hbm_gbs", 6800.0), "measured"
    except Exception:
        return 6800.0, "fallback"


def matvec_bytes(n, g, b, s, R):
    """algorithmic HBM bytes of one matvec for R RHS sharing D: per RHS s*9N (x read twice, y written) +
    s*12*gX*bY*bZ (the x-transformed intermediate written/read twice) + 14N (lattice indices), plus D once"""
    gX, gY, gZ = g
    bX, bY, bZ = b
    return R * (s * 9 * n + s * 12 * gX * bY * bZ + 14 * n) + s * 6 * gX * (gY // 2 + 1) * (gZ // 2 + 1)


class Clocks:
    """samples nvidia-smi during the timed region"""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def dist_init(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "ours" else "gloo"
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(world, v):
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def bench_config(method, world):
    """the workload description shared by both arms (the driver compares the two lines' config)"""
    return {"workload": WORKLOAD % ("QMR_CS" if method == "qmr" else "BiCGStab"), "method": method, "rhs": 2,
            "parallelism": "replicas" if world > 1 else "single",
            "l2": "inputs larger than L2 (D 204 MB FP32, Einc 106 MB)"}


class CpuArm:
    """The reference's algorithm on the host cores: the oracle (the reference's InitDmatrix / MatVec / QMR_CS /
    BiCGStab restated in C with OpenMP over lines and slices, FP64) on the same 128^3 sphere, with its inputs built by
    the oracle's own numpy restatement of the reference host (oracle/setup.py), so the GPU library is never loaded.
    One sample = `iters` iterations of the oracle's own solver on the Y polarisation from x_0 = 0 (no convergence
    test can stop it: eps = 1e-300); the time-to-solution is the time per iteration x the reference's iteration count
    on this workload, both polarisations solved one after the other as the reference does."""

    def __init__(self, method, nthreads, iters=None):
        from oracle import oracle as O
        from oracle.setup import SphereWorkload
        self.O = O
        self.method = method
        self.iters = iters or (2 if method == "bicgstab" else 4)
        self.nthreads = nthreads
        w = SphereWorkload(GRID, M_REF, DPL, O.lib().or_fftfit)
        t0 = time.perf_counter()
        self.o = O.Oracle(w.box, w.grid, w.pos, w.mat, w.gridspace, w.wavenum, nthreads)
        self.t_dmatrix = time.perf_counter() - t0
        self.o.set_cc(w.cc[0].reshape(1, 3))
        self.einc = w.einc[0]
        self.n = w.n

    def sample(self):
        """seconds per iteration of one right-hand side"""
        m = self.O.QMR_CS if self.method == "qmr" else self.O.BICGSTAB
        t0 = time.perf_counter()
        r = self.o.solve(self.einc, method=m, eps=1e-300, maxiter=self.iters, init_field=self.O.IF_ZERO, hist_cap=64)
        t = time.perf_counter() - t0
        if r["niter"] != self.iters:
            raise RuntimeError("oracle sample ran %d iterations, expected %d" % (r["niter"], self.iters))
        return t / self.iters

    def describe(self):
        return ("%d %s iterations of the oracle's FP64 solver (128^3 sphere, N=%d, Y polarisation, x_0 = 0) per "
                "sample; the matvec's FFT passes on %d threads, scatter/gather and BLAS-1 sequential as in the "
                "reference's seq build; time-to-solution = seconds per iteration x the reference's iteration count "
                "%s (both polarisations)" % (self.iters, "QMR_CS" if self.method == "qmr" else "BiCGStab", self.n,
                                             self.nthreads, list(REF_ITERS[self.method])))

    def close(self):
        self.o.close()


def run_reference(args):
    world, rank, local = dist_init(args)
    if rank != 0:
        return
    nthreads = os.cpu_count() or 1
    arm = CpuArm(args.method, nthreads)
    for _ in range(args.warmup):
        arm.sample()
    per_it = [arm.sample() for _ in range(args.steps)]
    arm.close()
    t_it = statistics.mean(per_it)
    value = t_it * sum(REF_ITERS[args.method])
    line = {"metric": METRIC, "value": value, "unit": "s", "impl": "reference", "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": value * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (generated particle, plane wave)",
            "config": bench_config(args.method, world),
            "seconds_per_iteration": t_it, "iterations_of_the_reference": list(REF_ITERS[args.method]),
            "cpu_baseline": {"value": value, "unit": "s", "cores": nthreads, "kind": "port",
                             "sample": arm.describe()},
            "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def accuracy(method, ce, ca):
    """relative errors of the mixed solve's cross sections (Y, X polarisation) against the reference's own runs of
    this workload: its solve with the same method to eps 1e-5 and its solves to residual 1e-8 (converged; the
    spec bar is 1e-6 against the converged FP64 cross sections)"""
    out = {}
    gd = os.path.join(ROOT, "tests", "golden")
    try:
        with open(os.path.join(gd, "reference_c2.json")) as f:
            run = json.load(f)["runs"][method]["cross"]
        out["reference_eps1e-5_same_method"] = {
            "Cext": [abs(ce[r] / run[p]["Cext"] - 1) for r, p in enumerate("YX")],
            "Cabs": [abs(ca[r] / run[p]["Cabs"] - 1) for r, p in enumerate("YX")]}
    except (OSError, KeyError):
        pass
    try:
        with open(os.path.join(gd, "reference_c2_converged.json")) as f:
            conv = json.load(f)["converged"]
        out["reference_converged"] = {"Cext": [abs(v / conv["Cext"] - 1) for v in ce],
                                      "Cabs": [abs(v / conv["Cabs"] - 1) for v in ca]}
    except (OSError, KeyError):
        pass
    return out


def run_ours(args):
    world, rank, local = dist_init(args)
    import torch
    torch.cuda.set_device(local)
    import adda_gb300 as A
    s = A.Setup(grid=GRID, m=M_REF, dpl=DPL)
    R = 2
    ctx = A.Context.from_setup(s, nrhs_max=R, device=local)
    einc = np.ascontiguousarray(np.stack(s.einc))
    d_e = torch.from_numpy(einc.view(np.float64)).cuda()
    d_x = torch.empty_like(d_e)
    d_p = torch.empty_like(d_e)
    opts = dict(method=args.method, eps=EPS)
    for _ in range(args.warmup):
        ctx.solve_device(d_e.data_ptr(), R, d_x.data_ptr(), d_p.data_ptr(), prec="mixed", **opts)
    torch.cuda.synchronize()
    barrier(world)
    l0 = A.kernel_launches()
    ms = []
    stats = None
    with Clocks(local) as clk:
        torch.cuda.synchronize()
        for _ in range(args.steps):
            stats = ctx.solve_device(d_e.data_ptr(), R, d_x.data_ptr(), d_p.data_ptr(), prec="mixed", **opts)
            ms.append(ctx.last_solve_ms())
        torch.cuda.synchronize()
    launches = A.kernel_launches() - l0
    barrier(world)
    t_solve = allmax(world, statistics.mean(ms) / 1e3)
    ce, ca = ctx.cross_sections(np.stack([s.prop, s.prop]), np.stack(s.incpol))
    # end to end through the host-pointer C ABI: Einc from pinned host memory, x and p back to host (right after the
    # timed device solves, in the same state of the GPU)
    pin_e = torch.from_numpy(einc.view(np.float64)).pin_memory()
    pin_x = torch.empty_like(pin_e).pin_memory()
    pin_p = torch.empty_like(pin_e).pin_memory()
    # the C-ABI calls a host makes (adda_gb300_solve with host Einc/x/p, then adda_gb300_cross_sections)
    import ctypes
    sp = A.SolveParams(A.ITERS[args.method], A.PREC["mixed"], EPS, 100000, A.INIT["auto"], 0, 0.0, 0, 0.0, 0)
    rst = (A.RhsStats * R)()
    props, incs = np.ascontiguousarray(np.stack([s.prop, s.prop])), np.ascontiguousarray(np.stack(s.incpol))
    h_ce, h_ca = np.zeros(R), np.zeros(R)

    def host_step():
        if ctx.L.adda_gb300_solve(ctx.h, ctypes.byref(sp), R, pin_e.data_ptr(), pin_x.data_ptr(), pin_p.data_ptr(),
                                  rst, None, 0) or \
                ctx.L.adda_gb300_cross_sections(ctx.h, R, props.ctypes.data, incs.ctypes.data, h_ce.ctypes.data,
                                                h_ca.ctypes.data):
            raise RuntimeError(A.lib().adda_gb300_last_error().decode())
        for r in range(R):
            if rst[r].status != 0 or not rst[r].resid <= EPS:
                raise RuntimeError("end-to-end solve did not converge: RHS %d status %d residual %g"
                                   % (r, rst[r].status, rst[r].resid))
    for _ in range(args.warmup):
        host_step()
    torch.cuda.synchronize()
    e2e, e2e_dev = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        host_step()  # x and p go straight into the pinned host buffers (the C ABI's xvec/pvec)
        e2e.append(time.perf_counter() - t0)
        e2e_dev.append(ctx.last_solve_ms() / 1e3)
    t_e2e = allmax(world, statistics.mean(e2e))
    # the variants with FP32 and with FP64 Krylov vectors, once each, for comparison
    st32 = ctx.solve_device(d_e.data_ptr(), R, d_x.data_ptr(), d_p.data_ptr(), prec="mixed_f32vec", **opts)
    t_f32vec = ctx.last_solve_ms() / 1e3
    st64v = ctx.solve_device(d_e.data_ptr(), R, d_x.data_ptr(), d_p.data_ptr(), prec="mixed_f64vec", **opts)
    t_f64vec = ctx.last_solve_ms() / 1e3
    # plain FP64 GPU solve on the same workload (one warm-up, one timed)
    ctx.solve_device(d_e.data_ptr(), R, d_x.data_ptr(), d_p.data_ptr(), prec="fp64", **opts)
    st64 = ctx.solve_device(d_e.data_ptr(), R, d_x.data_ptr(), d_p.data_ptr(), prec="fp64", **opts)
    t64 = allmax(world, ctx.last_solve_ms() / 1e3)
    ce64, ca64 = ctx.cross_sections(np.stack([s.prop, s.prop]), np.stack(s.incpol))
    # the configuration's other method (BiCGStab or QMR_CS), mixed, one warm-up and one timed solve
    other = "bicgstab" if args.method == "qmr" else "qmr"
    for _ in range(2):
        sto = ctx.solve_device(d_e.data_ptr(), R, d_x.data_ptr(), d_p.data_ptr(), prec="mixed", method=other,
                               eps=EPS)
    t_other = allmax(world, ctx.last_solve_ms() / 1e3)
    # FP32 matvec roofline (R=2 RHS sharing D), and the FP64 matvec time
    mv32 = ctx.time_matvec("fp32", R, iters=20)
    shape32 = list(ctx.fft_shape("fp32")) + ["chunk %d x-slabs" % ctx.l2_chunk("fp32")]
    mv64 = ctx.time_matvec("fp64", R, iters=3)
    bts = matvec_bytes(s.n, s.grid, s.box, 8, R)
    hbm, src = peaks()
    achieved = bts / (mv32 * 1e-3) / 1e9
    # DRAM bytes of one pipelined FP32 matvec from the committed ncu capture (not measured in this run; the file
    # names the capture and its date)
    traffic, traffic_src = None, None
    tf = os.path.join(ROOT, "profiles", "matvec_fp32_dram_bytes.json")
    if os.path.exists(tf):
        with open(tf) as f:
            tj = json.load(f)
        traffic, traffic_src = tj.get("bytes_per_matvec"), tj.get("source")
    line = {
        "metric": METRIC, "value": t_solve, "unit": "s", "n_gpus": world, "steps": args.steps,
        "rel_err_vs_reference": accuracy(args.method, ce, ca),
        "warmup": args.warmup, "ms_per_step": t_solve * 1e3, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "c64 matvec + double-float Krylov vectors + f64 scalars/refinement (mixed)", "data": "synthetic (generated particle, plane wave)",
        "config": bench_config(args.method, world),
        "timing": "CUDA events on the library stream around each solve; e2e: host wall clock around the C-ABI calls",
        "fp64_time_to_solution_s": t64,
        "mixed_f32vec_time_to_solution_s": t_f32vec,
        "mixed_f32vec_iterations": [x["niter"] for x in st32],
        "mixed_f64vec_time_to_solution_s": t_f64vec,
        "mixed_f64vec_iterations": [x["niter"] for x in st64v],
        "speedup_mixed_vs_fp64": t64 / t_solve,
        "other_method": {"method": other, "mixed_time_to_solution_s": t_other,
                         "iterations": [x["niter"] for x in sto]},
        "iterations": {"mixed": [x["niter"] for x in stats], "fp64": [x["niter"] for x in st64],
                       "fp64_matvecs_in_mixed": [x["matvecs_fp64"] for x in stats],
                       "refinements": [x["refinements"] for x in stats]},
        "residual": {"mixed": [x["resid"] for x in stats], "fp64": [x["resid"] for x in st64]},
        "Cext": {"mixed": list(map(float, ce)), "fp64": list(map(float, ce64))},
        "Cabs": {"mixed": list(map(float, ca)), "fp64": list(map(float, ca64))},
        "matvec": {"fp32_ms": mv32, "fp64_ms": mv64, "fp32_GBps": achieved, "rhs": R,
                   "algorithmic_bytes": bts, "fp32_tile_shape (w1, w2, pairs, threads; tuned)": shape32},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": traffic, "traffic_source": traffic_src,
                     "kernel": "FP32 matvec (K1..K3 sequence, 2 RHS)",
                     "peak_source": src},
        "e2e": {"value": t_e2e, "unit": "s", "h2d_bytes_per_step": einc.nbytes,
                "d2h_bytes_per_step": 2 * einc.nbytes + 16 * R,
                "device_solve_s_mean": statistics.mean(e2e_dev),
                "iterations_last_step": [rst[r].niter for r in range(R)]},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if not args.no_surface:
        ctx.close()
        try:
            line["surface"] = run_surface(args)
        except Exception as ex:  # reported, never fatal for the headline line
            line["surface"] = {"error": str(ex)}
    if not args.no_scale:
        try:
            line["scale_256sphere"] = run_scale(args)
        except Exception as ex:  # reported, never fatal for the headline line
            line["scale_256sphere"] = {"error": str(ex)}
    if args.batch_particles:
        try:
            line["batch_ellipsoids"] = run_batch(args)
        except Exception as ex:
            line["batch_ellipsoids"] = {"error": str(ex)}
        if args.group_particles > 0:
            try:
                line["batch_grouped"] = run_group(args)
            except Exception as ex:
                line["batch_grouped"] = {"error": str(ex)}
    if rank == 0 and world == 1 and not args.no_cpu:
        arm = CpuArm(args.method, os.cpu_count() or 1)
        arm.sample()
        t_it = statistics.mean(arm.sample() for _ in range(3))
        arm.close()
        v = t_it * sum(REF_ITERS[args.method])
        line["cpu_baseline"] = {"value": v, "unit": "s", "cores": arm.nthreads, "kind": "port",
                                "sample": arm.describe()}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def run_surface(args):
    """the bench sphere (128^3 box, grid 256^3, m = 1.33+0.01i, dpl 15) with its centre 30 um above a glass-like
    substrate (msub = 1.5, -surf 30 1.5 0 -int_surf img, light from above along -z): the reflected interaction R in
    the same FFT matvec (a second z transform per chunk and the D+R product). Mixed QMR_CS to 1e-5 on both
    polarisations, plus the FP32/FP64 matvec times against the free-space ones."""
    import torch
    import adda_gb300 as A
    s = A.Setup(grid=GRID, m=M_REF, dpl=DPL, prop=[0, 0, -1], surface=dict(h=30.0, msub=1.5, relation="img"))
    t0 = time.perf_counter()
    ctx = A.Context.from_setup(s, nrhs_max=2)
    torch.cuda.synchronize()
    t_init = time.perf_counter() - t0
    einc = np.ascontiguousarray(np.stack(s.einc))
    d_e = torch.from_numpy(einc.view(np.float64)).cuda()
    ctx.solve_device(d_e.data_ptr(), 2, None, None, method=args.method, prec="mixed", eps=EPS)
    st = ctx.solve_device(d_e.data_ptr(), 2, None, None, method=args.method, prec="mixed", eps=EPS)
    t_solve = ctx.last_solve_ms() / 1e3
    ce, ca = ctx.cross_sections_beam(einc, s.inc_scale)
    mv32 = ctx.time_matvec("fp32", 2, iters=10)
    mv64 = ctx.time_matvec("fp64", 2, iters=3)
    out = {"workload": "sphere 128^3 box, N=%d, grid 256^3, m=1.33+0.01i, dpl=15, centre 30 um above msub=1.5 "
           "(image relation), incidence -z, mixed %s to 1e-5, 2 RHS" % (s.n, args.method),
           "solve_s": t_solve, "iterations": [x["niter"] for x in st], "status": [x["status"] for x in st],
           "init_s (D + R matrices + setup)": t_init, "Cext": list(map(float, ce)), "Cabs": list(map(float, ca)),
           "fp32_matvec_ms": mv32, "fp64_matvec_ms": mv64}
    ctx.close()
    return out


def run_scale(args):
    """the scale workload: sphere on a 256^3 box (N = 8,783,848), FFT grid 512^3, m = 1.2, dpl 10, mixed solve to
    1e-5 (BiCGStab by default), both polarisations as 2 RHS, device-resident, capped at --scale-maxiter iterations:
    the Krylov methods converge slowly on this non-absorbing x = 80 sphere (BiCGStab: relative residual 1.5e-3 after
    3000 iterations, 1.8e-4 after 9000), so the line reports the time per iteration, the residual reached and the
    FP32 matvec at 512^3 rather than a time-to-solution"""
    import torch
    import adda_gb300 as A
    s = A.Setup(grid=256, m=1.2, dpl=10)
    t0 = time.perf_counter()
    ctx = A.Context.from_setup(s, nrhs_max=2)
    torch.cuda.synchronize()
    t_init = time.perf_counter() - t0
    einc = np.ascontiguousarray(np.stack(s.einc))
    d_e = torch.from_numpy(einc.view(np.float64)).cuda()
    log("scale workload: context + D matrix %.2f s, solving (maxiter %d)" % (t_init, args.scale_maxiter))
    st = ctx.solve_device(d_e.data_ptr(), 2, None, None, method=args.scale_method, prec="mixed", eps=EPS,
                          maxiter=args.scale_maxiter)
    t_solve = ctx.last_solve_ms() / 1e3
    ce, ca = ctx.cross_sections(np.stack([s.prop, s.prop]), np.stack(s.incpol))
    mv32 = ctx.time_matvec("fp32", 2, iters=5)
    bts = matvec_bytes(s.n, s.grid, s.box, 8, 2)
    hbm, _ = peaks()
    out = {"workload": "sphere 256^3 box, N=%d, FFT grid %s, m=1.2, dpl=10, mixed %s to 1e-5, 2 RHS"
           % (s.n, "x".join(map(str, s.grid)), args.scale_method),
           "solve_s": t_solve, "init_s (D matrix + setup)": t_init, "maxiter": args.scale_maxiter,
           "converged": all(x["status"] == "ok" for x in st), "status": [x["status"] for x in st],
           "ms_per_iteration": 1e3 * t_solve / max(1, max(x["niter"] for x in st)),
           "iterations": [x["niter"] for x in st], "residual": [x["resid"] for x in st],
           "Cext": list(map(float, ce)), "Cabs": list(map(float, ca)),
           "fp32_matvec_ms": mv32, "fp32_matvec_GBps": bts / (mv32 * 1e-3) / 1e9,
           "fp32_matvec_roofline_frac": bts / (mv32 * 1e-3) / 1e9 / hbm, "fp32_tile_shape": list(ctx.fft_shape())}
    ctx.close()
    return out


def run_batch(args):
    """the batching workload: seeded ellipsoids (numpy default_rng(20261203): box from {24,32,48,64,96}, aspect
    ratios U[0.5,1], m_re U[1.2,1.7], m_im U[0,0.05], dpl 10|m|), each with 16 orientations (zyz: alpha, gamma
    U[0,360), beta = arccos U[-1,1]) x 2 polarisations = 32 RHS solved together (mixed QMR_CS to 1e-5). Timed per
    particle with CUDA events (solve) and wall clock (lattice + D matrix + solve)."""
    import torch
    import adda_gb300 as A
    rng = np.random.default_rng(20261203)
    nrhs = 32
    solve_s, total_s, iters, boxes, nrhs_done, unconverged = 0.0, 0.0, [], [], 0, 0
    for _ in range(args.batch_particles):
        box = int(rng.choice([24, 32, 48, 64, 96]))
        r1, r2 = (float(v) for v in rng.uniform(0.5, 1.0, 2))
        m = complex(rng.uniform(1.2, 1.7), rng.uniform(0.0, 0.05))
        orients = [(rng.uniform(0, 360), math.degrees(math.acos(rng.uniform(-1, 1))), rng.uniform(0, 360))
                   for _ in range(nrhs // 2)]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s = A.Setup(grid=box, shape="ellipsoid", pars=(r1, r2), m=m)
        ctx = A.Context(s.box, s.pos, s.mat, s.gridspace, s.wavenum, s.grid, nrhs_max=nrhs)
        ctx.init_dmatrix()
        einc = []
        for k, o in enumerate(orients):
            prop, py, px = A.rotation(*o)
            for j, e in enumerate((py, px)):
                ctx.set_cc(2 * k + j, A.polarizability(s.m, s.kd, s.gridspace, prop, e).reshape(1, 3))
                einc.append(A.plane_wave(s.box, s.pos, s.gridspace, s.wavenum, prop, e))
        d_e = torch.from_numpy(np.ascontiguousarray(np.stack(einc)).view(np.float64)).cuda()
        st = ctx.solve_device(d_e.data_ptr(), nrhs, None, None, method=args.batch_method, prec="mixed", eps=EPS,
                              maxiter=args.batch_maxiter)
        torch.cuda.synchronize()
        total_s += time.perf_counter() - t0
        log("batch particle: box %s grid %s N %d: %.2f s, iterations <= %d, %d/%d converged"
            % (s.box, s.grid, s.n, ctx.last_solve_ms() / 1e3, max(x["niter"] for x in st),
               sum(x["status"] == "ok" for x in st), nrhs))
        unconverged += sum(x["status"] != "ok" for x in st)
        solve_s += ctx.last_solve_ms() / 1e3
        iters.append(max(x["niter"] for x in st))
        boxes.append(box)
        nrhs_done += nrhs
        ctx.close()
    return {"workload": "the first %d of the 64 seeded ellipsoids x 16 orientations x 2 polarisations (%d RHS), "
                        "mixed %s to 1e-5" % (args.batch_particles, nrhs_done, args.batch_method),
            "solve_s": solve_s, "total_s (lattice + D matrix + solve)": total_s,
            "rhs_per_s_solve": nrhs_done / solve_s, "rhs_per_s_total": nrhs_done / total_s,
            "maxiter": args.batch_maxiter, "rhs_not_converged": unconverged,
            "boxes": boxes, "max_iterations_per_particle": iters}


def run_group(args):
    """grouped batching: the first --group-particles of the seeded ellipsoids (run_batch's sequence) whose box is 24 or 32,
    at one lattice spacing (dpl 17 = 10 x the largest |m|, so that all share D), 16 orientations x 2 polarisations
    each, solved (mixed, --batch-method, to 1e-5) once one context per particle, once as one group context (all
    particles' RHS in every launch; the common box is the largest particle's cube, so the FFT grid is a power of two).
    CUDA-event solve times."""
    import torch
    import adda_gb300 as A
    rng = np.random.default_rng(20261203)
    nrhs, dpl = 32, 17.0
    parts = []
    while len(parts) < args.group_particles:
        box = int(rng.choice([24, 32, 48, 64, 96]))
        r1, r2 = (float(v) for v in rng.uniform(0.5, 1.0, 2))
        m = complex(rng.uniform(1.2, 1.7), rng.uniform(0.0, 0.05))
        orients = [(rng.uniform(0, 360), math.degrees(math.acos(rng.uniform(-1, 1))), rng.uniform(0, 360))
                   for _ in range(nrhs // 2)]
        if box <= 32:
            parts.append((A.Setup(grid=box, shape="ellipsoid", pars=(r1, r2), m=m, dpl=dpl), orients))

    def rhs(s, orients, box):
        cc, e = [], []
        for o in orients:
            prop, py, px = A.rotation(*o)
            for pol in (py, px):
                cc.append(A.polarizability(s.m, s.kd, s.gridspace, prop, pol).reshape(1, 3))
                e.append(A.plane_wave(box, s.pos, s.gridspace, s.wavenum, prop, pol))
        return cc, e
    seq_s, seq_it, unconv = 0.0, [], 0
    for s, orients in parts:
        ctx = A.Context(s.box, s.pos, s.mat, s.gridspace, s.wavenum, s.grid, nrhs_max=nrhs)
        ctx.init_dmatrix()
        cc, e = rhs(s, orients, s.box)
        for r in range(nrhs):
            ctx.set_cc(r, cc[r])
        d_e = torch.from_numpy(np.ascontiguousarray(np.stack(e)).view(np.float64)).cuda()
        st = ctx.solve_device(d_e.data_ptr(), nrhs, None, None, method=args.batch_method, prec="mixed", eps=EPS,
                              maxiter=args.batch_maxiter)
        seq_s += ctx.last_solve_ms() / 1e3
        seq_it.append(max(x["niter"] for x in st))
        unconv += sum(x["status"] != "ok" for x in st)
        ctx.close()
    # the common box rounded up to the power-of-two FFT grid of the largest particle class (compile-time transforms)
    gb = max(max(s.box) for s, _ in parts)
    g = A.Context.group([s for s, _ in parts], rhs_per_particle=nrhs, box=(gb, gb, gb))
    es = []
    for q, (s, orients) in enumerate(parts):
        cc, e = rhs(s, orients, g.box)
        for k in range(nrhs):
            g.set_cc(q * nrhs + k, cc[k])
        es.append(g.group_pad(np.stack(e), q))
    d_e = torch.from_numpy(np.ascontiguousarray(np.concatenate(es)).view(np.float64)).cuda()
    st = g.solve_device(d_e.data_ptr(), nrhs * len(parts), None, None, method=args.batch_method, prec="mixed",
                        eps=EPS, maxiter=args.batch_maxiter)
    grp_s = g.last_solve_ms() / 1e3
    gunconv = sum(x["status"] != "ok" for x in st)
    out = {"workload": "%d seeded ellipsoids with boxes of 24 or 32 (dpl 17) x 16 orientations x 2 polarisations "
                       "(%d RHS), mixed %s to 1e-5" % (len(parts), nrhs * len(parts), args.batch_method),
           "boxes": [list(s.box) for s, _ in parts], "group_box": list(g.box), "group_grid": list(g.grid),
           "one_context_per_particle": {"solve_s": seq_s, "rhs_per_s": nrhs * len(parts) / seq_s,
                                        "max_iterations_per_particle": seq_it, "rhs_not_converged": unconv},
           "group_context": {"solve_s": grp_s, "rhs_per_s": nrhs * len(parts) / grp_s,
                             "max_iterations": max(x["niter"] for x in st), "rhs_not_converged": gunconv}}
    g.close()
    return out


def run_profile(args):
    """small, fixed workloads for ncu: 'solve' = one warm-up + one mixed solve of the bench workload;
    'matvec' = three FP32 matvecs (2 RHS) of the bench workload; 'surface' = three FP32 matvecs (2 RHS) of the
    bench workload's substrate variant"""
    import torch
    import adda_gb300 as A
    surf = dict(h=30.0 * args.grid / 128, msub=1.5, relation="img") if args.mode == "profile-surface" else None
    s = A.Setup(grid=args.grid, m=M_REF, dpl=DPL, prop=[0, 0, -1] if surf else None, surface=surf)
    ctx = A.Context.from_setup(s, nrhs_max=2)
    torch.cuda.synchronize()
    if args.mode == "profile-solve":
        einc = np.ascontiguousarray(np.stack(s.einc))
        d_e = torch.from_numpy(einc.view(np.float64)).cuda()
        for _ in range(2):
            st = ctx.solve_device(d_e.data_ptr(), 2, None, None, method=args.method, prec="mixed", eps=EPS,
                                  maxiter=args.maxiter)
        print(json.dumps({"mode": args.mode, "ms": ctx.last_solve_ms(), "stats": st}))
    else:
        ms = ctx.time_matvec("fp32", 2, iters=3)
        slab_mb = 2 * 3 * s.grid[2] * s.box[1] * 8 / 2 ** 20
        print(json.dumps({"mode": args.mode, "fp32_matvec_ms": ms, "shape": list(ctx.fft_shape("fp32")),
                          "chunk_slabs": ctx.l2_chunk("fp32"), "chunk_mb": ctx.l2_chunk("fp32") * slab_mb}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--method", default="qmr", choices=["qmr", "bicgstab"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-surface", action="store_true", help="skip the substrate variant of the workload")
    ap.add_argument("--no-scale", action="store_true", help="skip the scale workload (256^3 sphere, 512^3 grid)")
    ap.add_argument("--group-particles", type=int, default=8,
                    help="small seeded ellipsoids solved one context each and as one group context (0 skips)")
    ap.add_argument("--batch-particles", type=int, default=4,
                    help="time the batching workload (64 seeded ellipsoids x 16 orientations) on this many particles "
                         "(0: skip)")
    ap.add_argument("--batch-maxiter", type=int, default=4000, help="iteration cap per particle of the batching workload")
    ap.add_argument("--batch-method", default="bicgstab", choices=["qmr", "bicgstab"])
    ap.add_argument("--scale-maxiter", type=int, default=300, help="iteration cap of the scale workload")
    ap.add_argument("--scale-method", default="bicgstab", choices=["qmr", "bicgstab"])
    ap.add_argument("--mode", default="bench", choices=["bench", "profile-solve", "profile-matvec", "profile-surface"])
    ap.add_argument("--grid", type=int, default=GRID, help="sphere box size for the profile modes")
    ap.add_argument("--maxiter", type=int, default=100000, help="iteration cap of the profile-solve mode")
    args = ap.parse_args()
    if args.mode != "bench":
        run_profile(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
