"""Benchmark of the nodal linear-elastic multigrid solve on GB300.

Workload (default, --config c2): 257^3 nodes on the unit cube, a cubic
Voronoi polycrystal of 64 grains (C11=1.68, C12=1.21, C44=0.75, Haar-random
rotations), uniaxial_stress_clamp loading u_x = 0.01 on the x+ face; stiffness
is major-minor (21 values per node).  Synthetic inputs, seeded, generated in
numpy (alamo_gb300/workloads.py) so both arms see the same bytes.

One step = one complete solve from the inputs resident in HBM: SetModel
(stiffness layout change), prepareForSolve (stiffness coarsening, diagonals,
bottom-level inverse), the learned initial guess (U-Net on the 65^3 level,
with its residual-based fallback to zero; --guess '' skips it), the Newton
right-hand side and the solve to 1e-8 relative residual (inf-norm of the
FP64 residual, tol_abs = 0).  Fast path: FGMRES preconditioned by one
V(1,1)-cycle, both in FP32, inside FP64 iterative refinement, with a direct
solve on a 5^3-node bottom level.  Two FP64 GPU comparisons: the reference's
algorithm (MLMG iterations that are F-cycles -- the reference sets
max_fmg_iter = 100000000 -- with V(2,2) damped-Jacobi smoothing and the
BiCGStab bottom, from zero), and FP64 FGMRES(V(1,1)) with the same direct
5^3 bottom as the fast path (what the solver choice buys without FP32).
`value` is seconds per solve (lower is better); `e2e` is the same solve
through the C ABI with host buffers (stiffness and right-hand side copied
in, displacement copied out, inside the timed region).

The CPU leg runs the reference's CPU path, restated in oracle/ (the
reference itself needs AMReX and cannot be built), on all host cores: one
whole FP64 solve to 1e-8 with the reference's solver settings, timed, then
continued to 1e-12 (untimed) as the FP64 oracle solution every GPU result's
error is stated against.  --impl reference times that same whole solve.

Other workloads (--extra, on by default): config 1 (33^3 inclusion: Fapply
and solve against the oracle), config 3 (513^3 spheres, mixed against FP64),
config 4 (held-out learned-guess evaluation at 129^3 and 257^3) and config 5
(256-grain polycrystal, learned guess + mixed against FP64).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# bytes each kernel family must move per fine-level node (each array once)
BYTES_PER_NODE = {
    "jacobi_f32": {2: 56, 21: 132},
    "jacobi_f64": {2: 112, 21: 264},
    "residual_f64": {2: 88, 21: 240},
    "residual_f32": {2: 44, 21: 120},
    "fapply_f64": {2: 64, 21: 216},
    "fapply_f32": {2: 32, 21: 108},
    # double-float outer residual: x, b and the stiffness as FP32 pairs in,
    # r rounded to FP32 out
    "residual_df": {2: 76, 21: 228},
}
FAMILY = {"fapply_f64": 0, "jacobi_f64": 1, "residual_f64": 2, "fapply_f32": 3, "jacobi_f32": 4, "residual_f32": 5,
          "restrict": 6, "prolong": 7, "bottom": 8, "krylov": 9, "residual_df": 10}
# dram__bytes_read.sum + dram__bytes_write.sum of one fine-level Jacobi
# sweep, from ncu captures at 129^3: the interior sweep per node (284.7 MB +
# 20.3 MB over 2,146,689 nodes; it streams every array once, so it scales
# with the nodes) and the boundary-face kernel per boundary node (28.1 MB +
# 0.1 MB over 98,306 boundary nodes); (per node, per boundary node).  The
# isotropic sweep's interior from a 257^3 capture (757.9 MB + 183.8 MB over
# 16,974,593 nodes); its faces were not captured (None: the figure is the
# interior sweep's alone)
TRAFFIC_PER_NODE = {("jacobi_f32", 21): ((284.697344e6 + 20.251904e6) / 2146689, (28.08704e6 + 0.097536e6) / 98306),
                    ("jacobi_f32", 2): ((757.910784e6 + 183.846656e6) / 16974593, None)}
TOL = 1e-8          # the metric's relative residual
ORACLE_TOL = 1e-10  # the FP64 oracle solution errors are stated against (FP64 rounding floors near 1e-11 at 257^3)
REF_BUDGET_S = 150.0  # --impl reference: start another whole solve only within this


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="agb", choices=["agb", "reference"])
    p.add_argument("--config", default="c2", choices=["c1", "c2", "c3"])
    p.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    p.add_argument("--solver", default="fgmres", choices=["fgmres", "vcycle"])
    p.add_argument("--inner", type=int, default=2, help="FP32 V-cycles per FP64 residual (vcycle solver)")
    p.add_argument("--inner-tol", type=float, default=1e-4, help="FP32 FGMRES reduction per FP64 residual")
    p.add_argument("--krylov", type=int, default=20)
    p.add_argument("--pre", type=int, default=1, help="Fsmooth calls before restriction in the FP32 V-cycle")
    p.add_argument("--post", type=int, default=1, help="Fsmooth calls after prolongation in the FP32 V-cycle")
    p.add_argument("--smoother", default="jacobi", choices=["jacobi", "gs"],
                   help="FP32 smoother: damped Jacobi (the reference's) or multicolour Gauss-Seidel")
    p.add_argument("--precond", default="v", choices=["v", "f"],
                   help="FGMRES preconditioner: one V-cycle or one F-cycle")
    p.add_argument("--outer", default="dfloat", choices=["fp64", "dfloat"],
                   help="outer residual and update of the mixed solve: FP64 or double-float on the FP32 pipe")
    p.add_argument("--no-plain", action="store_true", help="skip the FP64 comparison solves")
    p.add_argument("--no-cpu", action="store_true", help="skip the oracle (CPU baseline and error reference)")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-extra", action="store_true", help="skip configs 1, 3, 4 and 5")
    p.add_argument("--n", type=int, default=0, help="override the grid size (nodes per axis)")
    p.add_argument("--guess", default=os.path.join(ROOT, "alamo_gb300", "weights", "unet65.npy"),
                   help="U-Net weights of the learned initial guess ('' = solve from zero)")
    return p.parse_args()


def workload(cfg, n_override=0):
    """(name, n, C, F0, bc, dx) from the numpy generators (no CUDA library)."""
    from alamo_gb300 import bc as B
    from alamo_gb300 import workloads as W
    if cfg == "c1":
        n = n_override or 33
        C, F0, dx = W.inclusion_iso(n)
        return ("c1: %d^3 isotropic inclusion r=0.25 contrast 10, eigenstrain 0.01 I, zero-displacement faces" % n,
                n, C, F0, B.Constant(), dx)
    if cfg == "c2":
        n = n_override or 257
        C, dx = W.voronoi_cubic(n, 64, seed=1)
        return ("c2: %d^3 cubic Voronoi polycrystal, 64 grains, C11/C12/C44=1.68/1.21/0.75, "
                "uniaxial_stress_clamp u_x=0.01" % n, n, C, None, B.TensionTest("uniaxial_stress_clamp", disp=0.01),
                dx)
    n = n_override or 513
    C, F0, dx, placed = W.spheres_diffuse(n, 200, seed=3)
    return ("c3: %d^3 isotropic two-phase, %d spheres r in [0.02,0.06] with a diffuse interface of 4 node spacings, "
            "contrast 10, eigenstrain U[0,0.02]" % (n, placed), n, C, F0, B.Constant(), dx)


def config_dict(name, n, C):
    """The workload description both arms print (identical on both)."""
    return {"workload": name, "nodes": n ** 3, "tolerance": "%g relative inf-norm residual, tol_abs 0" % TOL,
            "l2": "inputs larger than L2 (%.1f GB of stiffness), no flush needed" % (C.nbytes / 1e9)}


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a run."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def nlevels(n):
    lev, m = 1, n
    while (m - 1) % 2 == 0 and (m - 1) // 2 >= 2:
        m = (m - 1) // 2 + 1
        lev += 1
    return lev


def rel_err(u, ref):
    """{rel_inf, rel_l2} of u against ref."""
    d = np.asarray(u) - np.asarray(ref)
    return {"rel_inf": float(np.abs(d).max() / max(np.abs(ref).max(), 1e-300)),
            "rel_l2": float(np.sqrt((d * d).sum()) / max(np.sqrt((np.asarray(ref) ** 2).sum()), 1e-300))}


# --------------------------------------------------------------- the oracle
def load_oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    return O, threads


def oracle_solve(O, C, F0, bc, dx, refine=True):
    """The reference's CPU path (oracle restatement) on all host threads:
    Newton right-hand side at u = 0, then the FP64 MLMG solve with the
    reference's settings (F-cycles, V(2,2), BiCGStab bottom, full
    coarsening) to 1e-8, timed; with refine, continued to 1e-12 (untimed)
    for the error reference.  Returns (x_1e-8, x_1e-12 or None, info)."""
    n = C.shape[0]
    bt, bv = bc.tables()
    u = np.zeros((3, n, n, n))
    t0 = time.perf_counter()
    b = O.bc_init(u, bt, bv)
    rhs = O.build_rhs(C, F0, bt, u, b, dx)
    t_rhs = time.perf_counter() - t0
    x, rep, hist = O.solve(C, bt, rhs, dx, tol_rel=TOL)
    seconds = time.perf_counter() - t0
    info = {"seconds": seconds, "rhs_s": t_rhs, "setup_s": rep.setup_seconds, "f_cycles": rep.iters,
            "status": rep.status, "final_rel_resnorm": rep.final_resnorm / rep.rhsnorm0}
    if rep.status != 0:
        info["error"] = "the oracle's solve did not reach %g (status %d)" % (TOL, rep.status)
    xr = None
    if refine:
        # continued with the exact 5^3 bottom (the reference's BiCGStab on
        # the singular 3^3 bottom of the clamp stalls well above 1e-12)
        t1 = time.perf_counter()
        xr, rep2, _ = O.solve(C, bt, rhs, dx, tol_rel=ORACLE_TOL, x0=x, max_iter=100, bottom_solver=1,
                              max_coarsening_level=max(nlevels(n) - 2, 0))
        info["refined"] = {"tol_rel": ORACLE_TOL, "extra_f_cycles": rep2.iters, "status": rep2.status,
                           "bottom": "direct 5^3", "final_rel_resnorm": rep2.final_resnorm / rep.rhsnorm0,
                           "seconds": time.perf_counter() - t1}
    return x, xr, info


def run_reference(args):
    """--impl reference: the reference's CPU path (oracle restatement) on
    all host cores, whole FP64 solves of the same workload; rank 0 only."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    name, n, C, F0, bc, dx = workload(args.config, args.n)
    O, threads = load_oracle()
    bt, _ = bc.tables()
    # warm-up: full-size operator applications (threads started, pages touched)
    z = np.zeros((3, n, n, n))
    for _ in range(args.warmup):
        O.fapply(C, bt, z, dx)
    times, infos = [], []
    t_start = time.perf_counter()
    while len(times) < args.steps:
        _, _, info = oracle_solve(O, C, F0, bc, dx, refine=False)
        times.append(info["seconds"])
        infos.append(info)
        if time.perf_counter() - t_start + info["seconds"] > REF_BUDGET_S:
            break
    v = float(np.mean(times))
    guess = bool(args.guess) and os.path.exists(args.guess)
    cpu = {"value": v, "unit": "s", "cores": threads, "kind": "port",
           "sample": "%d whole FP64 solve(s) to %g (RHS + set-up + %d F-cycles) of the full %d^3 workload by the "
                     "oracle (C++ restatement of the reference CPU path, OpenMP) on %d host threads; warm-up: %d "
                     "full-size Fapply calls" % (len(times), TOL, infos[-1]["f_cycles"], n, threads, args.warmup),
           "solves": infos}
    line = {"impl": "reference", "metric": metric_name(n, guess),
            "value": v, "unit": "s", "n_gpus": args.gpus, "steps": len(times), "warmup": args.warmup,
            "ms_per_step": v * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "config": config_dict(name, n, C),
            "cpu_baseline": cpu, "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def metric_name(n, guess):
    """The metric string both arms print (a comparison pairs them by it)."""
    return ("solve time to 1e-8 rel. residual @%d^3: %smixed FP32/FP64 vs plain FP64; Fapply HBM GB/s"
            % (n, "learned guess + " if guess else ""))


def reduce_max(x, dist, device):
    """x maximised over the ranks of the process group (one replica per GPU;
    the slowest replica sets the whole job's time).  dist None: one rank."""
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# --------------------------------------------------------------- GPU helpers
def fast_opts(A, n, args=None, smoother="jacobi", outer="dfloat", precond=None):
    """The fast path's options: mixed FGMRES(V(1,1)), direct 5^3 bottom,
    double-float outer residual."""
    pre = args.pre if args else 1
    post = args.post if args else 1
    kw = dict(precision=1, solver="fgmres", inner_tol=args.inner_tol if args else 1e-4,
              krylov_dim=args.krylov if args else 20, bottom_solver="direct",
              max_coarsening_level=max(nlevels(n) - 2, 0), pre_smooth=pre, post_smooth=post,
              outer_residual=outer, precond_cycle=precond or (args.precond if args else "v"))
    if smoother == "gs":
        kw["smoother"] = 1
    return A.default_opts(**kw)


def timed_solve(A, torch, n, C, F0, bc, dx, opts, net=None, repeats=1, sym=None, tol=TOL):
    """One Newton step (the linear solve from zero, or from the learned
    guess) on device-resident inputs; host wall time of the synchronous
    call, best of `repeats`.  Returns (u on the host, report, seconds)."""
    dev = torch.device("cuda", torch.cuda.current_device())
    sym = sym or ("isotropic" if C.shape[-1] == 2 else "majorminor")
    op = A.Elastic(n, dx, sym, opts)
    try:
        op.SetBC(bc)
        C_dev = torch.from_numpy(C).to(dev)
        F0_dev = torch.from_numpy(F0).to(dev) if F0 is not None else None
        F0keep = (A.DevicePtr(F0_dev.data_ptr()), 1) if F0_dev is not None else None
        u = torch.zeros((3, n, n, n), dtype=torch.float64, device=dev)
        b = torch.zeros_like(u)
        torch.cuda.synchronize()
        op.bc_init(A.DevicePtr(b.data_ptr()))
        newton = A.Newton(op)
        best, rep = None, None
        for _ in range(repeats):
            op.SetModel(A.DevicePtr(C_dev.data_ptr()))
            u.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            if net is not None:
                rep = newton.solve_guess(net, A.DevicePtr(u.data_ptr()), A.DevicePtr(b.data_ptr()), F0keep,
                                         tol_rel=tol, tol_abs=0.0, allow_not_converged=True)
            else:
                rep = newton.solve(A.DevicePtr(u.data_ptr()), A.DevicePtr(b.data_ptr()), F0keep, tol_rel=tol,
                                   tol_abs=0.0, allow_not_converged=True)
            torch.cuda.synchronize()
            s = time.perf_counter() - t0
            best = s if best is None else min(best, s)
        return u.cpu().numpy(), rep, best
    finally:
        op.close()


def rep_summary(rep, sec):
    d = {"seconds": sec, "cycles": rep.get("iters"), "status": rep.get("status"),
         "final_rel_resnorm": rep["final_resnorm"] / rep["rhsnorm0"] if rep.get("rhsnorm0") else None}
    if "guess_used" in rep:
        d["guess_used"] = rep["guess_used"]
    return d


def fp64_fgmres_opts(A, n, krylov=20):
    """FP64 FGMRES(V(1,1)) with the fast path's direct 5^3 bottom."""
    return A.default_opts(precision=0, solver="fgmres", krylov_dim=krylov, bottom_solver="direct",
                          max_coarsening_level=max(nlevels(n) - 2, 0), pre_smooth=1, post_smooth=1)


def guarded(fn):
    """Run one extra measurement; a failure is recorded, not raised."""
    try:
        return fn()
    except Exception as e:  # noqa: BLE001 -- reported in the line
        return {"error": "%s: %s" % (type(e).__name__, e)}


def compare_fp64(A, torch, n, C, F0, bc, dx, net, name):
    """Learned guess + mixed against the FP64 solves of the same input: the
    reference's settings (F-cycles, BiCGStab bottom) and FP64 FGMRES with the
    direct bottom; the mixed solution's error against the latter."""
    xm, repm, secm = timed_solve(A, torch, n, C, F0, bc, dx, fast_opts(A, n), net=net, repeats=2)
    out = {"workload": name, "learned_mixed": rep_summary(repm, secm),
           "timing": "host wall clock around one synchronous C-ABI call, device-resident inputs"}
    out["learned_mixed_gs_smoother"] = guarded(
        lambda: rep_summary(*timed_solve(A, torch, n, C, F0, bc, dx, fast_opts(A, n, smoother="gs"), net=net,
                                         repeats=2)[1:]))
    out["learned_mixed_fcycle_precond"] = guarded(
        lambda: rep_summary(*timed_solve(A, torch, n, C, F0, bc, dx, fast_opts(A, n, precond="f"), net=net,
                                         repeats=2)[1:]))
    x64, rep64, sec64 = timed_solve(A, torch, n, C, F0, bc, dx, fp64_fgmres_opts(A, n))
    out["fp64_fgmres_direct_bottom"] = rep_summary(rep64, sec64)
    out["mixed_vs_fp64"] = rel_err(xm, x64)
    del xm, x64

    def ref_settings():
        _, rep, sec = timed_solve(A, torch, n, C, F0, bc, dx, A.default_opts(precision=0))
        d = rep_summary(rep, sec)
        d["speedup_of_learned_mixed"] = sec / secm
        return d
    out["plain_fp64_fcycles"] = guarded(ref_settings)
    if net is not None:
        out["fallback_rate"] = float(not repm.get("guess_used", False))
    return out


def next_rows(A, torch, O, c2):
    """The rows beyond the benchmark step, each timed on the GPU (host wall
    clock around synchronous C-ABI calls) and by the oracle on all host
    threads, with the GPU result's distance from the oracle's: stress,
    strain and energy (Elastic::Stress/Strain/Energy) at 257^3, the psi
    void terms on the PlateHole plate (with its Kirsch errors), the Newton
    loop of a NeoHookean medium at 65^3, and the four-level AMR composite
    solve of the Eshelby inclusion."""
    import ctypes
    from alamo_gb300 import _lib as L
    from alamo_gb300 import bc as B
    from alamo_gb300 import workloads as W
    out = {}

    def stress():
        name, n, C, bc, dx = c2
        N = n ** 3
        u = np.random.default_rng(7).uniform(-1e-3, 1e-3, (3, n, n, n))
        dev = torch.device("cuda", torch.cuda.current_device())
        u_d = torch.from_numpy(u).to(dev)
        s_d = torch.empty(9 * N, dtype=torch.float64, device=dev)
        e_d = torch.empty(9 * N, dtype=torch.float64, device=dev)
        w_d = torch.empty(N, dtype=torch.float64, device=dev)
        with A.Elastic(n, dx, "majorminor") as op:
            op.SetModel(np.ascontiguousarray(C))
            op.SetBC(bc)

            def call():
                L.check(L.lib().agb_elastic_stress_strain(
                    op.h, ctypes.c_void_p(u_d.data_ptr()), None, 0, ctypes.c_void_p(s_d.data_ptr()),
                    ctypes.c_void_p(e_d.data_ptr()), ctypes.c_void_p(w_d.data_ptr()), L.MEM_DEVICE))
            call()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(5):
                call()
            torch.cuda.synchronize()
            sec = (time.perf_counter() - t0) / 5
        nbytes = N * (24 + 8 * C.shape[-1] + 72 + 72 + 8)
        d = {"workload": name + "; u uniform in [-1e-3, 1e-3]", "seconds": sec,
             "bytes_per_node": nbytes // N, "achieved_gbs": nbytes / sec / 1e9}
        if O:
            t0 = time.perf_counter()
            so, eo, wo = O.stress_strain(C, None, u, dx)
            d["oracle_seconds"] = time.perf_counter() - t0
            d["stress_vs_oracle"] = rel_err(s_d.view(n, n, n, 9).cpu().numpy(), so.reshape(n, n, n, 9))
            d["strain_vs_oracle"] = rel_err(e_d.view(n, n, n, 9).cpu().numpy(), eo.reshape(n, n, n, 9))
        return d
    out["stress_strain"] = guarded(stress)

    def psi():
        nxy, nz = 129, 17
        C, pc, bc, dx = W.platehole(nxy, nz)
        opts = A.default_opts(precision="fp64", solver="vcycle", bottom_solver="smoother", max_iter=400)
        with A.Elastic((nxy, nxy, nz), dx, "isotropic", opts) as op:
            op.SetModel(np.ascontiguousarray(C))
            op.SetBC(bc)
            op.SetPsi(pc, W.PLATEHOLE_SMALL)
            b = op.bc_init()
            u = np.zeros((3, nz, nxy, nxy))
            t0 = time.perf_counter()
            rep = A.Newton(op).solve(u, b, None, tol_rel=1e-10, tol_abs=1e-16)
            sec = time.perf_counter() - t0
            sg = op.stress_strain(u)[0]
        j = int(round((2.0 + W.PLATEHOLE_HALF) / dx))
        row = sg[nz // 2, j]
        xs = -W.PLATEHOLE_HALF + dx * np.arange(nxy)
        err = W.platehole_errors(xs, row[:, 0, 0], row[:, 1, 1], row[:, 0, 1])
        d = {"workload": "PlateHole restated as a z-invariant %d^2 x %d plate, psi void of radius 1" % (nxy, nz),
             "gpu": rep_summary(rep, sec), "kirsch_errors_xx_yy_xy": [float(e) for e in err],
             "kirsch_tolerance": 0.01}
        if O:
            bt, bv = bc.tables()
            O.set_psi(pc, W.PLATEHOLE_SMALL)
            try:
                t0 = time.perf_counter()
                zero = np.zeros_like(u)
                rhs = O.build_rhs(C, None, bt, zero, O.bc_init(np.zeros_like(u), bt, bv), dx)
                xo, rep_o, _ = O.solve(C, bt, rhs, dx, tol_rel=1e-10, tol_abs=1e-16,
                                       opts=O.default_opts(bottom_solver=2, max_iter=400))
                d["oracle_seconds"] = time.perf_counter() - t0
                d["oracle_cycles"] = rep_o.iters
            finally:
                O.set_psi(None)
            d["gpu_vs_oracle"] = rel_err(u, xo)
        return d
    out["psi_platehole"] = guarded(psi)

    def newton():
        n, nri = 65, 4
        model, bc, dx = W.neohookean_twophase(n)
        mcl = max(nlevels(n) - 2, 0)
        opts = A.default_opts(precision="mixed", solver="fgmres", bottom_solver="direct", max_coarsening_level=mcl)
        with A.Elastic(n, dx, "major", opts) as op:
            op.SetBC(bc)
            b = op.bc_init()
            u = np.zeros((3, n, n, n))
            t0 = time.perf_counter()
            rep = A.Newton(op, nriters=nri).solve_neohookean(np.ascontiguousarray(model), u, b, tol_rel=1e-10)
            sec = time.perf_counter() - t0
        d = {"workload": "two-phase NeoHookean cube %d^3, clamped x faces, u_x = 0.02, %d Newton iterations"
                         % (n, nri), "gpu_seconds": sec, "last_increment": rep["relnorm"]}
        if O:
            bt, bv = bc.tables()
            t0 = time.perf_counter()
            x = np.zeros((3, n, n, n))
            b0 = O.bc_init(x, bt, bv)
            for _ in range(nri):
                dw, ddw = O.neohookean_field(model, x, dx)
                rhs = O.rhs_dw(dw, bt, x, b0, dx)
                du, rep_o, _ = O.solve(np.ascontiguousarray(ddw), bt, rhs, dx, tol_rel=1e-10, max_iter=200,
                                       bottom_solver=1, max_coarsening_level=mcl)
                x = x + du
            d["oracle_seconds"] = time.perf_counter() - t0
            d["gpu_vs_oracle"] = rel_err(u, x)
        return d
    out["newton_neohookean"] = guarded(newton)

    def amr():
        from alamo_gb300.composite import Composite
        n0, dx0, boxes, Cs, F0s, hw = W.eshelby_amr_levels()
        mcl = nlevels(n0) - 2
        opts = A.default_opts(precision=0, bottom_solver="direct", max_coarsening_level=mcl, max_iter=80)
        with Composite(n0, dx0, boxes, "isotropic", opts) as c:
            c.SetBC(B.Constant())
            for l, C in enumerate(Cs):
                c.SetModel(l, C)
            t0 = time.perf_counter()
            ug, itg, rn = c.solve(F0=F0s, tol_rel=1e-7)
            sec = time.perf_counter() - t0
        d = {"workload": "Eshelby inclusion, 4 levels: 65^3 and boxes of 63^3, 63^3, 95^3 valid nodes",
             "gpu_seconds": sec, "iterations": itg, "final_rel_resnorm": rn}
        if O:
            import composite as CP
            bt, bv = B.Constant().tables()
            levels = [CP.Level((n0,) * 3, dx0, None, (n0,) * 3, Cs[0], bt, bv)]
            for l, (lo, nv) in enumerate(boxes, start=1):
                levels.append(CP.Level((nv + 2,) * 3, dx0 / 2 ** l, (lo,) * 3, (nv,) * 3, Cs[l], bt, bv))
            oo = O.default_opts(max_fmg_iter=0, bottom_solver=1, max_coarsening_level=mcl)
            t0 = time.perf_counter()
            uo, ito, _ = CP.Composite(levels, F0s=F0s, opts0=oo, optsf=oo).solve(tol_rel=1e-7, max_iter=80)
            d["oracle_seconds"] = time.perf_counter() - t0
            d["oracle_iterations"] = ito
            d["gpu_vs_oracle_max_over_levels"] = max(rel_err(a, b_)["rel_inf"] for a, b_ in zip(ug, uo))
        return d
    out["amr_composite"] = guarded(amr)
    return out


def extra_configs(A, torch, net, O, args):
    """Configs 1, 3, 4 and 5, each in minutes at most."""
    from alamo_gb300 import bc as B
    from alamo_gb300 import learn
    from alamo_gb300 import workloads as W
    out = {}

    def c1():
        # 33^3 inclusion: Fapply on U[-1,1] against the oracle, and the FP64
        # V(2,2) V-cycle iteration to 1e-10 against the oracle's
        name, n, C, F0, bc, dx = workload("c1")
        bt, bv = bc.tables()
        u = A.synth.uniform(A.synth.SEED_FAPPLY, (3, n, n, n))
        with A.Elastic(n, dx, "isotropic") as op:
            op.SetModel(np.ascontiguousarray(C))
            op.SetBC(bc)
            f = op.Fapply(u)
        d = {"workload": name, "fapply_vs_oracle": rel_err(f, O.fapply(C, bt, u, dx)) if O else None}
        x, rep, sec = timed_solve(A, torch, n, C, F0, bc, dx, A.default_opts(precision=0, max_fmg_iter=0), tol=1e-10)
        d["fp64_vcycles_to_1e-10"] = rep_summary(rep, sec)
        if O:
            b0 = O.bc_init(np.zeros((3, n, n, n)), bt, bv)
            rhs = O.build_rhs(C, F0, bt, np.zeros((3, n, n, n)), b0, dx)
            xo, rep_o, _ = O.solve(C, bt, rhs, dx, tol_rel=1e-10, max_fmg_iter=0)
            d["solution_vs_oracle_1e-10"] = rel_err(x, xo)
        return d
    out["c1"] = guarded(c1)

    def c3():
        name, n, C, F0, bc, dx = workload("c3")
        return compare_fp64(A, torch, n, C, F0, bc, dx, net, name)
    out["c3"] = guarded(c3)

    def c4():
        # held-out learned-guess evaluation on the training distribution
        # (inclusion media, zero-displacement faces)
        d = {}
        for n, count in ((129, 6), (257, 3)):
            rng = np.random.default_rng(1000003 + n)
            rows = []
            for _ in range(count):
                C, F0, dx = learn.inclusion_medium(n, rng)
                o = fast_opts(A, n)
                x0, r0, s0 = timed_solve(A, torch, n, C, F0, B.Constant(), dx, o, repeats=2)
                x1, r1, s1 = timed_solve(A, torch, n, C, F0, B.Constant(), dx, o, net=net, repeats=2)
                rows.append({"zero": rep_summary(r0, s0), "guess": rep_summary(r1, s1),
                             "guess_vs_zero_solution": rel_err(x1, x0)})
            used = [r["guess"]["guess_used"] for r in rows]
            d["%d^3" % n] = {"seeds": count, "fallback_rate": 1.0 - float(np.mean(used)),
                             "cycles_zero": float(np.mean([r["zero"]["cycles"] for r in rows])),
                             "cycles_guess": float(np.mean([r["guess"]["cycles"] for r in rows])),
                             "s_zero": float(np.mean([r["zero"]["seconds"] for r in rows])),
                             "s_guess": float(np.mean([r["guess"]["seconds"] for r in rows])), "runs": rows}
        return d
    if net is not None:
        out["c4"] = guarded(c4)

    def c5():
        n = 257
        C, dx = W.voronoi_cubic(n, 256, seed=5)
        bc = B.TensionTest("uniaxial_stress_clamp", disp=0.01)
        return compare_fp64(A, torch, n, C, None, bc, dx, net,
                            "c5: 257^3 cubic Voronoi polycrystal, 256 grains, uniaxial_stress_clamp u_x=0.01")
    out["c5"] = guarded(c5)
    return out


# --------------------------------------------------------------- GPU arm
def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import ctypes

    import torch

    import alamo_gb300 as A
    from alamo_gb300 import _lib

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl", rank=rank, world_size=world)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    name, n, C, F0, bc, dx = workload(args.config, args.n)
    N = n ** 3
    nc = C.shape[-1]
    sym = "isotropic" if nc == 2 else "majorminor"
    prec = 1 if args.precision == "mixed" else 0
    # the mixed FGMRES path runs V(1,1) as its preconditioner (fewer fine sweeps
    # per Krylov step; 53 steps of V(1,1) beat 36 of V(2,2) at 257^3); the
    # FP64 arms keep the reference's V(2,2)
    pre, post = (args.pre, args.post) if prec else (2, 2)
    okw = dict(precision=prec, inner_cycles=args.inner, solver=args.solver, inner_tol=args.inner_tol,
               krylov_dim=args.krylov, bottom_solver="direct", max_coarsening_level=max(nlevels(n) - 2, 0),
               pre_smooth=pre, post_smooth=post, precond_cycle=args.precond)
    if args.smoother == "gs":
        okw["smoother"] = 1
    if prec:
        okw["outer_residual"] = args.outer
    opts = A.default_opts(**okw)
    op = A.Elastic(n, dx, sym, opts)
    stream = torch.cuda.Stream()
    _lib.check(_lib.lib().agb_elastic_set_stream(op.h, ctypes.c_void_p(stream.cuda_stream)))
    op.SetBC(bc)
    dev = torch.device("cuda", local)
    C_dev = torch.from_numpy(C).to(dev)
    F0_dev = torch.from_numpy(F0).to(dev) if F0 is not None else None
    u_dev = torch.zeros((3, n, n, n), dtype=torch.float64, device=dev)
    b_dev = torch.zeros_like(u_dev)
    torch.cuda.synchronize()
    op.bc_init(A.DevicePtr(b_dev.data_ptr()))
    P = A.DevicePtr
    F0arg = (P(F0_dev.data_ptr()), 1) if F0_dev is not None else None
    newton = A.Newton(op)
    reports = []
    guesses = []
    net = None
    if args.guess and os.path.exists(args.guess):
        from alamo_gb300 import learn
        net = learn.UNet(65)
        net.load(args.guess)

    def step():
        op.SetModel(P(C_dev.data_ptr()))
        if net is not None:
            # learned initial guess with its residual-based fallback (zero
            # when the fallback fires) as the first iterate of the Newton
            # step's linear solve, in one call
            r = newton.solve_guess(net, P(u_dev.data_ptr()), P(b_dev.data_ptr()), F0arg, tol_rel=TOL, tol_abs=0.0)
            guesses.append({"used": r["guess_used"]})
            reports.append(r)
        else:
            with torch.cuda.stream(stream):
                u_dev.zero_()
            reports.append(newton.solve(P(u_dev.data_ptr()), P(b_dev.data_ptr()), F0arg, tol_rel=TOL,
                                        tol_abs=0.0))

    for _ in range(args.warmup):
        step()
    reports.clear()
    guesses.clear()
    op.profile(True)
    launches0 = op.launch_count()
    clocks = Clocks(local)
    clocks.start()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    barrier()
    ck = clocks.stop()
    launches = op.launch_count() - launches0
    sec = e0.elapsed_time(e1) / 1e3 / args.steps
    fam = {k: op.profile_get(v) for k, v in FAMILY.items()}
    krylov_bytes = op.profile_bytes(FAMILY["krylov"])
    op.profile(False)
    sec = reduce_max(sec, dist, dev)
    u_fast = u_dev.cpu().numpy()

    # dominant fine-level kernel and its roofline
    peaks, peak_kind = measured_peaks()
    tot = {k: v[1] for k, v in fam.items() if k in BYTES_PER_NODE and v[0] > 0}
    dom = max(tot, key=tot.get) if tot else None
    roof = None
    if dom:
        cnt, ms = fam[dom]
        per_launch_s = ms / cnt / 1e3
        alg_bytes = BYTES_PER_NODE[dom][nc] * N
        achieved = alg_bytes / per_launch_s / 1e9
        traf = TRAFFIC_PER_NODE.get((dom, nc)) if args.smoother == "jacobi" else None
        nb = N - (n - 2) ** 3  # boundary nodes
        roof = {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"],
                "traffic": (traf[0] * N + (traf[1] * nb if traf[1] is not None else 0.0)) if traf else None,
                "traffic_covers": (("interior sweep and boundary faces" if traf[1] is not None else
                                    "interior sweep only") if traf else None),
                "peak_source": peak_kind, "launches": cnt, "avg_launch_ms": ms / cnt,
                "alg_bytes_per_launch": alg_bytes, "share_of_step": ms / 1e3 / (sec * args.steps)}
    kernels = {k: {"launches": v[0], "ms": v[1]} for k, v in fam.items() if v[0] > 0}
    if fam["krylov"][0] > 0:
        # Gram-Schmidt and the other FGMRES vector kernels: algorithmic bytes
        # (every Krylov vector read or written once per launch) over their time
        kb = kernels["krylov"]
        kb["alg_bytes"] = krylov_bytes
        kb["achieved_gbs"] = krylov_bytes / (kb["ms"] / 1e3) / 1e9
        kb["frac_of_hbm_peak"] = kb["achieved_gbs"] / peaks["hbm_gbs"]

    # e2e through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        C_h = torch.from_numpy(C).pin_memory()
        b_h = b_dev.cpu().pin_memory()
        u_h = torch.zeros_like(b_h).pin_memory()
        F0_h = torch.from_numpy(F0).pin_memory() if F0 is not None else None

        def step_host():
            op.SetModel(C_h.numpy())
            F0x = F0_h.numpy() if F0_h is not None else None
            if net is not None:
                newton.solve_guess(net, u_h.numpy(), b_h.numpy(), F0x, tol_rel=TOL, tol_abs=0.0)
            else:
                u_h.zero_()
                newton.solve(u_h.numpy(), b_h.numpy(), F0x, tol_rel=TOL, tol_abs=0.0)

        step_host()
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            step_host()
        barrier()
        wall = (time.perf_counter() - t0) / args.steps
        wall = reduce_max(wall, dist, dev)
        vec = 3 * N * 8
        # stiffness, b (and F0) in, u out; the guess path's u is output only,
        # the plain Newton step copies its zero u in
        h2d = C.nbytes + (vec if net is not None else 2 * vec) + (F0.nbytes if F0 is not None else 0)
        d2h = vec
        e2e = {"value": wall, "unit": "s", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "timing": "host wall clock around synchronous C-ABI calls"}

    # FP64 GPU solves of the same input: (1) the reference's solver
    # settings (MLMG iterations that are all F-cycles, V(2,2), BiCGStab
    # bottom, full coarsening); (2) FP64 FGMRES(V(1,1)) with the fast path's
    # direct 5^3 bottom -- the solver without FP32
    plain, fp64_fgmres, u64 = None, None, None
    fp64_outer, u_fp64_outer = None, None
    if not args.no_plain and prec:
        # the fast path with the FP64 outer residual and update instead of
        # the double-float ones
        try:
            u_fp64_outer, r, s = timed_solve(A, torch, n, C, F0, bc, dx, fast_opts(A, n, args, outer="fp64"),
                                             net=net, repeats=3)
            fp64_outer = rep_summary(r, s)
            fp64_outer["solution_vs_fast_path"] = rel_err(u_fp64_outer, u_fast)
        except A.AgbError as e:
            fp64_outer = {"error": str(e)}
    # the colour-ordered (multicolour Gauss-Seidel) smoother in place of
    # damped Jacobi, same solver otherwise: cycles and time
    gs_arm = None
    if not args.no_plain and prec:
        def gs_run():
            ug, r, s = timed_solve(A, torch, n, C, F0, bc, dx, fast_opts(A, n, args, smoother="gs"), net=net,
                                   repeats=2)
            d = rep_summary(r, s)
            d["solution_vs_fast_path"] = rel_err(ug, u_fast)
            d["jacobi_cycles"] = reports[-1].get("iters") if reports else None
            return d
        gs_arm = guarded(gs_run)
    if not args.no_plain:
        try:
            u64, r, s = timed_solve(A, torch, n, C, F0, bc, dx, A.default_opts(precision=0))
            plain = rep_summary(r, s)
            plain["cycle"] = "F (max_fmg_iter 100000000), V(2,2), BiCGStab bottom, full coarsening"
        except A.AgbError as e:
            plain = {"error": str(e)}
        try:
            u64g, r, s = timed_solve(A, torch, n, C, F0, bc, dx, fp64_fgmres_opts(A, n, args.krylov), repeats=2)
            fp64_fgmres = rep_summary(r, s)
            fp64_fgmres["cycle"] = "FP64 FGMRES(%d) preconditioned by V(1,1), direct 5^3 bottom" % args.krylov
            fp64_fgmres["fast_path_speedup"] = s / sec
            del u64g
        except A.AgbError as e:
            fp64_fgmres = {"error": str(e)}

    # Fapply throughput (fine level, FP64 and FP32), 20 launches each
    op.SetModel(P(C_dev.data_ptr()))
    op.prepareForSolve()
    f_dev = torch.empty_like(u_dev)
    x_dev = torch.rand_like(u_dev)
    op.profile(True)
    for _ in range(20):
        op.Fapply(P(x_dev.data_ptr()), P(f_dev.data_ptr()))
    x32, f32 = x_dev.float(), torch.empty_like(x_dev, dtype=torch.float32)
    torch.cuda.synchronize()
    for _ in range(20):
        _lib.check(_lib.lib().agb_elastic_fapply_f32(op.h, 0, ctypes.c_void_p(x32.data_ptr()),
                                                     ctypes.c_void_p(f32.data_ptr()), 1))
    fap = {}
    for key, famid in [("fp64", FAMILY["fapply_f64"]), ("fp32", FAMILY["fapply_f32"])]:
        cnt, ms = op.profile_get(famid)
        per = ms / cnt / 1e3
        bpn = BYTES_PER_NODE["fapply_f64" if key == "fp64" else "fapply_f32"][nc]
        fap[key] = {"node_updates_per_s": N / per, "hbm_gbs": bpn * N / per / 1e9, "ms": per * 1e3,
                    "frac_of_hbm_peak": bpn * N / per / 1e9 / peaks["hbm_gbs"]}
    op.profile(False)
    del f_dev, x_dev, x32, f32

    # the oracle: CPU baseline (one whole solve to 1e-8) and the FP64
    # solution (continued to 1e-12) the GPU results are measured against
    cpu, oracle_err, O = None, None, None
    if rank == 0 and not args.no_cpu:
        O, threads = load_oracle()
        xo8, xo12, info = oracle_solve(O, C, F0, bc, dx, refine=True)
        bt, _ = bc.tables()
        fap_t = []
        for _ in range(5):
            t3 = time.perf_counter()
            O.fapply(C, bt, xo8, dx)
            fap_t.append(time.perf_counter() - t3)
        cpu = {"value": info["seconds"], "unit": "s", "cores": threads, "kind": "port",
               "sample": "one whole FP64 solve to %g (RHS + set-up + %d F-cycles) of the full %d^3 workload by the "
                         "oracle (C++ restatement of the reference CPU path, OpenMP) on %d host threads"
                         % (TOL, info["f_cycles"], n, threads),
               "solve": info, "fapply_s": float(np.median(fap_t)),
               "fapply_node_updates_per_s": float(N / np.median(fap_t))}
        ref = xo12 if xo12 is not None else xo8
        oracle_err = {"reference": "oracle FP64 solve continued to %g" % ORACLE_TOL,
                      "fast_path": rel_err(u_fast, ref),
                      "oracle_at_1e-8": rel_err(xo8, ref)}
        if u64 is not None:
            oracle_err["plain_fp64_gpu"] = rel_err(u64, ref)
        if u_fp64_outer is not None:
            oracle_err["fast_path_fp64_outer"] = rel_err(u_fp64_outer, ref)
        del xo8, xo12, ref

    extra = None
    op.close()
    del C_dev, F0_dev, u_dev, b_dev
    torch.cuda.empty_cache()
    nextr = None
    if rank == 0 and not args.no_extra and args.config == "c2" and not args.n:
        extra = guarded(lambda: extra_configs(A, torch, net, O, args))
        nextr = guarded(lambda: next_rows(A, torch, O, (name, n, C, bc, dx)))

    rep = reports[-1] if reports else {}
    line = {
        "metric": metric_name(n, net is not None),
        "value": sec, "unit": "s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": sec * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32-cycle/f64-refinement" if prec else "f64", "data": "synthetic",
        "config": config_dict(name, n, C),
        "gpu_solver": {"precision": args.precision, "solver": args.solver, "inner_tol": args.inner_tol,
                       "outer_residual": (args.outer if prec else "fp64"),
                       "krylov_dim": args.krylov, "bottom": "direct 5^3",
                       "preconditioner": {"v": "one V-cycle", "f": "one F-cycle"}[args.precond],
                       "smoothing": "V(%d,%d), %s" % (pre, post, "2 damped-Jacobi sweeps per Fsmooth call"
                                                      if args.smoother == "jacobi" else
                                                      "multicolour Gauss-Seidel sweeps"),
                       "parallelism": "replicas" if world > 1 else "single-gpu"},
        "e2e": e2e, "gpu_launches": launches, "roofline": roof, "cpu_baseline": cpu, "clocks": ck,
        "error_vs_fp64_oracle": oracle_err,
        "guess": ({"weights": os.path.relpath(args.guess, ROOT), "network_grid": 65,
                   "used_fraction": float(np.mean([g["used"] for g in guesses])) if guesses else None}
                  if net is not None else None),
        "solve": {"v_cycles": rep.get("iters"), "fp64_residuals": rep.get("fp64_residuals"),
                  "final_rel_resnorm_l2": (rep.get("final_resnorm_l2", 0) / rep["rhsnorm_l2"]) if rep else None,
                  "final_rel_resnorm": (rep.get("final_resnorm", 0) / rep["rhsnorm0"]) if rep else None,
                  "levels": rep.get("nlevels")},
        "plain_fp64": plain, "fp64_fgmres": fp64_fgmres, "fast_path_fp64_outer_residual": fp64_outer,
        "fast_path_gs_smoother": gs_arm,
        "speedup_vs_plain_fp64": (plain["seconds"] / sec) if plain and "seconds" in plain else None,
        "fapply": fap, "kernels_in_timed_region": kernels, "other_configs": extra, "next_rows": nextr,
    }
    if rank == 0:
        print(json.dumps(line))
    if net is not None:
        net.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
