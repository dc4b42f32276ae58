"""Benchmark of the nodal linear-elastic multigrid solve on GB300.

Workload (default, --config c2): 257^3 nodes on the unit cube, a cubic
Voronoi polycrystal of 64 grains (C11=1.68, C12=1.21, C44=0.75, Haar-random
rotations), uniaxial_stress_clamp loading u_x = 0.01 on the x+ face; stiffness
is major-minor (21 values per node).  Synthetic inputs, seeded.

One step = one complete solve from the inputs resident in HBM: SetModel
(stiffness layout change), prepareForSolve (stiffness coarsening, diagonals,
bottom-level inverse), the learned initial guess (U-Net on the 65^3 level,
with its residual-based fallback to zero; --guess '' skips it), the Newton
right-hand side and the solve to 1e-8 relative residual (inf-norm of the
FP64 residual, tol_abs = 0).  Fast path: FGMRES preconditioned by one
V(1,1)-cycle, both in FP32, inside FP64 iterative refinement, with a direct
solve on a 5^3-node bottom level.  The plain FP64 comparison is the reference's
algorithm on the GPU: MLMG iterations that are F-cycles (the reference sets
max_fmg_iter = 100000000) with V(2,2) damped-Jacobi smoothing and the
BiCGStab bottom, everything FP64, from zero.  `value` is seconds per solve (lower is
better); `e2e` is the same solve through the C ABI with host buffers
(stiffness and right-hand side copied in, displacement copied out, inside
the timed region).

--impl reference times the reference's CPU path restated in oracle/ (the
reference itself needs AMReX and cannot be built) on all host cores.
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

# FP64 multigrid iterations the reference algorithm needs to reach 1e-8 on
# each workload: F-cycles, since Linear::PrepareMLMG sets max_fmg_iter to
# 100000000 (the oracle and the GPU FP64 path iterate identically); used to
# scale the CPU sample to a whole solve when the run has no plain FP64 solve
# of its own to count them.
FP64_CYCLES = {"c1": 18, "c2": 50, "c3": 16}

# bytes each kernel family must move per fine-level node (each array once)
BYTES_PER_NODE = {
    "jacobi_f32": {2: 56, 21: 132},
    "jacobi_f64": {2: 112, 21: 264},
    "residual_f64": {2: 88, 21: 240},
    "residual_f32": {2: 44, 21: 120},
    "fapply_f64": {2: 64, 21: 216},
    "fapply_f32": {2: 32, 21: 108},
}
FAMILY = {"fapply_f64": 0, "jacobi_f64": 1, "residual_f64": 2, "fapply_f32": 3, "jacobi_f32": 4, "residual_f32": 5,
          "restrict": 6, "prolong": 7, "bottom": 8}
# dram__bytes_read.sum + dram__bytes_write.sum of one fine-level Jacobi
# sweep from 129^3 captures: the interior sweep per node (284.7 MB + 20.3 MB
# over 2,146,689 nodes, profiles/k_zmarch_tma_jacobi_mm_129.md; it streams
# every array once, so it scales with the nodes) and the boundary-face
# kernel per boundary node (28.1 MB + 0.1 MB over 98,306 boundary nodes,
# profiles/k_zt_faces_mm_129.md); (per node, per boundary node).  The
# isotropic sweep's interior from a 257^3 capture (757.9 MB + 183.8 MB over
# 16,974,593 nodes, profiles/k_zmarch_tma_jacobi_iso_257.md); its faces were
# not captured (None: the figure is the interior sweep's alone)
TRAFFIC_PER_NODE = {("jacobi_f32", 21): ((284.697344e6 + 20.251904e6) / 2146689, (28.08704e6 + 0.097536e6) / 98306),
                    ("jacobi_f32", 2): ((757.910784e6 + 183.846656e6) / 16974593, None)}


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
    p.add_argument("--no-plain", action="store_true", help="skip the plain FP64 comparison solve")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--n", type=int, default=0, help="override the grid size (nodes per axis)")
    p.add_argument("--guess", default=os.path.join(ROOT, "alamo_gb300", "weights", "unet65.npy"),
                   help="U-Net weights of the learned initial guess ('' = solve from zero)")
    return p.parse_args()


def workload(cfg, n_override=0):
    """(name, n, C, F0, bc, dx, sym)"""
    from alamo_gb300 import bc as B
    from alamo_gb300 import synth
    if cfg == "c1":
        n = n_override or 33
        C, F0, dx = synth.inclusion_iso(n)
        return ("c1: 33^3 isotropic inclusion r=0.25 contrast 10, eigenstrain 0.01 I, zero-displacement faces",
                n, C, F0, B.Constant(), dx)
    if cfg == "c2":
        n = n_override or 257
        C, dx = synth.voronoi_cubic(n, 64, seed=1)
        return ("c2: %d^3 cubic Voronoi polycrystal, 64 grains, C11/C12/C44=1.68/1.21/0.75, "
                "uniaxial_stress_clamp u_x=0.01" % n, n, C, None, B.TensionTest("uniaxial_stress_clamp", disp=0.01),
                dx)
    n = n_override or 513
    C, F0, dx, placed = synth.spheres_diffuse(n, 200, seed=3)
    return ("c3: %d^3 isotropic two-phase, %d spheres r in [0.02,0.06] with a diffuse interface of 4 node spacings, "
            "contrast 10, eigenstrain U[0,0.02]" % (n, placed), n, C, F0, B.Constant(), dx)


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


# --------------------------------------------------------------- CPU sample
def cpu_sample(cfg, n_override, C, F0, bc, dx, cycles):
    """Oracle (the reference's CPU path restated) on all host threads: time
    the right-hand side, the hierarchy set-up and six fixed F-cycles (the
    reference's MLMG iteration), and scale the per-cycle time to the FP64
    cycle count of the whole solve."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    n = C.shape[0]
    bt, bv = bc.tables()
    u = np.zeros((3, n, n, n))
    t0 = time.perf_counter()
    b = O.bc_init(u, bt, bv)
    rhs = O.build_rhs(C, F0, bt, u, b, dx)
    t_rhs = time.perf_counter() - t0
    sample_cycles = 6
    x, rep, _ = O.solve(C, bt, rhs, dx, fixed_iter=sample_cycles)
    per_cycle = (rep.seconds - rep.setup_seconds) / sample_cycles
    setup = rep.setup_seconds + t_rhs
    est = setup + per_cycle * cycles
    # one V-cycle (max_fmg_iter 0) for comparison with the GPU's V-cycles
    _, repv, _ = O.solve(C, bt, rhs, dx, fixed_iter=1, max_fmg_iter=0)
    v_cycle = repv.seconds - repv.setup_seconds
    # one operator application at full size, median of ten
    fap = []
    for _ in range(10):
        t3 = time.perf_counter()
        O.fapply(C, bt, x, dx)
        fap.append(time.perf_counter() - t3)
    return {"value": est, "unit": "s", "cores": threads, "kind": "port",
            "sample": "oracle (C++ restatement of the reference CPU path, OpenMP) on %d host threads: RHS build + "
                      "set-up + %d fixed FP64 F-cycles at the full %d^3 size; solve time = set-up + "
                      "per-cycle time x %d cycles (the FP64 F-cycle count of this input to 1e-8)"
                      % (threads, sample_cycles, n, cycles),
            "per_cycle_s": per_cycle, "v_cycle_s": v_cycle, "setup_s": setup, "fapply_s": float(np.median(fap)),
            "fapply_node_updates_per_s": float(n ** 3 / np.median(fap)), "sample_wall_s": time.perf_counter() - t0}


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


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    name, n, C, F0, bc, dx = workload(args.config, args.n)
    cycles = FP64_CYCLES[args.config]
    vals = []
    for s in range(args.warmup + args.steps):
        r = cpu_sample(args.config, args.n, C, F0, bc, dx, cycles)
        if s >= args.warmup:
            vals.append(r["value"])
        if s == 0 and r["sample_wall_s"] * (args.warmup + args.steps) > 240:
            # keep the whole run within minutes: the remaining steps reuse this sample
            vals = [r["value"]] * args.steps
            break
    v = float(np.mean(vals))
    r["value"] = v
    guess = bool(args.guess) and os.path.exists(args.guess)
    line = {"impl": "reference", "metric": metric_name(n, guess),
            "value": v, "unit": "s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": v * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "config": {"workload": name, "nodes": n ** 3},
            "cpu_baseline": r, "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# --------------------------------------------------------------- GPU arm
def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
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
    nlev = 1
    m = n
    while (m - 1) % 2 == 0 and (m - 1) // 2 >= 2:
        m = (m - 1) // 2 + 1
        nlev += 1
    # the mixed FGMRES path runs V(1,1) as its preconditioner (fewer fine sweeps
    # per Krylov step; 52 steps of V(1,1) beat 36 of V(2,2) at 257^3); the
    # FP64 arms keep the reference's V(2,2)
    pre, post = (args.pre, args.post) if prec else (2, 2)
    opts = A.default_opts(precision=prec, inner_cycles=args.inner, solver=args.solver, inner_tol=args.inner_tol,
                          krylov_dim=args.krylov, bottom_solver="direct", max_coarsening_level=max(nlev - 2, 0),
                          pre_smooth=pre, post_smooth=post)
    op = A.Elastic(n, dx, sym, opts)
    stream = torch.cuda.Stream()
    _lib.check(_lib.lib().agb_elastic_set_stream(op.h, __import__("ctypes").c_void_p(stream.cuda_stream)))
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
            r = newton.solve_guess(net, P(u_dev.data_ptr()), P(b_dev.data_ptr()), F0arg, tol_rel=1e-8, tol_abs=0.0)
            guesses.append({"used": r["guess_used"]})
            reports.append(r)
        else:
            with torch.cuda.stream(stream):
                u_dev.zero_()
            reports.append(newton.solve(P(u_dev.data_ptr()), P(b_dev.data_ptr()), F0arg, tol_rel=1e-8,
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
    op.profile(False)
    sec = reduce_max(sec, dist, dev)

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
        traf = TRAFFIC_PER_NODE.get((dom, nc))
        nb = N - (n - 2) ** 3  # boundary nodes
        roof = {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"],
                "traffic": (traf[0] * N + (traf[1] * nb if traf[1] is not None else 0.0)) if traf else None,
                "traffic_covers": (("interior sweep and boundary faces" if traf[1] is not None else
                                    "interior sweep only") if traf else None),
                "peak_source": peak_kind, "launches": cnt, "avg_launch_ms": ms / cnt,
                "alg_bytes_per_launch": alg_bytes, "share_of_step": ms / 1e3 / (sec * args.steps)}
    kernels = {k: {"launches": v[0], "ms": v[1]} for k, v in fam.items() if v[0] > 0}

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
                newton.solve_guess(net, u_h.numpy(), b_h.numpy(), F0x, tol_rel=1e-8, tol_abs=0.0)
            else:
                u_h.zero_()
                newton.solve(u_h.numpy(), b_h.numpy(), F0x, tol_rel=1e-8, tol_abs=0.0)

        step_host()
        barrier()
        t0 = time.perf_counter()
        e0.record(stream)
        for _ in range(args.steps):
            step_host()
        e1.record(stream)
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

    # plain FP64 solve of the same input with the reference's solver
    # settings: MLMG iterations that are all F-cycles (max_fmg_iter
    # 100000000), V(2,2) inside them, BiCGStab bottom
    plain = None
    if not args.no_plain:
        op.SetOpts(A.default_opts(precision=0))
        ts = []
        try:
            for _ in range(2):
                op.SetModel(P(C_dev.data_ptr()))
                with torch.cuda.stream(stream):
                    u_dev.zero_()
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                r = newton.solve(P(u_dev.data_ptr()), P(b_dev.data_ptr()), F0arg, tol_rel=1e-8, tol_abs=0.0)
                torch.cuda.synchronize()
                ts.append(time.perf_counter() - t0)
            plain = {"seconds": min(ts), "cycles": r["iters"], "cycle": "F (max_fmg_iter 100000000)",
                     "final_rel_resnorm": r["final_resnorm"] / r["rhsnorm0"]}
            u64 = u_dev.clone()
        except A.AgbError as e:
            plain = {"error": str(e)}
        op.SetOpts(opts)
        if "error" not in plain:
            step()
            diff = (u_dev - u64).abs().max().item() / u64.abs().max().item()
            plain["mixed_vs_fp64_solution_rel_inf"] = diff

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
        _lib.check(_lib.lib().agb_elastic_fapply_f32(op.h, 0, __import__("ctypes").c_void_p(x32.data_ptr()),
                                                     __import__("ctypes").c_void_p(f32.data_ptr()), 1))
    fap = {}
    for key, famid in [("fp64", FAMILY["fapply_f64"]), ("fp32", FAMILY["fapply_f32"])]:
        cnt, ms = op.profile_get(famid)
        per = ms / cnt / 1e3
        bpn = BYTES_PER_NODE["fapply_f64" if key == "fp64" else "fapply_f32"][nc]
        fap[key] = {"node_updates_per_s": N / per, "hbm_gbs": bpn * N / per / 1e9, "ms": per * 1e3,
                    "frac_of_hbm_peak": bpn * N / per / 1e9 / peaks["hbm_gbs"]}
    op.profile(False)

    cpu = None
    if rank == 0 and not args.no_cpu:
        cycles = plain["cycles"] if plain and "cycles" in plain else FP64_CYCLES[args.config]
        cpu = cpu_sample(args.config, args.n, C, F0, bc, dx, cycles)

    rep = reports[-1] if reports else {}
    line = {
        "metric": metric_name(n, net is not None),
        "value": sec, "unit": "s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": sec * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32-cycle/f64-refinement" if prec else "f64", "data": "synthetic",
        "config": {"workload": name, "nodes": N, "precision": args.precision, "solver": args.solver,
                   "inner_tol": args.inner_tol, "krylov_dim": args.krylov, "bottom": "direct 5^3",
                   "smoothing": "V(%d,%d), 2 damped-Jacobi sweeps per Fsmooth call" % (pre, post),
                   "parallelism": "replicas" if world > 1 else "single-gpu",
                   "l2": "inputs larger than L2 (%.1f GB of stiffness)" % (C.nbytes / 1e9)},
        "e2e": e2e, "gpu_launches": launches, "roofline": roof, "cpu_baseline": cpu, "clocks": ck,
        "guess": ({"weights": os.path.relpath(args.guess, ROOT), "network_grid": 65,
                   "used_fraction": float(np.mean([g["used"] for g in guesses])) if guesses else None}
                  if net is not None else None),
        "solve": {"v_cycles": rep.get("iters"), "fp64_residuals": rep.get("fp64_residuals"),
                  "final_rel_resnorm_l2": (rep.get("final_resnorm_l2", 0) / rep["rhsnorm_l2"]) if rep else None,
                  "final_rel_resnorm": (rep.get("final_resnorm", 0) / rep["rhsnorm0"]) if rep else None,
                  "levels": rep.get("nlevels")},
        "plain_fp64": plain,
        "speedup_vs_plain_fp64": (plain["seconds"] / sec) if plain and "seconds" in plain else None,
        "fapply": fap, "kernels_in_timed_region": kernels,
    }
    if rank == 0:
        print(json.dumps(line))
    op.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
