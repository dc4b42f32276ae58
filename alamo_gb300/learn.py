"""Learned initial guess for the elastic solve: the U-Net of the C ABI
(agb_unet_*, trained and run by hand-written tensor-core kernels), its
training-set generator and the guess-then-solve driver.

The network works on the node grid of one multigrid level (65^3 for the
trained model): inputs (lambda, mu, F0) are restricted from the fine grid to
that level, the predicted displacement is prolongated back, and the solver
starts from it unless the Newton right-hand side at the guess is larger than
at zero (the fallback).  The training set is plain-solver solutions of random
inclusion media (count 1-40, radius U[0.03, 0.15], contrast log-U[1, 20],
eigenstrain U[0, 0.02], zero-displacement faces), generated here on the GPU.
"""
import ctypes
import os

import numpy as np

from . import _lib as L
from . import bc as B
from . import synth
from .elastic import DevicePtr, Elastic, Newton, _arg, _same_where, default_opts


class UNet:
    """agb_unet: 4-level 3D U-Net (16/32/64/128) on an n^3 node grid."""

    def __init__(self, n=65, seed=1):
        self.n = int(n)
        h = ctypes.c_void_p()
        L.check(L.lib().agb_unet_create(ctypes.byref(h), self.n, ctypes.c_uint64(seed)))
        self.h = h

    def close(self):
        if self.h:
            L.lib().agb_unet_destroy(self.h)
            self.h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def num_params(self):
        c = ctypes.c_int64()
        L.check(L.lib().agb_unet_num_params(self.h, ctypes.byref(c)))
        return c.value

    def get_params(self):
        p = np.empty(self.num_params(), dtype=np.float32)
        L.check(L.lib().agb_unet_get_params(self.h, p.ctypes.data_as(ctypes.c_void_p)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != self.num_params():
            raise ValueError("parameter vector of %d values, the network has %d" % (p.size, self.num_params()))
        L.check(L.lib().agb_unet_set_params(self.h, p.ctypes.data_as(ctypes.c_void_p)))

    def save(self, path):
        np.save(path, self.get_params())

    def load(self, path):
        self.set_params(np.load(path))

    def train_step(self, features, target, lr):
        """One Adam step on one sample; features / target: (3, n, n, n)
        float64 arrays (lambda, mu, F0 / displacement) or DevicePtrs."""
        pf, wf = _arg(features)
        pt, wt = _arg(target)
        loss = ctypes.c_double()
        L.check(L.lib().agb_unet_train_step(self.h, pf, pt, ctypes.c_float(lr), ctypes.byref(loss),
                                            _same_where(wf, wt)))
        return loss.value

    def predict(self, features, u=None):
        if u is None:
            u = np.empty((3, self.n, self.n, self.n))
        pf, wf = _arg(features)
        pu, wu = _arg(u)
        L.check(L.lib().agb_unet_predict(self.h, pf, pu, _same_where(wf, wu)))
        return u


def learned_guess(op, net, b, F0=None, u=None, rhs=None):
    """agb_elastic_learned_guess: (u, rhs, (norm at guess, at zero), used);
    solve A u = rhs from u (agb_linear_solve) for the Newton step from 0."""
    n = op._vec_shape(0)
    if u is None:
        u = np.empty(n)
    if rhs is None and not isinstance(u, DevicePtr):
        rhs = np.empty(n)
    pb, wb = _arg(b)
    pu, wu = _arg(u)
    pr, wr = _arg(rhs)
    f0n, pF, wF = 0, None, None
    if F0 is not None:
        if isinstance(F0, tuple):
            F0, f0n = F0
        pF, wF = _arg(F0)
        if not f0n:
            f0n = 1 if F0.ndim == 3 else 9
    norms = (ctypes.c_double * 2)()
    used = ctypes.c_int()
    L.check(L.lib().agb_elastic_learned_guess(op.h, net.h, pb, pF, f0n, pu, pr, norms, ctypes.byref(used),
                                              _same_where(wb, wu, wF, wr if rhs is not None else None)))
    return u, rhs, (norms[0], norms[1]), bool(used.value)


def features_of(C, F0):
    """(3, n, n, n) lambda, mu, F0 of an isotropic medium (C: (n, n, n, 2))."""
    f = np.empty((3,) + C.shape[:3])
    f[0] = C[..., 0]
    f[1] = C[..., 1]
    f[2] = F0 if F0 is not None else 0.0
    return f


# diffuse-interface width of the inclusion media: 2 node spacings of the
# 65^3 training grid, the same physical width at every resolution
EPS_INCLUSION = 2.0 / 64.0


def inclusion_medium(n, rng):
    """One random inclusion medium of the training distribution: count
    U{1..40}, radius U[0.03, 0.15], contrast log-U[1, 20] (lambda = mu =
    contrast inside, 1 outside), eigenstrain U[0, 0.02] per inclusion, with
    the reference's diffuse interface (EPS_INCLUSION)."""
    count = int(rng.integers(1, 41))
    contrast = float(np.exp(rng.uniform(0.0, np.log(20.0))))
    seed = int(rng.integers(1, 2 ** 62))
    C, F0, dx, placed = synth.spheres_diffuse(n, count, seed=seed, rmin=0.03, rmax=0.15, eps=EPS_INCLUSION,
                                              contrast=contrast, smin=0.0, smax=0.02)
    return C, F0, dx


def solve_medium(C, F0, dx, tol=1e-8, opts=None):
    """Plain solve (mixed FGMRES) of a zero-displacement inclusion medium;
    returns (u, report)."""
    n = C.shape[0]
    nlev = _levels(n)
    o = opts or default_opts(precision="mixed", solver="fgmres", bottom_solver="direct",
                             max_coarsening_level=max(nlev - 2, 0))
    with Elastic(n, dx, "isotropic", o) as op:
        op.SetModel(np.ascontiguousarray(C))
        op.SetBC(B.Constant())
        u = np.zeros((3, n, n, n))
        b = op.bc_init()
        rep = Newton(op).solve(u, b, F0, tol_rel=tol, tol_abs=0.0, allow_not_converged=True)
    return u, rep


def _levels(n):
    lev, m = 1, n
    while (m - 1) % 2 == 0 and (m - 1) // 2 >= 2:
        m = (m - 1) // 2 + 1
        lev += 1
    return lev


def make_dataset(count, n=65, seed=1, device=None):
    """count training pairs (features, displacement) of the inclusion
    distribution, solved to 1e-8; returned as two (count, 3, n, n, n)
    float64 arrays (torch tensors on `device` when given)."""
    rng = np.random.default_rng(seed)
    feats, sols = [], []
    while len(feats) < count:
        C, F0, dx = inclusion_medium(n, rng)
        u, rep = solve_medium(C, F0, dx)
        if rep["status"] != 0:
            continue
        f = features_of(C, F0)
        if device is not None:
            import torch
            feats.append(torch.from_numpy(f).to(device))
            sols.append(torch.from_numpy(u).to(device))
        else:
            feats.append(f)
            sols.append(u)
    return feats, sols


def train(net, feats, sols, epochs=3, lr=1e-3, lr_end=1e-4, seed=0, log=None):
    """Adam over the samples in random order; learning rate decays
    geometrically from lr to lr_end.  Samples are numpy arrays or torch
    tensors on the GPU.  Returns the mean loss of each epoch."""
    rng = np.random.default_rng(seed)
    m = len(feats)
    total = epochs * m
    hist = []
    k = 0
    for ep in range(epochs):
        order = rng.permutation(m)
        acc = 0.0
        for i in order:
            rate = lr * (lr_end / lr) ** (k / max(total - 1, 1))
            f, s = feats[i], sols[i]
            if not isinstance(f, np.ndarray):
                f, s = DevicePtr(f.data_ptr()), DevicePtr(s.data_ptr())
            acc += net.train_step(f, s, rate)
            k += 1
        hist.append(acc / m)
        if log:
            log("epoch %d  mean loss %.4e" % (ep, hist[-1]))
    return hist


def guess_and_solve(n, C, F0, bc, dx, net=None, tol=1e-8, sym="isotropic"):
    """Mixed FGMRES Newton solve of one medium from the learned guess (net
    given, agb_newton_solve_guess: the guess, its fallback and the solve to
    the zero-start tolerance in one call) or from zero; returns (u, report,
    seconds, guess info).  Times the whole call on the host, guess included
    (GPU work is synchronous)."""
    import time
    nlev = _levels(n)
    o = default_opts(precision="mixed", solver="fgmres", bottom_solver="direct", max_coarsening_level=max(nlev - 2, 0))
    with Elastic(n, dx, sym, o) as op:
        op.SetModel(np.ascontiguousarray(C))
        op.SetBC(bc)
        b = op.bc_init()
        op.prepareForSolve()
        u = np.zeros((3, n, n, n))
        t0 = time.perf_counter()
        info = None
        if net is not None:
            rep = Newton(op).solve_guess(net, u, b, F0, tol_rel=tol, tol_abs=0.0, allow_not_converged=True)
            info = {"used": rep["guess_used"]}
        else:
            rep = Newton(op).solve(u, b, F0, tol_rel=tol, tol_abs=0.0, allow_not_converged=True)
        sec = time.perf_counter() - t0
    return u, rep, sec, info


# the trained 65^3 network shipped with the package
WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "unet65.npy")


def _main():
    import argparse
    import json
    import os
    import time
    ap = argparse.ArgumentParser(description="train / evaluate the learned initial guess")
    sub = ap.add_subparsers(dest="cmd", required=True)
    tr = sub.add_parser("train")
    tr.add_argument("--samples", type=int, default=2000)
    tr.add_argument("--epochs", type=int, default=3)
    tr.add_argument("--lr", type=float, default=1e-3)
    tr.add_argument("--seed", type=int, default=1)
    tr.add_argument("--out", required=True)
    pr = sub.add_parser("predict", help="time the network on one inclusion medium of its grid")
    pr.add_argument("--weights", default=WEIGHTS)
    pr.add_argument("--repeat", type=int, default=10)
    ev = sub.add_parser("evaluate")
    ev.add_argument("--weights", default=WEIGHTS)
    ev.add_argument("--n", type=int, default=129)
    ev.add_argument("--count", type=int, default=5)
    ev.add_argument("--seed", type=int, default=1000003)
    ev.add_argument("--voronoi", type=int, default=0, help="grains of an out-of-distribution polycrystal (config 5)")
    a = ap.parse_args()
    import torch
    dev = torch.device("cuda", 0)
    if a.cmd == "train":
        t0 = time.time()
        feats, sols = make_dataset(a.samples, 65, seed=a.seed, device=dev)
        t1 = time.time()
        with UNet(65, seed=a.seed) as net:
            hist = train(net, feats, sols, epochs=a.epochs, lr=a.lr, log=print)
            net.save(a.out)
        print(json.dumps({"samples": a.samples, "epochs": a.epochs, "dataset_s": t1 - t0, "train_s": time.time() - t1,
                          "loss_per_epoch": hist, "params": int(np.load(a.out).size)}))
        return
    net = UNet(65)
    net.load(a.weights)
    if a.cmd == "predict":
        C, F0, dx = inclusion_medium(65, np.random.default_rng(7))
        f = torch.from_numpy(features_of(C, F0)).to(dev)
        u = torch.empty_like(f)
        ts = []
        for _ in range(a.repeat):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            net.predict(DevicePtr(f.data_ptr()), DevicePtr(u.data_ptr()))
            ts.append(time.perf_counter() - t0)
        print(json.dumps({"grid": 65, "predict_ms_median": 1e3 * float(np.median(ts)),
                          "predict_ms_first": 1e3 * ts[0]}))
        net.close()
        return
    rng = np.random.default_rng(a.seed)
    rows = []
    for k in range(a.count):
        if a.voronoi:
            Cm, dx = synth.voronoi_cubic(a.n, a.voronoi, seed=int(rng.integers(1, 2 ** 31)))
            F0, bc, sym = None, B.TensionTest("uniaxial_stress_clamp", disp=0.01), "majorminor"
            C = Cm
        else:
            C, F0, dx = inclusion_medium(a.n, rng)
            bc, sym = B.Constant(), "isotropic"
        u0, r0, s0, _ = guess_and_solve(a.n, C, F0, bc, dx, None, sym=sym)
        u1, r1, s1, info = guess_and_solve(a.n, C, F0, bc, dx, net, sym=sym)
        err = float(np.abs(u1 - u0).max() / max(np.abs(u0).max(), 1e-300))
        rows.append({"zero": {"cycles": r0["iters"], "s": s0, "status": r0["status"]},
                     "guess": {"cycles": r1["iters"], "s": s1, "status": r1["status"], **info},
                     "solution_rel_diff": err})
        print(json.dumps(rows[-1]), flush=True)
    used = [r["guess"]["used"] for r in rows]
    print(json.dumps({"n": a.n, "count": a.count, "voronoi": a.voronoi, "fallback_rate": 1 - float(np.mean(used)),
                      "cycles_zero": float(np.mean([r["zero"]["cycles"] for r in rows])),
                      "cycles_guess": float(np.mean([r["guess"]["cycles"] for r in rows])),
                      "s_zero": float(np.mean([r["zero"]["s"] for r in rows])),
                      "s_guess": float(np.mean([r["guess"]["s"] for r in rows]))}))
    net.close()


if __name__ == "__main__":
    _main()
