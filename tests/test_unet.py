"""Learned initial guess: the tensor-core convolution against PyTorch's FP32
conv3d, the whole U-Net forward and one training step against an FP32
PyTorch replica that rounds to BF16 where the kernels store BF16, and the
guess-then-fallback path of the solver against the oracle's transfer
operators."""
import ctypes

import numpy as np
import pytest

import problems as P

torch = pytest.importorskip("torch")
# FP32 references: no TF32 inside PyTorch's convolutions and matmuls
torch.backends.cudnn.allow_tf32 = False
torch.backends.cuda.matmul.allow_tf32 = False


def _bf16(t):
    return t.to(torch.bfloat16).to(torch.float32)


def _conv_ref(x, w, b, relu):
    """x (1, Cin, nz, ny, nx) FP32, w (Cout, Cin, 27) FP32 (tap = 9 (dz+1) +
    3 (dy+1) + (dx+1)) -> FP32 reference of one 3x3x3 convolution."""
    cout, cin = w.shape[:2]
    y = torch.nn.functional.conv3d(x, w.reshape(cout, cin, 3, 3, 3), b, padding=1)
    return torch.relu(y) if relu else y


@pytest.mark.gpu
@pytest.mark.parametrize("cin,cout,dims", [(16, 16, (13, 21, 9)), (32, 64, (8, 16, 3)), (48, 16, (17, 17, 17)),
                                           (192, 64, (9, 9, 9)), (16, 192, (11, 5, 7)), (96, 32, (33, 9, 5)),
                                           (64, 128, (9, 9, 9)), (128, 48, (5, 6, 7))])
def test_conv3_matches_torch(agb, cin, cout, dims):
    dev = torch.device("cuda", 0)
    nx, ny, nz = dims
    g = torch.Generator().manual_seed(cin * 1000 + cout)
    X = _bf16(torch.randn(nz, ny, nx, cin, generator=g)).to(dev)
    W = _bf16(torch.randn(cout, cin, 27, generator=g) * 0.1).to(dev)
    bias = torch.randn(cout, generator=g).to(dev)
    Xb = X.to(torch.bfloat16).contiguous()
    for relu in (0, 1):
        Yf = torch.empty(nz, ny, nx, cout, device=dev)
        st = agb.lib().agb_conv3_bf16(ctypes.c_void_p(Xb.data_ptr()), cin, ctypes.c_void_p(W.data_ptr()),
                                      ctypes.c_void_p(bias.data_ptr()), cout, nx, ny, nz, relu, None,
                                      ctypes.c_void_p(Yf.data_ptr()), None)
        assert st == 0, agb.last_error()
        ref = _conv_ref(X.permute(3, 0, 1, 2)[None], W, bias, relu)[0].permute(1, 2, 3, 0)
        err = (Yf - ref).abs().max().item()
        assert err <= 1e-4 * ref.abs().max().item(), err
    # BF16 output: rounding only
    Yb = torch.empty(nz, ny, nx, cout, device=dev, dtype=torch.bfloat16)
    st = agb.lib().agb_conv3_bf16(ctypes.c_void_p(Xb.data_ptr()), cin, ctypes.c_void_p(W.data_ptr()), None, cout,
                                  nx, ny, nz, 0, ctypes.c_void_p(Yb.data_ptr()), None, None)
    assert st == 0, agb.last_error()
    ref = _conv_ref(X.permute(3, 0, 1, 2)[None], W, None, 0)[0].permute(1, 2, 3, 0)
    assert (Yb.float() - ref).abs().max().item() <= 8e-3 * ref.abs().max().item()


@pytest.mark.gpu
@pytest.mark.parametrize("cin,cinw,cout,dims", [(16, 16, 16, (13, 21, 9)), (32, 32, 64, (8, 16, 3)),
                                                (48, 48, 16, (17, 17, 17)), (192, 192, 64, (9, 9, 9)),
                                                (16, 3, 16, (11, 5, 7)), (96, 96, 32, (33, 9, 5)),
                                                (64, 64, 128, (9, 9, 9)), (128, 128, 48, (5, 6, 7)),
                                                (16, 16, 192, (7, 7, 7))])
def test_conv3_weight_gradient_matches_torch(agb, cin, cinw, cout, dims):
    """The convolution's weight and bias gradients, tensor-core kernel
    (training) and CUDA-core kernel, against PyTorch's conv3d_weight in FP32:
    the tensor-core kernel takes dY rounded to BF16, so its reference does
    too; both accumulate into dW / db (here from zero)."""
    dev = torch.device("cuda", 0)
    nx, ny, nz = dims
    g = torch.Generator().manual_seed(cin * 7 + cout)
    X = _bf16(torch.randn(nz, ny, nx, cin, generator=g))
    X[..., cinw:] = 0.0
    X = X.to(dev)
    dY = torch.randn(nz, ny, nx, cout, generator=g).to(dev)
    Xb = X.to(torch.bfloat16).contiguous()
    xin = X[..., :cinw].permute(3, 0, 1, 2)[None]
    for tc in (1, 0):
        dW = torch.zeros(cout, cinw, 27, device=dev)
        db = torch.zeros(cout, device=dev)
        st = agb.lib().agb_conv3_wgrad_bf16(ctypes.c_void_p(Xb.data_ptr()), cin, cinw, ctypes.c_void_p(dY.data_ptr()),
                                            cout, nx, ny, nz, ctypes.c_void_p(dW.data_ptr()),
                                            ctypes.c_void_p(db.data_ptr()), tc, None)
        assert st == 0, agb.last_error()
        go = (_bf16(dY) if tc else dY).permute(3, 0, 1, 2)[None]
        ref = torch.nn.grad.conv3d_weight(xin, (cout, cinw, 3, 3, 3), go, padding=1).reshape(cout, cinw, 27)
        assert (dW - ref).abs().max().item() <= 1e-4 * ref.abs().max().item()
        assert (db - dY.sum(dim=(0, 1, 2))).abs().max().item() <= 1e-4 * dY.abs().sum(dim=(0, 1, 2)).max().item()


def test_conv3_rejects_bad_shapes(agb):
    null = ctypes.c_void_p(16)
    assert agb.lib().agb_conv3_bf16(null, 12, null, None, 16, 4, 4, 4, 0, null, None, None) != 0
    assert agb.lib().agb_conv3_bf16(null, 16, null, None, 16, 4, 4, 4, 0, null, null, None) != 0


# ------------------------------------------------------- torch replica
SPEC = [(3, 16, 0), (16, 16, 0), (16, 32, 1), (32, 32, 1), (32, 64, 2), (64, 64, 2), (64, 128, 3), (128, 128, 3),
        (192, 64, 2), (64, 64, 2), (96, 32, 1), (32, 32, 1), (48, 16, 0), (16, 16, 0)]


def _unflatten(p):
    out, off = [], 0
    for cin, cout, _ in SPEC:
        w = p[off:off + cout * cin * 27].reshape(cout, cin, 27)
        off += cout * cin * 27
        b = p[off:off + cout]
        off += cout
        out.append((w, b))
    wh = p[off:off + 48].reshape(3, 16)
    bh = p[off + 48:off + 51]
    return out, wh, bh


def _down(x):
    c = x.shape[1]
    k1 = torch.tensor([0.25, 0.5, 0.25], dtype=x.dtype, device=x.device)
    k = (k1[:, None, None] * k1[None, :, None] * k1[None, None, :]).expand(c, 1, 3, 3, 3).contiguous()
    return torch.nn.functional.conv3d(x, k, stride=2, padding=1, groups=c)


def _up(x):
    c = x.shape[1]
    k1 = torch.tensor([0.5, 1.0, 0.5], dtype=x.dtype, device=x.device)
    k = (k1[:, None, None] * k1[None, :, None] * k1[None, None, :]).expand(c, 1, 3, 3, 3).contiguous()
    return torch.nn.functional.conv_transpose3d(x, k, stride=2, padding=1, groups=c)


def _replica(params, feats):
    """FP32 forward with BF16 rounding where the kernels store BF16."""
    convs, wh, bh = _unflatten(params)
    lam, mu, f0 = feats
    x = torch.zeros(1, 16, *lam.shape, device=lam.device)
    il = 1.0 / np.log(20.0)
    x[0, 0] = torch.log(torch.clamp(lam.float(), min=1e-6)) * il
    x[0, 1] = torch.log(torch.clamp(mu.float(), min=1e-6)) * il
    x[0, 2] = f0.float() * 50.0
    x = _bf16(x)

    def conv(i, h):
        w, b = convs[i]
        cin = w.shape[1]
        return _bf16(_conv_ref(h[:, :cin] if h.shape[1] != cin else h, _bf16(w), b, 1))

    a = [None] * 14
    a[0] = conv(0, x[:, :3])
    a[1] = conv(1, a[0])
    a[2] = conv(2, _bf16(_down(a[1])))
    a[3] = conv(3, a[2])
    a[4] = conv(4, _bf16(_down(a[3])))
    a[5] = conv(5, a[4])
    a[6] = conv(6, _bf16(_down(a[5])))
    a[7] = conv(7, a[6])
    a[8] = conv(8, torch.cat([_bf16(_up(a[7])), a[5]], 1))
    a[9] = conv(9, a[8])
    a[10] = conv(10, torch.cat([_bf16(_up(a[9])), a[3]], 1))
    a[11] = conv(11, a[10])
    a[12] = conv(12, torch.cat([_bf16(_up(a[11])), a[1]], 1))
    a[13] = conv(13, a[12])
    u = torch.einsum("oc,bcxyz->boxyz", wh, a[13]) + bh[None, :, None, None, None]
    return u[0] * 1e-3


def _sample(n, seed):
    from alamo_gb300 import learn
    rng = np.random.default_rng(seed)
    C, F0, dx = learn.inclusion_medium(n, rng)
    return learn.features_of(C, F0), C, F0, dx


@pytest.mark.gpu
def test_unet_forward_matches_replica(agb):
    from alamo_gb300 import learn
    dev = torch.device("cuda", 0)
    with learn.UNet(17, seed=3) as net:
        feats, _, _, _ = _sample(17, 5)
        u = net.predict(feats)
        p = torch.from_numpy(net.get_params()).to(dev)
        ref = _replica(p, torch.from_numpy(feats).to(dev)).double().cpu().numpy()
    err = np.linalg.norm(u - ref) / np.linalg.norm(ref)
    assert err <= 5e-3, err


@pytest.mark.gpu
def test_unet_train_step_follows_autograd(agb):
    """One Adam step moves every weight by -lr sign(g) (first step); the signs
    must agree with PyTorch autograd of the replica's loss on the entries
    whose gradient is not negligible."""
    from alamo_gb300 import learn
    dev = torch.device("cuda", 0)
    with learn.UNet(17, seed=4) as net:
        feats, C, F0, dx = _sample(17, 6)
        target = np.random.default_rng(7).standard_normal((3, 17, 17, 17)) * 1e-3
        p0 = net.get_params()
        lr = 1e-4
        loss = net.train_step(feats, target, lr)
        dp = net.get_params() - p0
    p = torch.from_numpy(p0).to(dev).requires_grad_(True)
    u = _replica(p, torch.from_numpy(feats).to(dev))
    t = torch.from_numpy(target).to(dev).float()
    ref_loss = (((u - t) / 1e-3) ** 2).mean()
    ref_loss.backward()
    assert abs(loss - ref_loss.item()) <= 1e-2 * ref_loss.item()
    g = p.grad.cpu().numpy()
    big = np.abs(g) > np.quantile(np.abs(g), 0.5)
    agree = np.mean(np.sign(dp[big]) == -np.sign(g[big]))
    assert agree >= 0.97, agree
    # first Adam step: |step| = lr |g| / (|g| + 1e-8)
    expect = lr * np.abs(g[big]) / (np.abs(g[big]) + 1e-8)
    assert abs(np.median(np.abs(dp[big]) / expect) - 1.0) <= 1e-2
    assert np.abs(dp).max() <= lr * (1 + 1e-3)


@pytest.mark.gpu
def test_learned_guess_transfers_and_fallback(agb, oracle):
    """The guess is the prediction on the network's level (features restricted
    from the fine grid with the multigrid weights) prolongated back; when the
    Newton right-hand side at the guess, restricted to the network's level,
    exceeds that at zero the guess is dropped."""
    from alamo_gb300 import learn
    n = 33
    C, F0, bc, dx = P.c1(n)
    with learn.UNet(17, seed=5) as net, agb.Elastic(n, dx, "isotropic") as op:
        op.SetModel(np.ascontiguousarray(C))
        op.SetBC(bc)
        b = op.bc_init()
        u, rhs, (rg, r0), used = learn.learned_guess(op, net, b, F0)
        f = learn.features_of(C, F0)
        pred = net.predict(oracle.restrict(f))
        expect = oracle.prolong_add(pred, np.zeros((3, n, n, n)))
        bt, _ = bc.tables()
        rhs0 = oracle.build_rhs(C, F0, bt, np.zeros_like(expect), b, dx)
        assert np.abs(rhs - rhs0).max() <= 1e-12 * np.abs(rhs0).max()
        res_g = oracle.restrict(rhs0 - oracle.fapply(C, bt, expect, dx))
        assert abs(rg - np.linalg.norm(res_g)) <= 1e-10 * np.linalg.norm(res_g)
        assert abs(r0 - np.linalg.norm(oracle.restrict(rhs0))) <= 1e-10 * np.linalg.norm(oracle.restrict(rhs0))
        if used:
            assert rg <= r0
            assert np.abs(u - expect).max() <= 1e-12 * max(np.abs(expect).max(), 1e-300)
        else:
            assert rg > r0
            assert not np.any(u)
        # the linear solve from the guess reaches the Newton-from-zero answer
        op.SetOpts(agb.default_opts(solver="fgmres"))
        x = u.copy()
        agb.Linear(op).solve(x, rhs, 1e-10, 0.0)
        u0 = np.zeros((3, n, n, n))
        agb.Newton(op).solve(u0, b, F0, tol_rel=1e-10, tol_abs=0.0)
        assert np.abs(x - u0).max() <= 1e-5 * np.abs(u0).max()


@pytest.mark.gpu
def test_learned_guess_rhs_without_eigenstrain(agb, oracle):
    """Without F0 the Newton right-hand side at zero displacement is b
    itself (every subtracted row is an exact zero); the guess path takes
    that shortcut and must agree with the oracle's full RHS bit for bit."""
    from alamo_gb300 import learn
    n = 33
    C, F0, bc, dx = P.voronoi_clamp(n)
    with learn.UNet(17, seed=6) as net, agb.Elastic(n, dx, "majorminor") as op:
        op.SetModel(np.ascontiguousarray(C))
        op.SetBC(bc)
        b = op.bc_init()
        u, rhs, _, used = learn.learned_guess(op, net, b, None)
    bt, _ = bc.tables()
    ref = oracle.build_rhs(C, None, bt, np.zeros((3, n, n, n)), b, dx)
    assert np.array_equal(rhs, ref)
    assert np.array_equal(rhs, b)


@pytest.mark.gpu
@pytest.mark.parametrize("where", ["host", "device"])
def test_newton_solve_guess_one_call(agb, where):
    """agb_newton_solve_guess does agb_elastic_learned_guess followed by
    agb_linear_solve in one call.  A kept guess starts the single call's
    mixed refinement from the FP32 residual of the fallback test (the two-call
    form computes an FP64 one), so the two agree to the solve tolerance; a
    dropped guess gives identical work."""
    from alamo_gb300 import learn
    n = 33
    C, F0, bc, dx = P.c1(n)
    opts = agb.default_opts(precision="mixed", solver="fgmres", bottom_solver="direct", max_coarsening_level=2)
    with learn.UNet(17, seed=8) as net, agb.Elastic(n, dx, "isotropic", opts) as op:
        op.SetModel(np.ascontiguousarray(C))
        op.SetBC(bc)
        b = op.bc_init()
        u0, rhs, _, used0 = learn.learned_guess(op, net, b, F0)
        r0 = agb.Linear(op).solve(u0, rhs, 1e-10, 0.0)
        if where == "host":
            u1 = np.full((3, n, n, n), np.nan)
            r1 = agb.Newton(op).solve_guess(net, u1, b, F0, tol_rel=1e-10, tol_abs=0.0)
        else:
            dev = torch.device("cuda", 0)
            ut = torch.full((3, n, n, n), float("nan"), dtype=torch.float64, device=dev)
            bt = torch.from_numpy(b).to(dev)
            Ft = torch.from_numpy(np.ascontiguousarray(F0)).to(dev)
            P_ = agb.DevicePtr
            r1 = agb.Newton(op).solve_guess(net, P_(ut.data_ptr()), P_(bt.data_ptr()), (P_(Ft.data_ptr()), 1),
                                            tol_rel=1e-10, tol_abs=0.0)
            u1 = ut.cpu().numpy()
    assert r1["guess_used"] == used0
    if used0:
        assert abs(r1["iters"] - r0["iters"]) <= 2
        assert np.abs(u1 - u0).max() <= 1e-7 * np.abs(u0).max()
    else:
        assert r1["iters"] == r0["iters"]
        assert np.array_equal(u1, u0)


@pytest.mark.gpu
def test_trained_guess_solve_matches_fp64(agb):
    """The trained 65^3 network on a training-distribution medium at 65^3:
    the single-call mixed solve from its guess (kept: the refinement starts
    from the FP32 residual; dropped: from zero) reaches the plain FP64
    solve's displacement."""
    import os
    from alamo_gb300 import learn
    w = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "alamo_gb300", "weights",
                     "unet65.npy")
    if not os.path.exists(w):
        pytest.skip("trained weights not present")
    n = 65
    C, F0, dx = learn.inclusion_medium(n, np.random.default_rng(2024))
    bc = agb.bc.Constant()
    opts = agb.default_opts(precision="mixed", solver="fgmres", bottom_solver="direct", max_coarsening_level=4,
                            pre_smooth=1, post_smooth=1)
    with learn.UNet(n) as net, agb.Elastic(n, dx, "isotropic", opts) as op:
        net.load(w)
        op.SetModel(np.ascontiguousarray(C))
        op.SetBC(bc)
        b = op.bc_init()
        u = np.zeros((3, n, n, n))
        r = agb.Newton(op).solve_guess(net, u, b, F0, tol_rel=1e-10, tol_abs=0.0)
        op.SetOpts(agb.default_opts(precision="fp64"))
        u64 = np.zeros((3, n, n, n))
        agb.Newton(op).solve(u64, b, F0, tol_rel=1e-10, tol_abs=0.0)
    assert r["status"] == 0
    assert np.abs(u - u64).max() <= 1e-7 * np.abs(u64).max()
    assert r["fp64_residuals"] >= 1
