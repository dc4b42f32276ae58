"""The allocation-free residual entry point, for callers that cannot call
cudaMalloc (a host code whose memory arena took the whole device, a plugin
inside one, a step loop that must not synchronise the device through
cudaMalloc/cudaFree): it must give what the ordinary residual entry point
and the oracle give, call after call, while using only the caller's arrays
and the library's fixed device scratch.

This file is collected last on purpose, so a run that stops at the first
failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

import problems as P


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_rejects_oversized_grid(agb):
    """Beyond the fixed scratch the call refuses, before touching the GPU."""
    from alamo_gb300 import _lib
    dx = (ctypes.c_double * 3)(1.0, 1.0, 1.0)
    bt = (ctypes.c_int * 78)()
    null = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    st = agb.lib().agb_residual_norms_noalloc(513, 513, 513, dx, 0, null, bt, null, null, null,
                                              (ctypes.c_double * 2)(), None)
    assert st == _lib.AGB_LIMIT
    assert "AGB_NOALLOC_MAX_BLOCKS" in _lib.last_error()


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["c1", "voronoi"])
def test_noalloc_matches_residual_entry_point(agb, oracle, case):
    torch = pytest.importorskip("torch")
    from alamo_gb300 import _lib
    if case == "c1":
        C, F0, bc, dx = P.c1(33)
    else:
        C, F0, bc, dx = P.voronoi_clamp(33)
    n = C.shape[0]
    sym = 0 if C.shape[-1] == 2 else 1
    bt, _ = bc.tables()
    dxa = np.ascontiguousarray(np.broadcast_to(np.asarray(dx, dtype=np.float64), (3,)))
    dev = torch.device("cuda", 0)
    C_soa = torch.from_numpy(np.ascontiguousarray(np.moveaxis(C, -1, 0))).to(dev)
    op = agb.Elastic(n, dx, "isotropic" if sym == 0 else "majorminor")
    op.SetModel(np.ascontiguousarray(C))
    op.SetBC(bc)
    for call in range(2):
        x = torch.from_numpy(P.random_field((3, n, n, n), 100 + call)).to(dev)
        b = torch.from_numpy(P.random_field((3, n, n, n), 200 + call)).to(dev)
        r = torch.full_like(x, float("nan"))
        norms = (ctypes.c_double * 2)()
        torch.cuda.synchronize()
        st = agb.lib().agb_residual_norms_noalloc(n, n, n, dxa.ctypes.data_as(ctypes.c_void_p), sym, _ptr(C_soa),
                                                  bt.ctypes.data_as(ctypes.c_void_p), _ptr(x), _ptr(b), _ptr(r),
                                                  norms, None)
        assert st == _lib.AGB_OK, _lib.last_error()
        r_ref, (inf_ref, l2_ref) = op.residual(x.cpu().numpy(), b.cpu().numpy())
        rr = r.cpu().numpy()
        assert np.abs(rr - r_ref).max() <= 1e-12 * np.abs(r_ref).max()
        assert abs(norms[0] - inf_ref) <= 1e-12 * inf_ref
        assert abs(norms[1] - l2_ref) <= 1e-12 * l2_ref
        # and the oracle's residual (Operator.cpp:635-657) on the same inputs
        r_orc, _ = oracle.residual(C, bt, x.cpu().numpy(), b.cpu().numpy(), dx)
        assert np.abs(rr - r_orc).max() <= 1e-12 * np.abs(r_orc).max()
        assert abs(norms[0] - np.abs(r_orc).max()) <= 1e-12 * np.abs(r_orc).max()
        assert abs(norms[1] - np.sqrt((r_orc ** 2).sum())) <= 1e-12 * np.sqrt((r_orc ** 2).sum())
    op.close()
