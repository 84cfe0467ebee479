"""Learned sparse preconditioner on the GPU.

* kNN, the P build (frame, features, MLP, rotation) and the sparse P / P^T
  products against the NumPy oracle (oracle/precond_oracle.py);
* the training kernels' forward pass and gradients against the oracle
  (gradient check on a small batch);
* a network that outputs the identity makes the preconditioned sqrtMdotW
  reproduce the plain one;
* with the shipped trained network: fewer Lanczos iterations than plain on a
  clustered system, and the samples keep the covariance M
  (fluctuation-dissipation, KS per component).
"""
import ctypes
from pathlib import Path

import numpy as np
import pytest

from test_lanczos_gpu import _ks_fdt
from test_mdot_gpu import compute_M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def po():
    from oracle import precond_oracle
    return precond_oracle


def _lib():
    from libmobility_gb300 import _capi
    return _capi.load()


def _clustered(rng, n, phi=0.2, sigma=4.0):
    from libmobility_gb300.precond import random_system
    return random_system(rng, n, phi, True, sigma)


def _random_params(po, rng, scale=0.3):
    d = {k: rng.normal(0, scale, shp) for k, shp in po.SHAPES}
    d["xstd"] = np.abs(d["xstd"]) + 1.0
    d["ystd"] = np.abs(d["ystd"]) + 0.5
    return po.pack(d)


def test_knn_matches_kdtree(cuda, po):
    import torch
    lib = _lib()
    rng = np.random.default_rng(0)
    for N, nper in ((300, 300), (600, 200), (4096, 4096)):
        p = rng.uniform(0, 20, (N, 3)).astype(np.float32)
        nb = torch.empty((17, N), dtype=torch.int32, device="cuda")  # nb[n][i]
        dp = torch.tensor(p, device="cuda")
        assert lib.lmg_internal_knn(ctypes.c_void_p(dp.data_ptr()), N, nper,
                                    ctypes.c_void_p(nb.data_ptr()), None) == 0
        torch.cuda.synchronize()
        got = nb.cpu().numpy().T
        for b0 in range(0, N, nper):
            ref, _ = po.neighbours(p[b0:b0 + nper].astype(np.float64))
            ref = ref + b0
            assert (got[b0:b0 + nper, 0] == np.arange(b0, b0 + nper)).all()
            # same neighbour sets (order may differ only between equal distances)
            assert all(set(got[b0 + i]) == set(ref[i]) for i in range(nper))


def test_build_and_apply_match_oracle(cuda, po):
    import torch
    lib = _lib()
    rng = np.random.default_rng(1)
    N = 256
    p = _clustered(rng, N).astype(np.float32)
    params = _random_params(po, rng)
    dp = torch.tensor(p, device="cuda")
    nb = torch.empty((17, N), dtype=torch.int32, device="cuda")          # nb[n][i]
    blocks = torch.empty((17, 9, N), dtype=torch.float32, device="cuda")  # blocks[n][e][i]
    dparams = torch.tensor(params, device="cuda")
    assert lib.lmg_internal_knn(ctypes.c_void_p(dp.data_ptr()), N, N,
                                ctypes.c_void_p(nb.data_ptr()), None) == 0
    a, scale = 1.3, 0.7
    assert lib.lmg_internal_precond_build(ctypes.c_void_p(dp.data_ptr()),
                                          ctypes.c_void_p(nb.data_ptr()), N,
                                          ctypes.c_void_p(dparams.data_ptr()),
                                          1.0 / a, scale, ctypes.c_void_p(blocks.data_ptr()),
                                          None) == 0
    torch.cuda.synchronize()
    ref, nb_ref = po.p_blocks(p.astype(np.float64), params, a=a, scale=scale)
    got = blocks.cpu().numpy().transpose(2, 0, 1).reshape(N, 17, 3, 3)
    nbg = nb.cpu().numpy().T
    # compare row by row, matching neighbours by index
    for i in range(N):
        m = {int(j): got[i, n] for n, j in enumerate(nbg[i])}
        for n, j in enumerate(nb_ref[i]):
            assert np.allclose(m[int(j)], ref[i, n], rtol=2e-3, atol=2e-4 * np.abs(ref[i]).max())
    # sparse products against the dense matrix
    P = po.dense_p(got.astype(np.float64), nbg)
    x = rng.normal(size=3 * N).astype(np.float32)
    dx = torch.tensor(x, device="cuda")
    out = torch.empty(3 * N, device="cuda")
    for tr, ref_y in ((0, P @ x), (1, P.T @ x)):
        assert lib.lmg_internal_precond_apply(ctypes.c_void_p(blocks.data_ptr()),
                                              ctypes.c_void_p(nb.data_ptr()), N,
                                              ctypes.c_void_p(dx.data_ptr()),
                                              ctypes.c_void_p(out.data_ptr()), tr, None) == 0
        torch.cuda.synchronize()
        assert np.allclose(out.cpu().numpy(), ref_y, rtol=1e-4, atol=1e-5 * np.abs(ref_y).max())


@pytest.mark.parametrize("K,H", [(32, 64), (48, 64), (48, 256), (16, 128)])
def test_wider_networks_match_oracle(cuda, po, K, H):
    """kNN, P build and P / P^T products for networks over K = 16, 32 and
    48 neighbours and 64 to 256 hidden units, against the NumPy oracle."""
    import torch
    lib = _lib()
    rng = np.random.default_rng(K + H)
    N = 200
    p = _clustered(rng, N).astype(np.float32)
    d = {k: rng.normal(0, 0.3, shp) for k, shp in po.shapes(K, H)}
    d["W2"] *= np.sqrt(64 / H)
    d["W3"] *= np.sqrt(64 / H)
    d["xstd"] = np.abs(d["xstd"]) + 1.0
    d["ystd"] = np.abs(d["ystd"]) + 0.5
    params = np.concatenate([np.asarray(d[k], np.float32).ravel() for k, _ in po.shapes(K, H)])
    dp = torch.tensor(p, device="cuda")
    nb = torch.empty((K + 1, N), dtype=torch.int32, device="cuda")
    blocks = torch.empty((K + 1, 9, N), dtype=torch.float32, device="cuda")
    dparams = torch.tensor(params, device="cuda")
    assert lib.lmg_internal_knn_k(K, ctypes.c_void_p(dp.data_ptr()), N, N,
                                  ctypes.c_void_p(nb.data_ptr()), None) == 0
    a, scale = 1.3, 0.7
    assert lib.lmg_internal_precond_build_kh(K, H, ctypes.c_void_p(dp.data_ptr()),
                                            ctypes.c_void_p(nb.data_ptr()), N,
                                            ctypes.c_void_p(dparams.data_ptr()), 1.0 / a, scale,
                                            ctypes.c_void_p(blocks.data_ptr()), None) == 0
    torch.cuda.synchronize()
    ref, nb_ref = po.p_blocks(p.astype(np.float64), params, a=a, scale=scale)
    got = blocks.cpu().numpy().transpose(2, 0, 1).reshape(N, K + 1, 3, 3)
    nbg = nb.cpu().numpy().T
    for i in range(N):
        assert set(nbg[i]) == set(nb_ref[i])
        m = {int(j): got[i, n] for n, j in enumerate(nbg[i])}
        for n, j in enumerate(nb_ref[i]):
            assert np.allclose(m[int(j)], ref[i, n], rtol=2e-3, atol=2e-4 * np.abs(ref[i]).max())
    P = po.dense_p(got.astype(np.float64), nbg)
    x = rng.normal(size=3 * N).astype(np.float32)
    dx = torch.tensor(x, device="cuda")
    out = torch.empty(3 * N, device="cuda")
    for tr, ref_y in ((0, P @ x), (1, P.T @ x)):
        assert lib.lmg_internal_precond_apply_k(K, ctypes.c_void_p(blocks.data_ptr()),
                                                ctypes.c_void_p(nb.data_ptr()), N,
                                                ctypes.c_void_p(dx.data_ptr()),
                                                ctypes.c_void_p(out.data_ptr()), tr, None) == 0
        torch.cuda.synchronize()
        assert np.allclose(out.cpu().numpy(), ref_y, rtol=1e-4, atol=1e-5 * np.abs(ref_y).max())


@pytest.mark.parametrize("K,H", [(16, 64), (48, 128)])
def test_wall_network_build_matches_oracle(cuda, po, K, H):
    """The wall network's features (frame about the wall normal, height input,
    clamped at one radius) and P blocks against the NumPy oracle, on a slab
    above the wall with heights from below the radius up."""
    import torch
    lib = _lib()
    rng = np.random.default_rng(70 + K)
    N = 240
    p = np.column_stack([rng.uniform(0, 30, N), rng.uniform(0, 30, N),
                         rng.uniform(0.4, 12, N)]).astype(np.float32)
    d = {k: rng.normal(0, 0.3, shp) for k, shp in po.shapes(K, H, True)}
    d["xstd"] = np.abs(d["xstd"]) + 1.0
    d["ystd"] = np.abs(d["ystd"]) + 0.5
    params = np.concatenate([np.asarray(d[k], np.float32).ravel()
                             for k, _ in po.shapes(K, H, True)])
    dp = torch.tensor(p, device="cuda")
    nb = torch.empty((K + 1, N), dtype=torch.int32, device="cuda")
    blocks = torch.empty((K + 1, 9, N), dtype=torch.float32, device="cuda")
    dparams = torch.tensor(params, device="cuda")
    assert lib.lmg_internal_knn_k(K, ctypes.c_void_p(dp.data_ptr()), N, N,
                                  ctypes.c_void_p(nb.data_ptr()), None) == 0
    a, scale = 1.2, 0.9
    assert lib.lmg_internal_precond_build_wall(K, H, ctypes.c_void_p(dp.data_ptr()),
                                              ctypes.c_void_p(nb.data_ptr()), N,
                                              ctypes.c_void_p(dparams.data_ptr()), 1.0 / a,
                                              scale, ctypes.c_void_p(blocks.data_ptr()),
                                              None) == 0
    torch.cuda.synchronize()
    ref, nb_ref = po.p_blocks(p.astype(np.float64), params, a=a, scale=scale)
    got = blocks.cpu().numpy().transpose(2, 0, 1).reshape(N, K + 1, 3, 3)
    nbg = nb.cpu().numpy().T
    for i in range(N):
        assert set(nbg[i]) == set(nb_ref[i])
        m = {int(j): got[i, n] for n, j in enumerate(nbg[i])}
        for n, j in enumerate(nb_ref[i]):
            assert np.allclose(m[int(j)], ref[i, n], rtol=2e-3, atol=2e-4 * np.abs(ref[i]).max())


@pytest.mark.parametrize("K", [16, 48, 64])
def test_half_block_products_match_dense(cuda, po, K):
    """P x and P^T x with half-precision blocks (the solver's storage), the
    transposed one through the float4 work array given or allocated, against
    the dense P of the same half-rounded blocks."""
    import torch
    lib = _lib()
    rng = np.random.default_rng(K)
    N = 3 * K + 50
    p = _clustered(rng, N).astype(np.float32)
    dp = torch.tensor(p, device="cuda")
    nb = torch.empty((K + 1, N), dtype=torch.int32, device="cuda")
    assert lib.lmg_internal_knn_k(K, ctypes.c_void_p(dp.data_ptr()), N, N,
                                  ctypes.c_void_p(nb.data_ptr()), None) == 0
    blocks = torch.tensor(rng.normal(0, 0.3, (K + 1, 9, N)), dtype=torch.float16, device="cuda")
    got = blocks.float().cpu().numpy().transpose(2, 0, 1).reshape(N, K + 1, 3, 3)
    P = po.dense_p(got.astype(np.float64), nb.cpu().numpy().T)
    x = rng.normal(size=3 * N).astype(np.float32)
    dx = torch.tensor(x, device="cuda")
    pad = torch.full((4 * N,), 7.0, device="cuda")  # the product zeroes it first
    for tr, ref_y in ((0, P @ x), (1, P.T @ x)):
        for work in (pad, None):
            out = torch.full((3 * N,), 5.0, device="cuda")  # overwritten
            assert lib.lmg_internal_precond_apply_kh(
                K, ctypes.c_void_p(blocks.data_ptr()), 1, ctypes.c_void_p(nb.data_ptr()), N,
                ctypes.c_void_p(dx.data_ptr()), ctypes.c_void_p(out.data_ptr()), tr,
                None if work is None else ctypes.c_void_p(work.data_ptr()), None) == 0
            torch.cuda.synchronize()
            assert np.allclose(out.cpu().numpy(), ref_y, rtol=1e-4,
                               atol=1e-5 * np.abs(ref_y).max()), (tr, work is None)


@pytest.mark.parametrize("ta,tb", [(0, 0), (1, 0), (0, 1), (1, 1)])
def test_large_gemm_matches_numpy(cuda, ta, tb):
    """The register-blocked GEMM (used from 64 output tiles of 128 x 128 on):
    all transpositions, ragged sizes, bias, tanh and beta, against FP64."""
    import torch
    lib = _lib()
    rng = np.random.default_rng(10 * ta + tb)
    M, N, K = 1037, 1131, 150
    Am = rng.normal(size=(K, M) if ta else (M, K)).astype(np.float32)
    Bm = rng.normal(size=(N, K) if tb else (K, N)).astype(np.float32)
    bias = rng.normal(size=N).astype(np.float32)
    C0 = rng.normal(size=(M, N)).astype(np.float32)
    dA, dB = torch.tensor(Am, device="cuda"), torch.tensor(Bm, device="cuda")
    dbias, dC = torch.tensor(bias, device="cuda"), torch.tensor(C0, device="cuda")
    opA = Am.T if ta else Am
    opB = Bm.T if tb else Bm
    for act, beta in ((0, 0.0), (1, 0.0), (0, 0.5)):
        dC.copy_(torch.tensor(C0))
        rc = lib.lmg_internal_gemm(ta, tb, M, N, K, ctypes.c_void_p(dA.data_ptr()),
                                   Am.shape[1], ctypes.c_void_p(dB.data_ptr()), Bm.shape[1],
                                   ctypes.c_void_p(dC.data_ptr()), N,
                                   ctypes.c_void_p(dbias.data_ptr()), act, ctypes.c_float(beta),
                                   None)
        assert rc == 0
        torch.cuda.synchronize()
        ref = opA.astype(np.float64) @ opB.astype(np.float64) + bias + beta * C0
        if act:
            ref = np.tanh(ref)
        assert np.abs(dC.cpu().numpy() - ref).max() <= 1e-4 * max(1.0, np.abs(ref).max())


def test_training_kernels_gradient_check(cuda, po):
    """Forward pass and gradients of the project's GEMM/tanh/MSE/colsum
    kernels against the NumPy oracle."""
    import torch
    from libmobility_gb300 import precond
    lib = _lib()
    rng = np.random.default_rng(2)
    B = 96
    params = _random_params(po, rng)
    X = rng.normal(size=(B, 48)).astype(np.float32)
    T = rng.normal(size=(B, 150)).astype(np.float32)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    net = precond.GpuMLP(lib, torch, params, stream)
    dX = torch.tensor(X, device="cuda")
    dT = torch.tensor(T, device="cuda")
    H1 = torch.empty(B, 64, device="cuda")
    H2 = torch.empty_like(H1)
    Yp = torch.empty(B, 150, device="cuda")
    dY = torch.empty_like(Yp)
    dH1 = torch.empty_like(H1)
    dH2 = torch.empty_like(H1)
    net.forward(dX, H1, H2, Yp)
    net.backward(dX, H1, H2, Yp, dT, dY, dH2, dH1)
    torch.cuda.synchronize()
    d = po.unpack(params)
    h1, h2, y = po.forward(d, X.astype(np.float64))
    assert np.allclose(Yp.cpu().numpy(), y, rtol=1e-4, atol=1e-5 * np.abs(y).max())
    g = po.backward(d, X.astype(np.float64), h1, h2, y, T.astype(np.float64))
    for k in ("W1", "b1", "W2", "b2", "W3", "b3"):
        got = net.gview[k].cpu().numpy().reshape(g[k].shape)
        err = np.abs(got - g[k]).max() / np.abs(g[k]).max()
        assert err < 1e-4, (k, err)
    loss = float(net.loss.item()) / (B * 150)
    assert abs(loss - np.mean((y - T) ** 2)) < 1e-4 * np.mean((y - T) ** 2)


def test_identity_network_reproduces_plain(cuda, po):
    from libmobility_gb300 import NBody
    rng = np.random.default_rng(3)
    N = 300
    p = _clustered(rng, N)
    dW = rng.normal(size=3 * N)
    out = []
    for prec in (False, True):
        s = NBody("open", "open", "open", precision="float")
        s.setParameters()
        s.initialize(viscosity=1.0, hydrodynamicRadius=1.0, tolerance=1e-6)
        if prec:
            s.setPreconditioner("mlp", po.identity_params())
        s.setPositions(p)
        u, _, it, _ = s.sqrtMdotW_noise(dW)
        out.append((u.ravel(), it))
    (u0, it0), (u1, it1) = out
    # S = M / t0 up to FP32 rounding (P^T v is accumulated with atomics), and
    # the FP32 successive-iterate error sits near its floor at 1e-6, so the
    # stopping step may move by a few iterations; both results approximate
    # sqrt(M) dW to the tolerance scale
    assert abs(it0 - it1) <= 4
    assert np.linalg.norm(u1 - u0) / np.linalg.norm(u0) < 2e-5


def _trained():
    from libmobility_gb300 import precond
    if not precond.DEFAULT_WEIGHTS.exists():
        pytest.skip("no trained preconditioner weights shipped")
    return precond.DEFAULT_WEIGHTS


def test_trained_network_reduces_iterations(cuda, oracle):
    _trained()
    from libmobility_gb300 import NBody
    rng = np.random.default_rng(4)
    N = 2048
    p = _clustered(rng, N)
    res = {}
    for prec in ("none", "mlp"):
        s = NBody("open", "open", "open", precision="float")
        s.setParameters()
        s.initialize(viscosity=1.0, hydrodynamicRadius=1.0, tolerance=1e-6, seed=5)
        s.setPreconditioner(prec)
        s.setPositions(p)
        its = []
        for k in range(4):
            dW = np.random.default_rng(10 + k).normal(size=3 * N)
            u, _, it, _ = s.sqrtMdotW_noise(dW)
            its.append(it)
        res[prec] = np.mean(its[1:])
    assert res["mlp"] < 0.75 * res["none"], res


@pytest.mark.parametrize("ang", [False, True])
def test_trained_network_keeps_statistics(cuda, ang):
    """Fluctuation-dissipation with the preconditioner on (N = 64, clustered:
    above the K + 1 particles the shipped network needs), KS test per
    component of M^{-1/2} y as in the reference tests."""
    from libmobility_gb300 import precond
    w = precond.load_weights(_trained())
    k, _ = precond.shape_of_params(len(w))
    from libmobility_gb300 import NBody
    rng = np.random.default_rng(6)
    N = 64
    assert N >= k + 1
    p = _clustered(rng, N, phi=0.15, sigma=2.0)
    s = NBody("open", "open", "open", precision="float")
    s.setParameters()
    s.initialize(viscosity=1.0, hydrodynamicRadius=1.0, includeAngular=ang, tolerance=1e-6,
                 seed=11)
    s.setPreconditioner("mlp")
    s.setPositions(p)
    M = compute_M(s, N, ang)

    def draw():
        u, w = s.sqrtMdotW(prefactor=1.0)
        return np.concatenate([u.ravel(), w.ravel()]) if ang else u.ravel()

    _ks_fdt(M, draw)
