"""The tensor-core GEMM of the preconditioner network (tcgen05.mma of
kind::tf32, TMA-fed, accumulator in tensor memory): C = act(A Bt^T + bias)
against an FP64 reference on the same FP32 inputs.  TF32 keeps 10 mantissa
bits of each operand, so the bound is 3e-3 of the largest |C| (measured
errors are a few 1e-4 of it); shapes cover partial tiles in M and N, K not a
multiple of the 32-wide stages (zero-filled by TMA), padded leading
dimensions, and both activations.  The status word of the kernel's bounded
waits must stay clear.  Then the preconditioner build with the network on
the tensor cores against the CUDA-core build: the same P within TF32
rounding, and a preconditioned solve that converges in about as many
iterations."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [
    # M, N, K, lda, ldbt, act
    (128, 256, 32, 32, 32, 0),      # one tile, one stage
    (1000, 512, 145, 148, 148, 1),  # first layer of the wall network
    (4096, 438, 512, 512, 512, 0),  # output layer
    (129, 17, 7, 8, 8, 1),          # tiny, partial tiles everywhere
    (300, 600, 40, 44, 40, 1),      # three column tiles, padded A
]


@pytest.mark.parametrize("M,N,K,lda,ldbt,act", SHAPES)
def test_tc_gemm_matches_fp64(cuda, M, N, K, lda, ldbt, act):
    import torch
    from libmobility_gb300 import _capi
    lib = _capi.load()
    if lib.lmg_internal_tc_status(1) != 0:
        pytest.fail("status word set before the test")
    rng = np.random.default_rng(M + 7 * N + K)
    A = np.zeros((M, lda), np.float32)
    A[:, :K] = rng.normal(size=(M, K))
    Bt = np.zeros((N, ldbt), np.float32)
    Bt[:, :K] = rng.normal(size=(N, K)) / np.sqrt(K)
    bias = rng.normal(size=N).astype(np.float32)
    ref = A[:, :K].astype(np.float64) @ Bt[:, :K].astype(np.float64).T + bias
    if act:
        ref = np.tanh(ref)
    dA = torch.tensor(A, device="cuda")
    dB = torch.tensor(Bt, device="cuda")
    db = torch.tensor(bias, device="cuda")
    dC = torch.full((M, N), float("nan"), device="cuda")
    p = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    rc = lib.lmg_internal_tc_gemm(M, N, K, p(dA), lda, p(dB), ldbt, p(dC), N, p(db), act,
                                  ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0
    C = dC.cpu().numpy().astype(np.float64)
    assert lib.lmg_internal_tc_status(1) == 0
    assert np.isfinite(C).all()
    err = np.abs(C - ref).max() / np.abs(ref).max()
    assert err <= 3e-3, err


def test_tc_gemm_rejects_bad_arguments(cuda):
    import torch
    from libmobility_gb300 import _capi
    lib = _capi.load()
    d = torch.zeros(64 * 64, device="cuda")
    p = ctypes.c_void_p(d.data_ptr())
    odd = ctypes.c_void_p(d.data_ptr() + 4)  # not 16-byte aligned
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.lmg_internal_tc_gemm(8, 8, 6, p, 6, p, 8, p, 8, None, 0, s) != 0  # lda % 4
    assert lib.lmg_internal_tc_gemm(8, 8, 8, odd, 8, p, 8, p, 8, None, 0, s) != 0
    assert lib.lmg_internal_tc_gemm(8, 8, 8, p, 4, p, 8, p, 8, None, 0, s) != 0  # lda < K
    assert lib.lmg_internal_tc_gemm(8, 8, 8, p, 8, p, 8, p, 8, None, 2, s) != 0  # act


@pytest.mark.parametrize("wall", [0, 1])
def test_precond_build_on_tensor_cores(cuda, wall):
    import torch
    from libmobility_gb300 import NBody, _capi
    from libmobility_gb300 import precond as pc
    lib = _capi.load()
    rng = np.random.default_rng(5 + wall)
    N = 6000
    L = (N * 4 * np.pi / 3 / 0.2) ** (1 / 3)
    pos = rng.uniform(0, L, (N, 3))
    if wall:
        pos[:, 2] = rng.uniform(1.0, 8.0, N)
    params = pc.load_weights(pc.default_weights(bool(wall)), wall=bool(wall))
    k, h = pc.shape_of_params(len(params))
    dpos = torch.tensor(pos, dtype=torch.float32, device="cuda")
    dparams = torch.tensor(params, dtype=torch.float32, device="cuda")
    nb = torch.empty((k + 1, N), dtype=torch.int32, device="cuda")
    assert lib.lmg_internal_knn_k(k, ctypes.c_void_p(dpos.data_ptr()), N, N,
                                  ctypes.c_void_p(nb.data_ptr()), None) == 0
    fn = lib.lmg_internal_precond_build_wall if wall else lib.lmg_internal_precond_build_kh
    blocks = {}
    try:
        for tc in (0, 1):
            assert lib.lmg_internal_precond_tc(tc) == 0
            out = torch.zeros((k + 1, 9, N), dtype=torch.float32, device="cuda")
            rc = fn(k, h, ctypes.c_void_p(dpos.data_ptr()), ctypes.c_void_p(nb.data_ptr()), N,
                    ctypes.c_void_p(dparams.data_ptr()), 1.0, 1.0,
                    ctypes.c_void_p(out.data_ptr()), None)
            assert rc == 0
            torch.cuda.synchronize()
            blocks[tc] = out.cpu().numpy().astype(np.float64)
        assert lib.lmg_internal_tc_status(1) == 0
        ref = blocks[0]
        assert np.abs(blocks[1] - ref).max() <= 2e-2 * np.abs(ref).max()
        # the preconditioned solve converges as well (any nonsingular P keeps
        # the statistics; only the iteration count depends on P)
        its = {}
        z = rng.normal(size=3 * N)
        for tc in (0, 1):
            assert lib.lmg_internal_precond_tc(tc) == 0
            s = NBody("open", "open", "single_wall" if wall else "open", precision="float")
            if wall:
                s.setParameters("advise", wallHeight=0.0)
            else:
                s.setParameters("advise")
            s.initialize(viscosity=1.0, hydrodynamicRadius=1.0, tolerance=1e-4)
            s.setPositions(pos)
            s.setPreconditioner("mlp")
            _, _, its[tc], _ = s.sqrtMdotW_noise(z)
        assert abs(its[1] - its[0]) <= max(2, 0.1 * its[0])
    finally:
        lib.lmg_internal_precond_tc(0)
