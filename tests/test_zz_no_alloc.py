"""The allocation-free Mdot entry point (lmg_mdot_noalloc_f32).

It serves callers that may not allocate device memory themselves or through
this library (programs that own all device memory through their own pool, or
loops that cannot take the device-wide synchronisation of cudaMalloc/cudaFree).
This test calls it through the C ABI with device buffers it prepared
beforehand, twice in a row per case, and checks each result against the handle
API's Mdot within the FP32 tolerance of the other Mdot tests (1e-5 relative);
the scratch it shares between calls must not leak one call into the next.
After the first call has set up the device, a call must leave the device's
free memory unchanged.

The file is named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(x, ref):
    x = np.asarray(x, np.float64)
    ref = np.asarray(ref, np.float64)
    return np.abs(x - ref).max() / np.abs(ref).max()


CASES = [
    # (single_wall, includeAngular, torques, N, NperBatch)
    (1, 1, 1, 16384, -1),   # bench-size wall problem: split sources, scratch in use
    (0, 0, 0, 4096, -1),    # open, forces only
    (0, 1, 1, 3000, 1000),  # batches
    (1, 1, 0, 777, -1),     # odd size, forces with angular output
    (1, 0, 0, 1, -1),       # single particle
]


@pytest.mark.parametrize("case", CASES)
def test_noalloc_matches_handle_mdot(cuda, case):
    import torch
    from libmobility_gb300 import NBody, _capi
    lib = _capi.load()
    wall, ang, has_t, N, nper = case
    rng = np.random.default_rng(N + 10 * wall)
    if wall:
        pos = np.column_stack([rng.uniform(0, 128, N), rng.uniform(0, 128, N),
                               rng.uniform(0.5, 20, N)])
    else:
        L = (N * 4 * np.pi / 3 / 0.05) ** (1 / 3)
        pos = rng.uniform(0, L, (N, 3))
    F = rng.normal(size=(N, 3))
    T = rng.normal(size=(N, 3)) if has_t else None
    a, eta = 1.0, 1 / (6 * np.pi)

    ref = NBody("open", "open", "single_wall" if wall else "open", precision="float")
    if wall:
        ref.setParameters("advise", -1 if nper < 0 else N // nper, nper, wallHeight=0.0)
    else:
        ref.setParameters("advise", -1 if nper < 0 else N // nper, nper)
    ref.initialize(viscosity=eta, hydrodynamicRadius=a, includeAngular=bool(ang))
    ref.setPositions(pos)
    U_ref, W_ref = ref.Mdot(F, T)

    f32 = dict(dtype=torch.float32, device="cuda")
    dpos = torch.tensor(pos, **f32)
    dF = torch.tensor(F, **f32)
    dT = torch.tensor(T, **f32) if has_t else None
    U = torch.empty((N, 3), **f32)
    W = torch.empty((N, 3), **f32) if ang else None
    err = ctypes.create_string_buffer(256)
    stream = torch.cuda.current_stream().cuda_stream
    ptr = lambda t: None if t is None else ctypes.c_void_p(t.data_ptr())
    torch.cuda.synchronize()
    for call in range(2):
        U.fill_(float("nan"))
        if W is not None:
            W.fill_(float("nan"))
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        rc = lib.lmg_mdot_noalloc_f32(ptr(dpos), ptr(dF), ptr(dT), ptr(U), ptr(W), N, nper,
                                      wall, eta, a, ang, ctypes.c_void_p(stream), err, 256)
        assert rc == 0, err.value.decode()
        torch.cuda.synchronize()
        if call == 1:  # set-up is done: this call must not take device memory
            assert torch.cuda.mem_get_info()[0] == free_before
        assert _rel(U.cpu().numpy(), U_ref) <= 1e-5, call
        if ang:
            assert _rel(W.cpu().numpy(), W_ref) <= 1e-5, call


def test_noalloc_rejects_bad_arguments(cuda):
    import torch
    from libmobility_gb300 import _capi
    lib = _capi.load()
    err = ctypes.create_string_buffer(256)
    d = torch.zeros((4, 3), device="cuda")
    p = ctypes.c_void_p(d.data_ptr())
    too_many = (1 << 24) + 1
    rc = lib.lmg_mdot_noalloc_f32(p, p, None, p, None, too_many, -1, 0, 1.0, 1.0, 0, None,
                                  err, 256)
    assert rc == 1 and b"numberParticles must be in" in err.value
    host = np.zeros((4, 3), np.float32)
    rc = lib.lmg_mdot_noalloc_f32(ctypes.c_void_p(host.ctypes.data), p, None, p, None, 4, -1, 0,
                                  1.0, 1.0, 0, None, err, 256)
    assert rc == 1 and b"device buffers only" in err.value
    rc = lib.lmg_mdot_noalloc_f32(p, p, p, p, None, 4, -1, 0, 1.0, 1.0, 0, None, err, 256)
    assert rc == 1 and b"angular" in err.value


@pytest.mark.parametrize("wall,ang,N", [(1, 1, 2048), (0, 0, 4096)])
def test_noalloc_matches_fp64_oracle(cuda, oracle, wall, ang, N):
    """Parity of the allocation-free entry point on its own, independent of the
    handle API: two calls in a row against the FP64 oracle (1e-5 relative)."""
    import torch
    from libmobility_gb300 import _capi
    lib = _capi.load()
    rng = np.random.default_rng(900 + N)
    if wall:
        pos = np.column_stack([rng.uniform(0, 64, N), rng.uniform(0, 64, N),
                               rng.uniform(0.5, 15, N)])
    else:
        pos = rng.uniform(0, (N * 4 * np.pi / 3 / 0.05) ** (1 / 3), (N, 3))
    F = rng.normal(size=(N, 3))
    T = rng.normal(size=(N, 3)) if ang else None
    a, eta = 1.1, 0.7
    Uo, Wo = oracle.mdot(pos, F, T, a=a, viscosity=eta, wall=wall, include_angular=ang)
    f32 = dict(dtype=torch.float32, device="cuda")
    dpos, dF = torch.tensor(pos, **f32), torch.tensor(F, **f32)
    dT = torch.tensor(T, **f32) if ang else None
    U = torch.empty((N, 3), **f32)
    W = torch.empty((N, 3), **f32) if ang else None
    err = ctypes.create_string_buffer(256)
    ptr = lambda t: None if t is None else ctypes.c_void_p(t.data_ptr())  # noqa: E731
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        U.fill_(float("nan"))
        rc = lib.lmg_mdot_noalloc_f32(ptr(dpos), ptr(dF), ptr(dT), ptr(U), ptr(W), N, -1, wall,
                                      eta, a, ang, stream, err, 256)
        assert rc == 0, err.value.decode()
        torch.cuda.synchronize()
        assert _rel(U.cpu().numpy(), Uo) <= 1e-5, call
        if ang:
            assert _rel(W.cpu().numpy(), Wo) <= 1e-5, call


def test_noalloc_needs_forces_or_torques(cuda):
    import torch
    from libmobility_gb300 import _capi
    lib = _capi.load()
    err = ctypes.create_string_buffer(256)
    d = torch.zeros((4, 3), device="cuda")
    p = ctypes.c_void_p(d.data_ptr())
    rc = lib.lmg_mdot_noalloc_f32(p, None, None, p, None, 4, -1, 0, 1.0, 1.0, 0, None, err, 256)
    assert rc == 1 and b"F and/or T" in err.value
