"""The symmetric open-space product (FP32, forces only) on the GPU.

FP32 handles with an open boundary, forces only and no angular part take the
kernel that evaluates each unordered pair once and applies it to both
particles (csrc/mdot_sym.cu).  It is checked against the FP64 oracle (FP32
tolerance 1e-5 relative, as every Mdot test) on ragged tiles and batches,
with the rotation steps cut over many different numbers of warps, in every
register-budget build, on overlapping and coincident particles, and against
mdot_kernel on the same handle; two calls in a row give bitwise the same
result (the barrier count is per plan and the fold order is fixed).
"""
import numpy as np
import pytest

from test_mdot_gpu import make_solver, rel_err

pytestmark = pytest.mark.gpu
TOL = 1e-5


@pytest.fixture()
def lib(cuda):
    from libmobility_gb300 import _capi
    lib = _capi.load()
    yield lib
    lib.lmg_internal_sym_override(0, 0)
    lib.lmg_internal_sym_override(2, 0)


def _cube(rng, N, phi):
    L = (N * 4 * np.pi / 3 / phi) ** (1 / 3)
    return rng.uniform(0, L, (N, 3))


@pytest.mark.parametrize("warps", [0, 1, 3, 7, 37, 200])
def test_sym_matches_oracle_ragged_batches(lib, oracle, warps):
    """Ragged tiles and batches; the rotation steps spread over `warps` warps
    (0: the planner's choice), so tile pairs are cut at many different steps
    and their sums come from one or several warps.  (33, 11) and (1000, 250)
    have batches the kernel declines (not a multiple of 4): mdot_kernel runs."""
    rng = np.random.default_rng(501 + warps)
    assert lib.lmg_internal_sym_override(0, warps) == 0
    for N, nper in ((1, 1), (5, 5), (33, 11), (128, 128), (129, 129), (257, 257),
                    (1000, 250), (1537, 1537), (3000, 1000), (640, 128)):
        p = _cube(rng, N, 0.1)
        F = rng.normal(size=(N, 3))
        s = make_solver(0, 0, 1.1, 0.9, "float", N, nper)
        s.setPositions(p)
        U, _ = s.Mdot(F, None)
        Uo, _ = oracle.mdot(p, F, None, a=1.1, viscosity=0.9, wall=0, include_angular=0,
                            nper_batch=nper)
        assert rel_err(U, Uo) <= TOL, (N, nper, warps)


@pytest.mark.parametrize("variant", [2, 3, 4])
def test_sym_every_register_budget(lib, oracle, variant):
    rng = np.random.default_rng(60 + variant)
    assert lib.lmg_internal_sym_override(variant, 0) == 0
    for N in (257, 4096):
        p = _cube(rng, N, 0.2)
        F = rng.normal(size=(N, 3))
        s = make_solver(0, 0, 1.0, 1 / (6 * np.pi), "float")
        s.setPositions(p)
        U, _ = s.Mdot(F, None)
        Uo, _ = oracle.mdot(p, F, None, a=1.0, viscosity=1 / (6 * np.pi), wall=0,
                            include_angular=0)
        assert rel_err(U, Uo) <= TOL, (N, variant)


def test_sym_overlapping_and_coincident(lib, oracle):
    """Dense packing (many pairs closer than 2a) and exact duplicates (r = 0
    between distinct particles) take the exact near-field formula."""
    rng = np.random.default_rng(77)
    for N in (300, 2048):
        p = _cube(rng, N, 0.45)
        p[N // 2:N // 2 + 7] = p[3]          # coincident with particle 3
        p[N - 5:] = p[N - 10:N - 5] + 1e-3   # nearly coincident pairs
        F = rng.normal(size=(N, 3))
        s = make_solver(0, 0, 1.0, 1 / (6 * np.pi), "float")
        s.setPositions(p)
        U, _ = s.Mdot(F, None)
        Uo, _ = oracle.mdot(p, F, None, a=1.0, viscosity=1 / (6 * np.pi), wall=0,
                            include_angular=0)
        assert rel_err(U, Uo) <= TOL, N


def test_sym_agrees_with_tiled_kernel_and_repeats_bitwise(lib):
    rng = np.random.default_rng(5)
    N = 4096
    p = _cube(rng, N, 0.05)
    F = rng.normal(size=(N, 3))
    s = make_solver(0, 0, 1.0, 1 / (6 * np.pi), "float")
    s.setPositions(p)
    U1, _ = s.Mdot(F, None)
    U2, _ = s.Mdot(F, None)
    assert np.array_equal(U1, U2)
    assert lib.lmg_internal_sym_override(1, 0) == 0
    Uk, _ = s.Mdot(F, None)
    assert rel_err(U1, Uk) <= 2 * TOL
    assert not np.array_equal(U1, Uk)  # the two kernels really are different code


def test_sym_open4k_full_rows_vs_oracle(lib, oracle):
    """N = 4096 open, volume fraction 0.05, a = 1, viscosity 1/(6 pi): every row
    against the FP64 oracle."""
    rng = np.random.default_rng(2024)
    N = 4096
    p = _cube(rng, N, 0.05)
    F = rng.normal(size=(N, 3))
    s = make_solver(0, 0, 1.0, 1 / (6 * np.pi), "float")
    s.setPositions(p)
    U, _ = s.Mdot(F, None)
    Uo, _ = oracle.mdot(p, F, None, a=1.0, viscosity=1 / (6 * np.pi), wall=0,
                        include_angular=0)
    assert rel_err(U, Uo) <= TOL
