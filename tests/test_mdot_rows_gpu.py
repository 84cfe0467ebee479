"""Row products (lmg_mdot_rows / NBody.Mdot_rows): rows [b, e) of M.[F;T]
for forces and torques of all particles, the matrix-vector product of one rank
of a row-partitioned solve.  Each case is checked against the FP64 oracle's
rows on the inputs the solver holds (rounded to FP32 for "float"; 1e-5
relative in FP32, 1e-12 in FP64, the Mdot tolerances) and against
the same rows of the whole product from lmg_mdot (same tolerances: the two
launches may split the sources differently, so the sums may round apart)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {"float": 1e-5, "double": 1e-12}


def _rel(x, ref):
    x = np.asarray(x, np.float64)
    ref = np.asarray(ref, np.float64)
    return np.abs(x - ref).max() / max(np.abs(ref).max(), 1e-300)


def _system(N, wall, seed):
    rng = np.random.default_rng(seed)
    if wall:
        L = (N * 4 * np.pi / 3 / 0.1) ** 0.5
        pos = np.column_stack([rng.uniform(0, L, N), rng.uniform(0, L, N),
                               rng.uniform(0.6, 6.0, N)])
    else:
        L = (N * 4 * np.pi / 3 / 0.05) ** (1 / 3)
        pos = rng.uniform(0, L, (N, 3))
    return pos, rng.normal(size=(N, 3)), rng.normal(size=(N, 3))


CASES = [
    # (precision, wall, includeAngular, torques, N, NperBatch, rows)
    ("float", 0, 0, 0, 4096, -1, (0, 1000)),
    ("float", 0, 0, 0, 4096, -1, (1000, 4096)),
    ("float", 0, 0, 0, 4096, -1, (17, 18)),
    ("float", 1, 1, 1, 16384, -1, (5000, 9001)),
    ("float", 1, 1, 0, 3000, 1000, (900, 2100)),   # crosses batch boundaries
    ("float", 0, 1, 1, 3000, 750, (0, 3000)),      # all rows: the whole product
    ("double", 0, 0, 0, 2048, -1, (333, 1500)),
    ("double", 1, 1, 1, 2048, 512, (500, 1100)),
]


@pytest.mark.parametrize("case", CASES)
def test_rows_match_oracle_and_full_mdot(cuda, oracle, case):
    from libmobility_gb300 import NBody
    prec, wall, ang, has_t, N, nper, (b, e) = case
    pos, F, T = _system(N, wall, 7 * N + b)
    T = T if has_t else None
    a, eta = 1.0, 1 / (6 * np.pi)
    s = NBody("open", "open", "single_wall" if wall else "open", precision=prec)
    nb = -1 if nper < 0 else N // nper
    if wall:
        s.setParameters("advise", nb, nper, wallHeight=0.0)
    else:
        s.setParameters("advise", nb, nper)
    s.initialize(viscosity=eta, hydrodynamicRadius=a, includeAngular=bool(ang))
    s.setPositions(pos)
    U, W = s.Mdot_rows(b, e, F, T)
    assert U.shape == (e - b, 3)
    # the oracle on the inputs the solver holds (rounded to FP32 in "float")
    held = (lambda x: x) if prec == "double" else (
        lambda x: None if x is None else x.astype(np.float32).astype(np.float64))
    Uo, Wo = oracle.mdot(held(pos), held(F), held(T), a=a, viscosity=eta, wall=wall,
                         include_angular=ang, nper_batch=None if nper < 0 else nper,
                         rows=(b, e))
    assert _rel(U, Uo) <= TOL[prec]
    Uf, Wf = s.Mdot(F, T)
    assert _rel(U, Uf[b:e]) <= TOL[prec]
    if ang:
        assert W.shape == (e - b, 3)
        assert _rel(W, Wo) <= TOL[prec]
        assert _rel(W, Wf[b:e]) <= TOL[prec]
    else:
        assert W is None


def test_rows_device_buffers_and_repeat(cuda):
    """Torch CUDA inputs and outputs; two calls give identical rows, and a
    call for other rows in between does not disturb them."""
    import torch
    from libmobility_gb300 import NBody
    N = 8192
    pos, F, _ = _system(N, 0, 3)
    s = NBody("open", "open", "open", precision="float")
    s.setParameters("advise")
    s.initialize(viscosity=1.0, hydrodynamicRadius=1.0)
    s.setPositions(torch.tensor(pos, dtype=torch.float32, device="cuda"))
    Fd = torch.tensor(F, dtype=torch.float32, device="cuda")
    U1, _ = s.Mdot_rows(1024, 5000, Fd)
    s.Mdot_rows(0, 77, Fd)
    U2, _ = s.Mdot_rows(1024, 5000, Fd)
    assert U1.is_cuda and torch.equal(U1, U2)
    Uf, _ = s.Mdot(Fd)
    assert _rel(U1.cpu().numpy(), Uf[1024:5000].cpu().numpy()) <= 1e-5


def test_rows_rejects_bad_ranges(cuda):
    from libmobility_gb300 import NBody
    N = 64
    pos, F, _ = _system(N, 0, 1)
    s = NBody("open", "open", "open", precision="float")
    s.setParameters("advise")
    s.initialize(viscosity=1.0, hydrodynamicRadius=1.0)
    s.setPositions(pos)
    for b, e in [(-1, 4), (10, 10), (20, 10), (0, N + 1)]:
        with pytest.raises(RuntimeError, match="row_begin"):
            s.Mdot_rows(b, e, F)
