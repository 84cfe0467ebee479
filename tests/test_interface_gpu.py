"""Behaviour of the Python interface, ported from libMobility's
tests/test_interface.py, test_initialization.py, test_precision.py,
test_array_origins.py and test_thermal_drift.py for the NBody solver (open and
single wall), running on the GPU through the C ABI."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CONFIGS = [("open", "open", "open"), ("open", "open", "single_wall")]


def sane(periodicity):
    return {"algorithm": "advise", "delta": 1e-3,
            **({"wallHeight": 0.0} if periodicity[2] == "single_wall" else {})}


def init(periodicity, includeAngular=False, seed=None, precision=None):
    from libmobility_gb300 import NBody
    s = NBody(*periodicity, precision=precision)
    s.setParameters(**sane(periodicity))
    s.initialize(viscosity=1.0, hydrodynamicRadius=1.0, includeAngular=includeAngular, seed=seed)
    return s


def box(n):
    p = np.random.rand(n, 3) - 0.5
    p[:, 2] += 0.5
    return p * 10


@pytest.mark.parametrize("periodicity", CONFIGS)
def test_contiguous_and_shapes(cuda, periodicity):
    s = init(periodicity)
    s.setPositions(np.random.rand(1, 3))
    s.setPositions(np.random.rand(3, 3)[:, 0])  # non-contiguous column
    s = init(periodicity)
    pos = np.random.rand(2, 3)
    f = np.random.rand(2, 3)
    s.setPositions(pos)
    mf, mt = s.Mdot(f)
    assert mf.shape == f.shape and mt is None
    mf, mt = s.Mdot(f.reshape(6))
    assert mf.shape == (6,) and mt is None


@pytest.mark.parametrize("periodicity", CONFIGS)
def test_torques_and_forces_return_both(cuda, periodicity):
    s = init(periodicity, includeAngular=True)
    s.setPositions(np.random.rand(5, 3))
    t = np.random.rand(5, 3)
    for tt in (t, t.reshape(15)):
        mf, mt = s.Mdot(torques=tt)
        assert mf.shape == tt.shape and mt.shape == tt.shape
        assert np.linalg.norm(mf) > 0 and np.linalg.norm(mt) > 0
        mf, mt = s.Mdot(forces=tt)
        assert mf.shape == tt.shape and mt.shape == tt.shape
        assert np.linalg.norm(mf) > 0 and np.linalg.norm(mt) > 0
    for fs, ts in (((3,), (1, 3)), ((1, 3), (3,)), ((1, 3), (1, 3)), ((3,), (3,))):
        s.setPositions(box(1))
        u, w = s.Mdot(np.random.rand(*fs), np.random.rand(*ts))
        assert u.shape == fs and w.shape == ts


@pytest.mark.parametrize("periodicity", CONFIGS)
def test_returned_shapes_follow_positions(cuda, periodicity):
    s = init(periodicity)
    for shape in ((1, 3), (3,)):
        pos = box(1).reshape(shape)
        s.setPositions(pos)
        assert s.sqrtMdotW()[0].shape == shape
        assert s.divM()[0].shape == shape
        v, _ = s.LangevinVelocities(1.0, 1.0)
        assert v.shape == shape
        f = np.random.rand(1, 3)
        v, _ = s.LangevinVelocities(1.0, 1.0, f)
        assert v.shape == f.shape
    s = init(periodicity, includeAngular=True)
    s.setPositions(box(1))
    v, w = s.LangevinVelocities(1.0, 1.0, np.random.rand(3), np.random.rand(1, 3))
    assert v.shape == (3,) and w.shape == (1, 3)


@pytest.mark.parametrize("periodicity", CONFIGS)
def test_errors(cuda, periodicity):
    s = init(periodicity, includeAngular=False)
    s.setPositions(np.random.rand(1, 3))
    with pytest.raises(RuntimeError):
        s.Mdot(np.random.rand(1, 3), np.random.rand(1, 3))
    s = init(periodicity)
    s.setPositions(np.random.rand(5, 3))
    for nw in (4, 6):
        with pytest.raises(RuntimeError):
            s.Mdot(forces=np.random.rand(3 * nw))
    s = init(periodicity, includeAngular=True)
    s.setPositions(np.random.rand(5, 3))
    for nw in (4, 6):
        with pytest.raises(RuntimeError):
            s.Mdot(torques=np.random.rand(3 * nw))


@pytest.mark.parametrize("nbatch,nper", [(1, 12), (12, 1)])
def test_good_batch_parameters(cuda, nbatch, nper):
    """test_initialization.py: NBatch x NperBatch particles are accepted."""
    from libmobility_gb300 import NBody
    s = NBody("open", "open", "open")
    s.setParameters("advise", nbatch, nper)
    s.initialize(viscosity=1.0, hydrodynamicRadius=1.5)
    s.setPositions(np.random.rand(nbatch * nper, 3))


def test_default_and_no_parameters(cuda):
    """test_initialization.py: setParameters("advise") alone, and no
    setParameters at all (default algorithm, every particle in one batch),
    both take positions and give the same Mdot."""
    from libmobility_gb300 import NBody
    pos = np.random.rand(10, 3)
    out = []
    for with_params in (True, False):
        s = NBody("open", "open", "open")
        if with_params:
            s.setParameters("advise")
        s.initialize(viscosity=1.0, hydrodynamicRadius=1.5)
        s.setPositions(pos)
        mf, mt = s.Mdot(pos)
        assert mf.shape == (10, 3) and mt is None
        out.append(mf)
    assert np.array_equal(out[0], out[1])


@pytest.mark.parametrize("periodicity", CONFIGS)
@pytest.mark.parametrize("ang", [True, False])
def test_langevin_kbt0_equals_mdot(cuda, periodicity, ang):
    s = init(periodicity, includeAngular=ang)
    s.setPositions(np.random.rand(1, 3))
    args = (np.random.rand(1, 3), np.random.rand(1, 3)) if ang else (np.random.rand(1, 3),)
    mf, mt = s.Mdot(*args)
    bf, bt = s.LangevinVelocities(1.0, 0.0, *args)
    assert np.allclose(mf, bf, atol=1e-6)
    if ang:
        assert np.allclose(mt, bt, atol=1e-6)


@pytest.mark.parametrize("periodicity", CONFIGS)
@pytest.mark.parametrize("ang", [True, False])
def test_changing_number_of_particles(cuda, periodicity, ang):
    s = init(periodicity, includeAngular=ang)
    for n in (1, 2, 3):
        s.setPositions(np.random.rand(n, 3))
        args = (np.random.rand(n, 3), np.random.rand(n, 3)) if ang else (np.random.rand(n, 3),)
        mf, mt = s.Mdot(*args)
        assert mf.shape == (n, 3)
        dw, dt = s.sqrtMdotW()
        assert dw.shape == (n, 3)
        bf, bt = s.LangevinVelocities(1.0, 1.0, *args)
        assert bf.shape == (n, 3)
        if ang:
            assert bt.shape == dt.shape == mt.shape == (n, 3)


def test_wall_position_errors(cuda):
    from libmobility_gb300 import NBody
    s = NBody("open", "open", "single_wall")
    s.setParameters(wallHeight=1.0)
    s.initialize(viscosity=1.0, hydrodynamicRadius=1.0)
    with pytest.raises(RuntimeError, match="fallen below the wall"):
        s.setPositions(np.array([1.0, 2.0, 0.5]))
    import torch
    with pytest.raises(RuntimeError, match="fallen below the wall"):
        s.setPositions(torch.tensor([1.0, 2.0, 0.5], device="cuda"))
    s.setPositions(torch.tensor([1.0, 2.0, 1.5], device="cuda"))  # device path accepts


@pytest.mark.parametrize("periodicity", CONFIGS)
def test_precision(cuda, periodicity):
    for prec, good, bad in (("float", np.float32, np.float64), ("double", np.float64, np.float32)):
        s = init(periodicity, precision=prec)
        s.setPositions(np.random.rand(1, 3).astype(bad))
        s.setPositions(np.random.rand(1, 3).astype(good))
        mf, _ = s.Mdot(np.ones(3, dtype=bad))
        assert mf.dtype == good and (mf != 0).all()


@pytest.mark.parametrize("periodicity", CONFIGS)
@pytest.mark.parametrize("framework", ["numpy", "torch_cpu", "torch_cuda"])
@pytest.mark.parametrize("use_torques", [False, True])
@pytest.mark.parametrize("method", ["Mdot", "divM", "sqrtMdotW", "LangevinVelocities"])
def test_framework_round_trip(cuda, periodicity, framework, use_torques, method):
    import torch
    s = init(periodicity, includeAngular=use_torques)
    n = 10
    pos, f, t = box(n).astype(np.float32), np.random.rand(n, 3).astype(np.float32), \
        np.random.rand(n, 3).astype(np.float32)
    if framework != "numpy":
        dev = "cuda" if framework == "torch_cuda" else "cpu"
        pos, f, t = (torch.tensor(x, device=dev) for x in (pos, f, t))
    if not use_torques:
        t = None
    s.setPositions(pos)
    if method == "Mdot":
        mf, mt = s.Mdot(f, t)
    elif method == "divM":
        mf, mt = s.divM()
    elif method == "sqrtMdotW":
        mf, mt = s.sqrtMdotW()
    else:
        mf, mt = s.LangevinVelocities(1.0, 1.0, f, t)
    assert type(mf) == type(pos)
    if use_torques:
        assert type(mt) == type(pos)
    if framework != "numpy":
        assert mf.device == pos.device
        if use_torques:
            assert mt.device == pos.device


@pytest.mark.parametrize("periodicity", CONFIGS)
def test_divM_does_not_change_positions(cuda, periodicity):
    for wh in (0.0, 3.0):
        from libmobility_gb300 import NBody
        s = NBody(*periodicity)
        p = sane(periodicity)
        if "wallHeight" in p:
            p["wallHeight"] = wh
        s.setParameters(**p)
        s.initialize(viscosity=1.0, hydrodynamicRadius=1.0)
        pos = box(10)
        pos[:, 2] += wh
        s.setPositions(pos)
        f = np.random.normal(size=pos.shape)
        mf, _ = s.Mdot(f)
        s.divM()
        mf2, _ = s.Mdot(f)
        assert np.allclose(mf, mf2, atol=1e-7, rtol=1e-7)


@pytest.mark.parametrize("ang", [False, True])
def test_divM_returns_different_numbers(cuda, ang):
    s = init(CONFIGS[1], includeAngular=ang)
    s.setPositions(box(10) * 0.8)
    r1, _ = s.divM()
    r2, _ = s.divM()
    assert np.any(np.abs(r1 - r2) > 1e-5)
    s = init(CONFIGS[0], includeAngular=ang)
    s.setPositions(box(10))
    assert not s.divM()[0].any()  # no thermal drift in open space


def _deterministic_div_m(s, positions, ang, delta):
    N = positions.size // 3
    size = 6 * N if ang else 3 * N
    pos = positions.ravel()
    out = np.zeros(size)
    for j in range(3 * N):
        pp = pos.copy()
        pm = pos.copy()
        pp[j] += 0.5 * delta
        pm[j] -= 0.5 * delta
        e = np.zeros(size)
        e[j] = 1.0
        f = e[: 3 * N]
        t = e[3 * N:] if ang else None
        s.setPositions(pp)
        a, b = s.Mdot(forces=f, torques=t)
        s.setPositions(pm)
        c, d = s.Mdot(forces=f, torques=t)
        out[: 3 * N] += a - c
        if ang:
            out[3 * N:] += b - d
    s.setPositions(positions)
    return out / delta


@pytest.mark.parametrize("ang", [False, True])
@pytest.mark.parametrize("a", [0.4, 1.0, 2.5])
def test_thermal_drift_matches_finite_differences(cuda, ang, a):
    """test_thermal_drift.py: the running average of RFD divM converges to a
    deterministic central difference (tol 1e-3, checked every 5000 samples)."""
    from libmobility_gb300 import NBody
    s = NBody("open", "open", "single_wall", precision="double")
    s.setParameters(wallHeight=0.0, delta=1e-3)
    s.initialize(viscosity=1.0, hydrodynamicRadius=a, includeAngular=ang, seed=99)
    np.random.seed(7)
    pos = box(10)
    s.setPositions(pos)
    det = _deterministic_div_m(s, pos, ang, 1e-3 * a)
    acc_m = np.zeros(30)
    acc_d = np.zeros(30)
    tol = 1e-3
    ok = False
    for i in range(1, 250002):
        m, d = s.divM()
        acc_m += m.ravel()
        if ang:
            acc_d += d.ravel()
        if i % 5000 == 0:
            good = np.allclose(acc_m / i, det[:30], atol=tol, rtol=tol)
            if ang:
                good = good and np.allclose(acc_d / i, det[30:], atol=tol, rtol=tol)
            if good:
                ok = True
                break
    assert ok
