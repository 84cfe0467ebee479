"""Host-side logic of the ensemble and the learned preconditioner, on a
machine without a GPU: argument checks of the ensemble that come before any
CUDA call, and the network-shape bookkeeping (parameter layouts, the shipped
weights, the C side agreeing with the Python side on every supported size)."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def lib():
    from libmobility_gb300 import _build
    _build.build()
    from libmobility_gb300 import _capi
    return _capi.load()


def test_ensemble_argument_checks(lib):
    from libmobility_gb300.ensemble import Ensemble
    e = Ensemble(precision="float")
    with pytest.raises(RuntimeError, match="at least one particle"):
        e.setSystems([10, 0], [0, 1])
    with pytest.raises(RuntimeError, match="geometry"):
        e.setSystems([10, 5], [0, 2])
    with pytest.raises(RuntimeError, match="open.*single_wall"):
        e.setSystems([10, 5], ["open", "periodic"])
    with pytest.raises(RuntimeError, match="one entry per system"):
        e.setSystems([10, 5], [0, 1], [0.0])
    with pytest.raises(RuntimeError, match="no systems"):
        e.setPositions(np.zeros((3, 3)))
    with pytest.raises(RuntimeError):
        Ensemble(precision="half")
    assert e.describe()["systems"] == 0


def test_network_layouts_are_distinct_and_match_the_oracle():
    from libmobility_gb300 import precond
    from oracle import precond_oracle as po
    seen = {}
    for k in (16, 32, 48, 64):
        for h in (64, 128, 256, 512, 1024):
            n = sum(int(np.prod(s)) for _, s in precond.layout(k, h))
            assert n not in seen, (k, h, seen.get(n))
            seen[n] = (k, h)
            assert precond.shape_of_params(n) == (k, h)
            assert [s for _, s in precond.layout(k, h)] == [s for _, s in po.shapes(k, h)]
    with pytest.raises(ValueError):
        precond.shape_of_params(12345)


def test_shipped_weights_load():
    from libmobility_gb300 import precond
    w = precond.load_weights()
    k, h = precond.shape_of_params(len(w))
    assert (k, h) == (48, 512) and np.isfinite(w).all()
    w16 = precond.load_weights(precond.weights_path(16))
    assert precond.shape_of_params(len(w16)) == (16, 64)
