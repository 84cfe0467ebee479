"""Host-side pieces of the wall-aware learned preconditioner (no GPU).

* The NumPy wall translational mobility the wall network is trained on
  (libmobility_gb300.precond.wall_uf_matrix) against the FP64 C oracle, which
  restates the reference's BottomWall::dotProduct_UF entry by entry: heights
  below the radius (damping, clamping) included.
* The frame of wall networks turns about the wall normal only, so features are
  unchanged by rotations about z and horizontal shifts.
* Parameter counts tell open and wall networks apart.
"""
import numpy as np
import pytest


def test_wall_mobility_matches_oracle(oracle):
    from libmobility_gb300 import precond
    rng = np.random.default_rng(12)
    for N in (2, 7, 40):
        p = np.column_stack([rng.uniform(0, 12, N), rng.uniform(0, 12, N),
                             rng.uniform(0.3, 9, N)])
        M = precond.wall_uf_matrix(p[None])[0]
        Mo = oracle.dense(p, a=1.0, viscosity=1 / (6 * np.pi), wall=True,
                          include_angular=False)
        assert np.abs(M - Mo).max() <= 1e-12 * np.abs(Mo).max(), N


def test_wall_features_invariant_about_the_normal():
    from libmobility_gb300 import precond
    rng = np.random.default_rng(3)
    p = precond.random_system(rng, 400, 0.05, False, slab=(1.5, 20.0))
    ids = np.arange(20)
    X, Y = precond.samples_from_wall_system(p, ids, 16)
    th = 0.7
    Rz = np.array([[np.cos(th), -np.sin(th), 0], [np.sin(th), np.cos(th), 0], [0, 0, 1]])
    q = p @ Rz.T + np.array([5.0, -3.0, 0.0])
    X2, Y2 = precond.samples_from_wall_system(q, ids, 16)
    assert np.allclose(X, X2, atol=1e-4) and np.allclose(Y, Y2, atol=1e-4)
    E = precond.wall_frames(p[:5, None, :] - p[5:10, None, :])
    assert np.allclose(E[:, 2], [0, 0, 1]) and np.allclose(E @ E.transpose(0, 2, 1), np.eye(3))


def test_open_and_wall_layouts_are_told_apart():
    from libmobility_gb300 import precond
    seen = set()
    for wall in (False, True):
        for k in (16, 32, 48, 64):
            for h in (64, 128, 256, 512, 1024):
                n = sum(int(np.prod(s)) for _, s in precond.layout(k, h, wall))
                assert n not in seen
                seen.add(n)
                assert precond.kind_of_params(n) == (k, h, wall)
    with pytest.raises(ValueError):
        precond.kind_of_params(777)
