"""Training and loading of the learned sparse preconditioner (see
csrc/precond.cuh for what P is and why it is sparse).

Training data are made by the method itself: random small particle systems
(N uniform in max(64, K+1)..512, volume fraction uniform in 0.05..0.3, half of them as
Gaussian clusters of ~128 particles with sigma = 4a, overlaps at 2a removed);
for sampled particles the (K+1)-particle neighbourhood mobility (open-boundary
RPY, t0 = 1, a = 1; K = 16, 32, 48 or 64 nearest neighbours) is inverted-square-
rooted exactly in FP64 (dense eigh) and its first block row, rotated into the
particle's canonical frame, is the target.

Wall networks (--wall) are trained the same way on slabs above a single bottom
wall (x, y uniform, heights uniform between 1a or 1.5a and 8a..60a, volume
fraction 0.01..0.2, overlaps at 2a removed), with the neighbourhood's
translational wall mobility (RPY plus the Swan-Brady image, the reference's
BottomWall::dotProduct_UF) as the matrix, a frame that turns about the wall
normal only, and the particle's height as one more input.

The network is trained on the GPU by this project's own kernels
(lmg_internal_gemm / _tanh_backward / _mse_grad / _colsum / _adam in
csrc/precond.cu); PyTorch only provides device memory.

    python -m libmobility_gb300.precond train --k 48 --systems 20000 --out weights.npz
"""
import argparse
import ctypes
import json
import math
import multiprocessing as mp
import os
import time
from pathlib import Path

import numpy as np

NH = 64  # default hidden width
WEIGHTS_DIR = Path(__file__).resolve().parent / "weights"


def weights_path(k, h=NH, wall=False):
    if wall:
        return WEIGHTS_DIR / f"precond_wall_k{k}_h{h}.npz"
    return WEIGHTS_DIR / (f"precond_open_k{k}.npz" if h == NH else f"precond_open_k{k}_h{h}.npz")


def default_weights(wall=False):
    """The shipped network used by setPreconditioner("mlp"): for a wall
    handle the wall network when one is shipped; otherwise the widest open one
    present (48 neighbours, 512 hidden units, when shipped), else K = 16."""
    if wall:
        for k, h in ((48, 512), (48, 256), (32, 256), (16, NH)):
            if weights_path(k, h, True).exists():
                return weights_path(k, h, True)
    for k, h in ((48, 512), (32, 256), (16, NH)):
        if weights_path(k, h).exists():
            return weights_path(k, h)
    return weights_path(16)


DEFAULT_WEIGHTS = default_weights()
SYM = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]


# ---------------------------------------------------------------------------
# data
# ---------------------------------------------------------------------------
def rpy_uf_blocks(r):
    """Open-boundary RPY translational blocks M_ij(r) for r = r_i - r_j in
    units of a, with t0 = 1 (solvers/NBody/extra/hydrodynamicKernels.cuh:41-57,
    143-150).  r: (..., 3) -> (..., 3, 3)."""
    d = np.linalg.norm(r, axis=-1)
    ds = np.maximum(d, 1e-12)
    far = d >= 2.0
    f = np.where(far, 0.75 / ds + 0.5 / ds ** 3, 1.0 - 0.28125 * d)
    g = np.where(far, (0.75 - 1.5 / ds ** 2) / ds ** 3, np.where(d > 0, 0.09375 / ds, 0.0))
    eye = np.eye(3)
    return f[..., None, None] * eye + g[..., None, None] * r[..., :, None] * r[..., None, :]


def wall_uf_matrix(P):
    """Translational mobility of particles P (B, n, 3) above a bottom wall at
    z = 0 (units of a, t0 = 1): (B, 3n, 3n).  As the reference's
    BottomWall::dotProduct_UF (solvers/NBody/extra/hydrodynamicKernels.cuh:
    362-400): heights clamped at a, every block damped by b_i b_j with
    b = clamp(z, 0, 1); pair blocks are the open RPY block plus the Swan-Brady
    image of wallCorrection_UF (:203-247) for R = r_i - r_j + 2 h_j z; self
    blocks the identity plus the self image (:190-202)."""
    z = P[..., 2]
    b = np.clip(z, 0.0, 1.0)
    h = np.maximum(z, 1.0)
    Pc = P.copy()
    Pc[..., 2] = h
    d = Pc[:, :, None, :] - Pc[:, None, :, :]          # r_i - r_j
    M = rpy_uf_blocks(d)                                # B, n, n, 3, 3
    R = d.copy()
    R[..., 2] = h[:, :, None] + h[:, None, :]
    Rn = np.linalg.norm(R, axis=-1)
    iR = 1.0 / Rn
    e = R * iR[..., None]
    ez = e[..., 2]
    hh = h[:, None, :] / R[..., 2]                      # h_j / R_z
    iR3, iR5 = iR ** 3, iR ** 5
    ez2 = ez * ez
    h1 = hh * (1.0 - hh)
    A = -0.25 * (3 * (1 + 2 * h1 * ez2) * iR + 2 * (1 - 3 * ez2) * iR3
                 - 2 * (1 - 5 * ez2) * iR5)
    B = -0.25 * (3 * (1 - 6 * h1 * ez2) * iR - 6 * (1 - 5 * ez2) * iR3
                 + 10 * (1 - 7 * ez2) * iR5)
    C = 0.5 * ez * (3 * hh * (1 - 6 * (1 - hh) * ez2) * iR - 6 * (1 - 5 * ez2) * iR3
                    + 10 * (2 - 7 * ez2) * iR5)
    D = 0.5 * ez * (3 * hh * iR - 10 * iR5)
    E = -(3 * hh * hh * ez2 * iR + 3 * ez2 * iR3 + (2 - 15 * ez2) * iR5)
    zv = np.array([0.0, 0.0, 1.0])
    img = (A[..., None, None] * np.eye(3)
           + B[..., None, None] * e[..., :, None] * e[..., None, :]
           + C[..., None, None] * e[..., :, None] * zv[None, :]
           + D[..., None, None] * zv[:, None] * e[..., None, :]
           + E[..., None, None] * np.outer(zv, zv))
    n = P.shape[1]
    ih = 1.0 / h
    cxy = -(9 * ih - 2 * ih ** 3 + ih ** 5) / 16.0
    cz = -(9 * ih - 4 * ih ** 3 + ih ** 5) / 8.0
    diag = np.zeros(P.shape[:2] + (3, 3))
    diag[..., 0, 0] = cxy
    diag[..., 1, 1] = cxy
    diag[..., 2, 2] = cz
    ii = np.arange(n)
    img[:, ii, ii] = diag
    M = (M + img) * (b[:, :, None] * b[:, None, :])[..., None, None]
    return M.transpose(0, 1, 3, 2, 4).reshape(P.shape[0], 3 * n, 3 * n)


def random_system(rng, n, phi, clustered, sigma=4.0, max_rounds=5000, slab=None):
    """Positions (units of a) with no pair closer than 2a: points are drawn
    (uniform in a cube of volume fraction phi, from Gaussian clusters of
    ~128 particles with width sigma, or uniform in a slab above a wall when
    slab = (zlo, zhi) gives the range of heights), and every point that overlaps an
    accepted one is redrawn from its own distribution until it fits -- hard-
    sphere rejection, done in rounds over all rejected points at once.  The
    few points still rejected after 50 rounds are drawn 2 % wider every 50
    rounds (the core of a 128-particle cluster of width 4a is too dense for
    the last ones)."""
    from scipy.spatial import cKDTree
    L = (n * 4 * math.pi / 3 / phi) ** (1 / 3)
    widen = [1.0]  # the last few points of a dense cluster rarely fit at width sigma
    if slab is not None:  # above a wall: x, y uniform, heights uniform in slab
        zlo, zhi = slab
        L = math.sqrt(n * 4 * math.pi / 3 / phi / (zhi - zlo))

        def draw(idx):
            return np.column_stack([rng.uniform(0, L, len(idx)), rng.uniform(0, L, len(idx)),
                                    rng.uniform(zlo, zhi, len(idx))])
    elif clustered:
        ncl = max(1, n // 128)
        centres = rng.uniform(0, L, (ncl, 3))
        lab = rng.integers(0, ncl, n)

        def draw(idx):
            return centres[lab[idx]] + rng.normal(0, sigma * widen[0], (len(idx), 3))
    else:
        def draw(idx):
            return rng.uniform(0, L, (len(idx), 3))
    p = draw(np.arange(n))
    # first pass: drop one point of every overlapping pair
    pairs = cKDTree(p).query_pairs(2.0, output_type="ndarray")
    pending = np.unique(pairs[:, 1]) if len(pairs) else np.zeros(0, int)
    accepted = np.ones(n, bool)
    accepted[pending] = False
    tree = None
    recent = np.zeros((0, 3))  # accepted since the tree was built
    for rnd in range(max_rounds):
        if len(pending) == 0:
            break
        if rnd and rnd % 50 == 0:
            widen[0] *= 1.02
        if tree is None or len(recent) > 2048:
            tree = cKDTree(p[accepted])
            recent = np.zeros((0, 3))
        cand = draw(pending)
        hit = tree.query_ball_point(cand, 2.0, return_length=True, workers=-1) > 0
        if len(recent):
            hit |= cKDTree(recent).query_ball_point(cand, 2.0, return_length=True) > 0
        ok = ~hit
        # among the candidates that fit, keep one of each overlapping pair
        if ok.sum() > 1:
            sub = np.flatnonzero(ok)
            cp = cKDTree(cand[sub]).query_pairs(2.0, output_type="ndarray")
            if len(cp):
                ok[sub[np.unique(cp[:, 1])]] = False
        idx = pending[ok]
        p[idx] = cand[ok]
        accepted[idx] = True
        recent = np.concatenate([recent, cand[ok]])
        pending = pending[~ok]
    if len(pending):
        raise RuntimeError(f"could not place {len(pending)} particles without overlap")
    return p


def canonical_frames(rel):
    """rel: (B, K, 3) neighbours sorted by distance -> E (B, 3, 3), rows = axes
    (x to the nearest neighbour, y to the first non-collinear one)."""
    B = rel.shape[0]
    ex = rel[:, 0] / np.linalg.norm(rel[:, 0], axis=1, keepdims=True)
    ey = np.zeros_like(ex)
    done = np.zeros(B, bool)
    for n in range(1, rel.shape[1]):
        a = rel[:, n] - ex * np.sum(rel[:, n] * ex, axis=1, keepdims=True)
        nn = np.sum(a * a, axis=1)
        take = (~done) & (nn > 1e-12)
        ey[take] = a[take] / np.sqrt(nn[take])[:, None]
        done |= take
    ey[~done] = [0.0, 1.0, 0.0]
    ez = np.cross(ex, ey)
    return np.stack([ex, ey, ez], axis=1)


def wall_frames(rel):
    """rel: (B, K, 3) neighbours sorted by distance -> E (B, 3, 3), rows = axes
    turning about the wall normal only: x to the horizontal offset of the
    nearest neighbour that has one, z the wall normal."""
    hh = rel[..., 0] ** 2 + rel[..., 1] ** 2
    has = hh > 1e-12
    first = np.argmax(has, axis=1)
    ok = has[np.arange(len(rel)), first]
    hx = rel[np.arange(len(rel)), first, 0]
    hy = rel[np.arange(len(rel)), first, 1]
    ln = np.sqrt(np.where(ok, hh[np.arange(len(rel)), first], 1.0))
    c = np.where(ok, hx / ln, 1.0)
    s_ = np.where(ok, hy / ln, 0.0)
    E = np.zeros((len(rel), 3, 3))
    E[:, 0, 0], E[:, 0, 1] = c, s_
    E[:, 1, 0], E[:, 1, 1] = -s_, c
    E[:, 2, 2] = 1.0
    return E


def samples_from_wall_system(p, ids, K=16):
    """Features X (B, 3K + 1) and targets Y (B, 6 + 9K) for particles `ids` of
    a system above a bottom wall at z = 0 (samples whose neighbourhood
    mobility is not positive definite are dropped)."""
    from scipy.spatial import cKDTree
    _, nb = cKDTree(p).query(p[ids], K + 1)
    rel = p[nb[:, 1:]] - p[ids][:, None, :]
    E = wall_frames(rel)
    X = np.concatenate([np.einsum("bnk,bck->bnc", rel, E).reshape(len(ids), -1),
                        np.maximum(p[ids, 2], 1.0)[:, None]], 1)
    Mp = wall_uf_matrix(p[nb])
    lam, Q = np.linalg.eigh(Mp)
    good = lam[:, 0] > 1e-8
    lam, Q, E, X = lam[good], Q[good], E[good], X[good]
    B = int(good.sum())
    row = np.einsum("bij,bj,bkj->bik", Q[:, :3, :], 1.0 / np.sqrt(lam), Q)
    rb = row.reshape(B, 3, K + 1, 3).transpose(0, 2, 1, 3)
    rc = np.einsum("bij,bnjk,blk->bnil", E, rb, E)
    Y = np.concatenate([np.stack([rc[:, 0, i, j] for i, j in SYM], 1),
                        rc[:, 1:].reshape(B, -1)], 1)
    return X.astype(np.float32), Y.astype(np.float32)


def samples_from_system(p, ids, K=16):
    """Features X (B, 3K) and targets Y (B, 6 + 9K) for particles `ids` of p."""
    from scipy.spatial import cKDTree
    _, nb = cKDTree(p).query(p[ids], K + 1)
    rel = p[nb[:, 1:]] - p[ids][:, None, :]
    E = canonical_frames(rel)
    X = np.einsum("bnk,bck->bnc", rel, E).reshape(len(ids), -1)
    P = p[nb]                                                   # B, K+1, 3
    blocks = rpy_uf_blocks(P[:, :, None, :] - P[:, None, :, :])  # B,K+1,K+1,3,3
    Mp = blocks.transpose(0, 1, 3, 2, 4).reshape(len(ids), 3 * (K + 1), 3 * (K + 1))
    lam, Q = np.linalg.eigh(Mp)
    row = np.einsum("bij,bj,bkj->bik", Q[:, :3, :], 1.0 / np.sqrt(lam), Q)  # B,3,3(K+1)
    rb = row.reshape(len(ids), 3, K + 1, 3).transpose(0, 2, 1, 3)         # B,K+1,3,3
    rc = np.einsum("bij,bnjk,blk->bnil", E, rb, E)                         # canonical frame
    Y = np.concatenate([np.stack([rc[:, 0, i, j] for i, j in SYM], 1),
                        rc[:, 1:].reshape(len(ids), -1)], 1)
    return X.astype(np.float32), Y.astype(np.float32)


def _make_chunk(args):
    seed, nsys, per_sys, k, wall = args
    rng = np.random.default_rng(seed)
    Xs, Ys = [], []
    for _ in range(nsys):
        if wall:
            n = int(rng.integers(max(128, k + 1), 1025))
            phi = float(np.exp(rng.uniform(np.log(0.01), np.log(0.2))))
            slab = (1.0 if rng.random() < 0.3 else 1.5, float(rng.uniform(8.0, 60.0)))
            p = random_system(rng, n, phi, False, slab=slab)
            ids = rng.choice(n, min(n, per_sys), replace=False)
            X, Y = samples_from_wall_system(p, ids, k)
        else:
            n = int(rng.integers(max(64, k + 1), 513))  # every particle has k neighbours
            phi = float(rng.uniform(0.05, 0.3))
            p = random_system(rng, n, phi, rng.random() < 0.5)
            ids = rng.choice(n, min(n, per_sys), replace=False)
            X, Y = samples_from_system(p, ids, k)
        Xs.append(X)
        Ys.append(Y)
    return np.concatenate(Xs), np.concatenate(Ys)


def make_dataset(systems, per_sys=32, seed=0, workers=None, log=None, k=16, wall=False):
    workers = workers or max(1, (os.cpu_count() or 1))
    # one BLAS thread per worker: the pool already uses every core
    for var in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[var] = "1"
    chunk = max(1, systems // (4 * workers))
    jobs = []
    s = 0
    while s < systems:
        jobs.append((seed * 1000003 + len(jobs), min(chunk, systems - s), per_sys, k, wall))
        s += chunk
    ctx = mp.get_context("spawn")
    parts = []
    t0 = time.time()
    with ctx.Pool(workers) as pool:
        for k, part in enumerate(pool.imap_unordered(_make_chunk, jobs)):
            parts.append(part)
            if log and (k + 1) % max(1, len(jobs) // 10) == 0:
                log(f"  dataset {k + 1}/{len(jobs)} chunks, {time.time() - t0:.1f}s")
    return np.concatenate([a for a, _ in parts]), np.concatenate([b for _, b in parts])


# ---------------------------------------------------------------------------
# parameters
# ---------------------------------------------------------------------------
def layout(k, h=NH, wall=False):
    """Parameter layout for k neighbours and h hidden units (one more input,
    the height, for a wall network), as csrc/precond.cuh (PrecLayout)."""
    nin, nout = 3 * k + (1 if wall else 0), 6 + 9 * k
    return [("W1", (nin, h)), ("b1", (h,)), ("W2", (h, h)), ("b2", (h,)),
            ("W3", (h, nout)), ("b3", (nout,)), ("xmean", (nin,)), ("xstd", (nin,)),
            ("ymean", (nout,)), ("ystd", (nout,))]


def ntrain(k, h=NH, wall=False):
    """Length of the trainable prefix (weights and biases)."""
    nin, nout = 3 * k + (1 if wall else 0), 6 + 9 * k
    return nin * h + h + h * h + h + h * nout + nout


def kind_of_params(n):
    """(k, h, wall) of a flat parameter vector of length n."""
    for wall in (False, True):
        for k in (16, 32, 48, 64):
            for h in (64, 128, 256, 512, 1024):
                if n == sum(int(np.prod(s)) for _, s in layout(k, h, wall)):
                    return k, h, wall
    raise ValueError(f"{n} is not the parameter count of a K = 16, 32, 48 or 64 network "
                     "with 64, 128, 256, 512 or 1024 hidden units")


def shape_of_params(n):
    """(k, h) of a flat parameter vector of length n."""
    return kind_of_params(n)[:2]


LAYOUT = layout(16)


def flat_params(d):
    return np.concatenate([np.asarray(d[name], np.float32).ravel() for name, _ in LAYOUT])


def load_weights(path=None, wall=False):
    """Flat FP32 parameter vector in the layout of csrc/precond.cuh (the
    default network for the geometry when no path is given)."""
    path = Path(path) if path else default_weights(wall)
    if not path.exists():
        raise FileNotFoundError(f"preconditioner weights {path} not found")
    z = np.load(path)
    return flat_params(z)


# ---------------------------------------------------------------------------
# training on the GPU with this project's kernels
# ---------------------------------------------------------------------------
class GpuMLP:
    def __init__(self, lib, torch, params, stream):
        self.lib, self.torch, self.s = lib, torch, stream
        self.k, self.h, self.wall = kind_of_params(len(params))
        self.nin, self.nout = 3 * self.k + (1 if self.wall else 0), 6 + 9 * self.k
        self.ntrain = ntrain(self.k, self.h, self.wall)
        self.p = torch.tensor(params, device="cuda")
        self.g = torch.zeros(self.ntrain, device="cuda")
        self.m = torch.zeros(self.ntrain, device="cuda")
        self.v = torch.zeros(self.ntrain, device="cuda")
        self.loss = torch.zeros(1, dtype=torch.float64, device="cuda")
        off = 0
        self.view = {}
        self.gview = {}
        for name, shp in layout(self.k, self.h, self.wall):
            n = int(np.prod(shp))
            self.view[name] = self.p[off:off + n]
            if off < self.ntrain:
                self.gview[name] = self.g[off:off + n]
            off += n

    def _ptr(self, t):
        return ctypes.c_void_p(t.data_ptr())

    def gemm(self, ta, tb, M, N, K_, A, lda, B, ldb, C, ldc, bias=None, act=0, beta=0.0):
        rc = self.lib.lmg_internal_gemm(int(ta), int(tb), M, N, K_, self._ptr(A), lda,
                                        self._ptr(B), ldb, self._ptr(C), ldc,
                                        self._ptr(bias) if bias is not None else None, act,
                                        ctypes.c_float(beta), self.s)
        assert rc == 0, rc

    def forward(self, X, H1, H2, Yp):
        B = X.shape[0]
        v = self.view
        NIN, NOUT, NH = self.nin, self.nout, self.h
        self.gemm(0, 0, B, NH, NIN, X, NIN, v["W1"], NH, H1, NH, v["b1"], 1)
        self.gemm(0, 0, B, NH, NH, H1, NH, v["W2"], NH, H2, NH, v["b2"], 1)
        self.gemm(0, 0, B, NOUT, NH, H2, NH, v["W3"], NOUT, Yp, NOUT, v["b3"], 0)

    def backward(self, X, H1, H2, Yp, T, dY, dH2, dH1):
        B = X.shape[0]
        v, g, lib = self.view, self.gview, self.lib
        NIN, NOUT, NH = self.nin, self.nout, self.h
        scale = ctypes.c_float(2.0 / (B * NOUT))
        assert lib.lmg_internal_mse_grad(ctypes.c_size_t(B * NOUT), self._ptr(Yp), self._ptr(T),
                                         self._ptr(dY), scale, self._ptr(self.loss), self.s) == 0
        self.gemm(1, 0, NH, NOUT, B, H2, NH, dY, NOUT, g["W3"], NOUT)         # dW3 = H2^T dY
        assert lib.lmg_internal_colsum(B, NOUT, self._ptr(dY), self._ptr(g["b3"]), self.s) == 0
        self.gemm(0, 1, B, NH, NOUT, dY, NOUT, v["W3"], NOUT, dH2, NH)       # dH2 = dY W3^T
        assert lib.lmg_internal_tanh_backward(ctypes.c_size_t(B * NH), self._ptr(H2),
                                              self._ptr(dH2), self.s) == 0
        self.gemm(1, 0, NH, NH, B, H1, NH, dH2, NH, g["W2"], NH)             # dW2 = H1^T dH2
        assert lib.lmg_internal_colsum(B, NH, self._ptr(dH2), self._ptr(g["b2"]), self.s) == 0
        self.gemm(0, 1, B, NH, NH, dH2, NH, v["W2"], NH, dH1, NH)            # dH1 = dH2 W2^T
        assert lib.lmg_internal_tanh_backward(ctypes.c_size_t(B * NH), self._ptr(H1),
                                              self._ptr(dH1), self.s) == 0
        self.gemm(1, 0, NIN, NH, B, X, NIN, dH1, NH, g["W1"], NH)            # dW1 = X^T dH1
        assert lib.lmg_internal_colsum(B, NH, self._ptr(dH1), self._ptr(g["b1"]), self.s) == 0

    def adam(self, lr, step):
        assert self.lib.lmg_internal_adam(ctypes.c_size_t(self.ntrain), self._ptr(self.p),
                                          self._ptr(self.g), self._ptr(self.m), self._ptr(self.v),
                                          ctypes.c_float(lr), ctypes.c_float(0.9),
                                          ctypes.c_float(0.999), ctypes.c_float(1e-8), step,
                                          self.s) == 0


def init_params(X, Y, seed=0, NH=NH):
    rng = np.random.default_rng(seed)
    NIN, NOUT = X.shape[1], Y.shape[1]
    d = {}
    d["W1"] = rng.normal(0, 1 / math.sqrt(NIN), (NIN, NH))
    d["b1"] = np.zeros(NH)
    d["W2"] = rng.normal(0, 1 / math.sqrt(NH), (NH, NH))
    d["b2"] = np.zeros(NH)
    d["W3"] = rng.normal(0, 1 / math.sqrt(NH), (NH, NOUT))
    d["b3"] = np.zeros(NOUT)
    d["xmean"], d["xstd"] = X.mean(0), X.std(0) + 1e-6
    d["ymean"], d["ystd"] = Y.mean(0), Y.std(0) + 1e-6
    return d


def train(X, Y, epochs=60, batch=4096, lr=2e-3, seed=0, log=print, val_frac=0.05, hidden=NH):
    import torch
    from . import _capi
    lib = _capi.load()
    NH = hidden
    d = init_params(X, Y, seed, NH)
    k = X.shape[1] // 3
    wall = X.shape[1] % 3 == 1
    NIN, NOUT = 3 * k + (1 if wall else 0), 6 + 9 * k
    params = np.concatenate([np.asarray(d[name], np.float32).ravel()
                             for name, _ in layout(k, NH, wall)])
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    net = GpuMLP(lib, torch, params, stream)
    xm, xs = d["xmean"].astype(np.float32), d["xstd"].astype(np.float32)
    ym, ys = d["ymean"].astype(np.float32), d["ystd"].astype(np.float32)
    Xn = torch.tensor((X - xm) / xs, device="cuda")
    Yn = torch.tensor((Y - ym) / ys, device="cuda")
    n = Xn.shape[0]
    nval = max(1, int(val_frac * n))
    g = torch.Generator(device="cpu").manual_seed(seed)
    perm = torch.randperm(n, generator=g).cuda()
    Xv, Yv = Xn[perm[:nval]], Yn[perm[:nval]]
    Xt, Yt = Xn[perm[nval:]], Yn[perm[nval:]]
    ntr = Xt.shape[0]
    H1 = torch.empty(batch, NH, device="cuda")
    H2 = torch.empty_like(H1)
    Yp = torch.empty(batch, NOUT, device="cuda")
    dY = torch.empty_like(Yp)
    dH1 = torch.empty_like(H1)
    dH2 = torch.empty_like(H1)
    step = 0
    hist = []
    t0 = time.time()
    for ep in range(epochs):
        order = torch.randperm(ntr, generator=g).cuda()
        cur_lr = lr * (0.5 * (1 + math.cos(math.pi * ep / epochs)))
        net.loss.zero_()
        for b0 in range(0, ntr - batch + 1, batch):
            idx = order[b0:b0 + batch]
            xb = Xt[idx].contiguous()
            tb = Yt[idx].contiguous()
            net.forward(xb, H1, H2, Yp)
            net.backward(xb, H1, H2, Yp, tb, dY, dH2, dH1)
            step += 1
            net.adam(cur_lr, step)
        train_mse = float(net.loss.item()) / ((ntr // batch) * batch * NOUT)
        val = evaluate(net, Xv, Yv, batch, torch)
        hist.append((ep, train_mse, val))
        if ep % 5 == 0 or ep == epochs - 1:
            log(f"epoch {ep:3d} train mse {train_mse:.4f} val mse {val:.4f} ({time.time()-t0:.1f}s)")
    out = {name: net.view[name].detach().cpu().numpy().reshape(shp)
           for name, shp in layout(k, NH, wall)}
    out["xmean"], out["xstd"], out["ymean"], out["ystd"] = xm, xs, ym, ys
    return out, hist


def evaluate(net, Xv, Yv, batch, torch):
    tot = 0.0
    for b0 in range(0, Xv.shape[0], batch):
        xb = Xv[b0:b0 + batch].contiguous()
        B = xb.shape[0]
        H1 = torch.empty(B, net.h, device="cuda")
        H2 = torch.empty_like(H1)
        Yp = torch.empty(B, net.nout, device="cuda")
        net.forward(xb, H1, H2, Yp)
        tot += float(((Yp - Yv[b0:b0 + B]) ** 2).sum())
    return tot / (Xv.shape[0] * net.nout)


def main():
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd")
    t = sub.add_parser("train")
    t.add_argument("--k", type=int, default=16, choices=[16, 32, 48, 64])
    t.add_argument("--hidden", type=int, default=NH, choices=[64, 128, 256, 512, 1024])
    t.add_argument("--systems", type=int, default=20000)
    t.add_argument("--per-system", type=int, default=32)
    t.add_argument("--epochs", type=int, default=60)
    t.add_argument("--out", default=None)
    t.add_argument("--seed", type=int, default=0)
    t.add_argument("--wall", action="store_true",
                   help="train for a single bottom wall (slabs above it, height input)")
    a = ap.parse_args()
    if a.cmd == "train":
        t0 = time.time()
        X, Y = make_dataset(a.systems, a.per_system, a.seed,
                            log=lambda m: print(m, flush=True), k=a.k, wall=a.wall)
        print(f"dataset {X.shape} {Y.shape} in {time.time()-t0:.1f}s", flush=True)
        w, hist = train(X, Y, epochs=a.epochs, seed=a.seed, hidden=a.hidden)
        out = a.out or str(weights_path(a.k, a.hidden, a.wall))
        Path(out).parent.mkdir(parents=True, exist_ok=True)
        np.savez(out, **w, history=np.array(hist),
                 info=np.array(json.dumps({"systems": a.systems, "per_system": a.per_system,
                                           "epochs": a.epochs, "samples": int(X.shape[0]),
                                           "k": a.k, "hidden": a.hidden,
                                           "wall": a.wall})))
        print("saved", out)


if __name__ == "__main__":
    main()
