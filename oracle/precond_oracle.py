"""NumPy restatement of the learned preconditioner's pieces, for tests
(TEST INFRASTRUCTURE ONLY; the product never imports it).

Written independently of libmobility_gb300/precond.py: neighbour lists from
scipy's k-d tree, the canonical frame, the MLP forward and backward passes
(48 -> 64 tanh -> 64 tanh -> 150) and the sparse P blocks in the lab frame.
"""
import numpy as np

K = 16
NH = 64


def shapes(k=K, h=NH, wall=False):
    """Parameter layout of the network for k neighbours and h hidden units
    (3k -> h -> h -> 6 + 9k; one more input, the height, above a wall)."""
    nin, nout = 3 * k + (1 if wall else 0), 6 + 9 * k
    return [("W1", (nin, h)), ("b1", (h,)), ("W2", (h, h)), ("b2", (h,)),
            ("W3", (h, nout)), ("b3", (nout,)), ("xmean", (nin,)), ("xstd", (nin,)),
            ("ymean", (nout,)), ("ystd", (nout,))]


SHAPES = shapes(K)
NIN, NOUT = 3 * K, 6 + 9 * K


def khw_of(flat):
    """(neighbours, hidden units, wall) of a flat parameter vector."""
    for wall in (False, True):
        for k in (16, 32, 48, 64):
            for h in (64, 128, 256, 512, 1024):
                if len(flat) == sum(int(np.prod(s)) for _, s in shapes(k, h, wall)):
                    return k, h, wall
    raise ValueError("not a preconditioner parameter vector")


def kh_of(flat):
    """(neighbours, hidden units) of a flat parameter vector."""
    return khw_of(flat)[:2]


def k_of(flat):
    return kh_of(flat)[0]


def unpack(flat):
    out, o = {}, 0
    for k, shp in shapes(*khw_of(flat)):
        n = int(np.prod(shp))
        out[k] = np.asarray(flat[o:o + n], np.float64).reshape(shp)
        o += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], np.float32).ravel() for name, _ in SHAPES])


def neighbours(pos, k=K):
    from scipy.spatial import cKDTree
    d, nb = cKDTree(pos).query(pos, k + 1)
    return nb, d


def frame(rel):
    """Rows: x to rel[0], y to the first rel[n] not collinear with it."""
    x = rel[0] / np.linalg.norm(rel[0])
    y = np.array([0.0, 1.0, 0.0])
    for n in range(1, len(rel)):
        a = rel[n] - x * (rel[n] @ x)
        if a @ a > 1e-12:
            y = a / np.linalg.norm(a)
            break
    return np.stack([x, y, np.cross(x, y)])


def wall_frame(rel):
    """Rows: x to the horizontal offset of the first neighbour that has one,
    y = z cross x, z the wall normal."""
    for r in rel:
        hh = r[0] ** 2 + r[1] ** 2
        if hh > 1e-12:
            c, s_ = r[0] / np.sqrt(hh), r[1] / np.sqrt(hh)
            break
    else:
        c, s_ = 1.0, 0.0
    return np.array([[c, s_, 0.0], [-s_, c, 0.0], [0.0, 0.0, 1.0]])


def forward(d, X):
    """Returns (H1, H2, Ynorm) for normalised inputs X (B, 48)."""
    H1 = np.tanh(X @ d["W1"] + d["b1"])
    H2 = np.tanh(H1 @ d["W2"] + d["b2"])
    return H1, H2, H2 @ d["W3"] + d["b3"]


def backward(d, X, H1, H2, Y, T):
    """Gradients of mean((Y - T)^2) with respect to W1..b3."""
    B = X.shape[0]
    dY = 2.0 * (Y - T) / (B * Y.shape[1])
    g = {"W3": H2.T @ dY, "b3": dY.sum(0)}
    dH2 = (dY @ d["W3"].T) * (1 - H2 ** 2)
    g["W2"], g["b2"] = H1.T @ dH2, dH2.sum(0)
    dH1 = (dH2 @ d["W2"].T) * (1 - H1 ** 2)
    g["W1"], g["b1"] = X.T @ dH1, dH1.sum(0)
    return g


def p_blocks(pos, flat, a=1.0, scale=1.0):
    """Lab-frame blocks (N, K+1, 3, 3) and neighbour lists (N, K+1); a wall
    network (3K + 1 inputs) takes its frame about the wall normal and the
    height max(z, a)/a as its last input."""
    d = unpack(flat)
    K, _, wall = khw_of(flat)
    nb, _ = neighbours(pos, K)
    N = pos.shape[0]
    out = np.zeros((N, K + 1, 3, 3))
    for i in range(N):
        rel = (pos[nb[i, 1:]] - pos[i]) / a
        E = wall_frame(rel) if wall else frame(rel)
        feat = (rel @ E.T).ravel()
        if wall:
            feat = np.append(feat, max(pos[i, 2] / a, 1.0))
        x = (feat - d["xmean"]) / d["xstd"]
        _, _, y = forward(d, x[None, :])
        y = y[0] * d["ystd"] + d["ymean"]
        b = [np.array([[y[0], y[1], y[2]], [y[1], y[3], y[4]], [y[2], y[4], y[5]]])]
        b += list(y[6:].reshape(K, 3, 3))
        for n in range(K + 1):
            out[i, n] = E.T @ b[n] @ E * scale
    return out, nb


def dense_p(blocks, nb):
    N = blocks.shape[0]
    P = np.zeros((3 * N, 3 * N))
    for i in range(N):
        for n in range(nb.shape[1]):
            j = nb[i, n]
            P[3 * i:3 * i + 3, 3 * j:3 * j + 3] += blocks[i, n]
    return P


def identity_params(k=K):
    """A network whose output is the identity self block and zero neighbour
    blocks for every input (all weights zero, output mean = identity)."""
    d = {name: np.zeros(shp) for name, shp in shapes(k)}
    d["xstd"][:] = 1.0
    d["ystd"][:] = 1.0
    d["ymean"][[0, 3, 5]] = 1.0
    return pack(d)
