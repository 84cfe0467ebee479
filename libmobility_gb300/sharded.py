"""Row-partitioned sqrtMdotW: one system's Lanczos solve spread over the
ranks of a torch.distributed process group.

The reference solves on one device: lanczos::Solver::run
(include/lanczos/LanczosAlgorithm.cu:173-232) calls the whole Mdot once per
iteration and keeps every Krylov vector whole.  Here rank r owns the
particles [b_r, e_r) of a contiguous partition (``row_partition``): it keeps
only those rows of every Krylov vector, and per iteration

  * gathers the current Krylov vector from all ranks (one all-gather: the
    all-pairs product needs every source),
  * computes its rows of M v (``NBodyRows``: lmg_mdot_rows on its own GPU,
    the positions of all N particles set on every rank's handle),
  * and combines the two inner products of the recurrence with FP64
    all-reduces.

Every rank then holds the same tridiagonal matrix, takes the same square
root on the host and the same decisions (breakdown, convergence), so the
ranks stay in lockstep without further messages.  The recurrence, the
breakdown rule (LanczosAlgorithm.cu:120-153), the estimate
(LanczosAlgorithm.cu:158-167), the error (LanczosAlgorithm.cu:202-222) and
the adaptive check schedule (LanczosAlgorithm.h:266-284,
LanczosAlgorithm.cu:224-232) are the reference's; the Krylov scalars are FP64
as in the single-GPU solver.

Vectors follow the reference's layout [linear; angular] (3N values each,
angular only with includeAngular); a rank's local piece is
[linear rows; angular rows] of its particles.
"""
import math

import numpy as np
import torch
import torch.distributed as dist


def row_partition(N, world_size):
    """Contiguous particle ranges as equal as possible: rank r owns
    [b_r, e_r).  Every row sums over all sources of its batch, so equal rows
    are equal work."""
    if world_size < 1 or N < world_size:
        raise RuntimeError("[libmobility_gb300] every rank needs at least one particle")
    base, rem = divmod(int(N), int(world_size))
    out, b = [], 0
    for r in range(world_size):
        e = b + base + (1 if r < rem else 0)
        out.append((b, e))
        b = e
    return out


def _tridiag_sqrt_e1(hdiag, hsup):
    """T^{1/2} e1 of the m x m symmetric tridiagonal matrix (diagonal hdiag,
    off-diagonal hsup[:m-1]) through its eigen-decomposition, FP64
    (KrylovSubspace::computeSquareRoot, LanczosAlgorithm.cu:48-85)."""
    m = len(hdiag)
    T = np.diag(np.asarray(hdiag, np.float64))
    if m > 1:
        off = np.asarray(hsup[: m - 1], np.float64)
        T += np.diag(off, 1) + np.diag(off, -1)
    lam, P = np.linalg.eigh(T)
    with np.errstate(invalid="ignore"):
        s = np.sqrt(lam) * P[0, :]
    return P @ s


class ShardedLanczos:
    """The Lanczos solver of one rank.  Keeps the adaptive check interval
    across calls as lanczos::Solver does; every rank must make the same
    calls in the same order."""

    def __init__(self, N, include_angular=False, group=None, hard_limit=200,
                 dtype=torch.float32, device="cpu"):
        self.N = int(N)
        self.include_angular = bool(include_angular)
        self.group = group
        if dist.is_available() and dist.is_initialized():
            self.world_size = dist.get_world_size(group)
            self.rank = dist.get_rank(group)
            self._host_comm = dist.get_backend(group) == "gloo"
        else:
            self.world_size, self.rank, self._host_comm = 1, 0, False
        self.rows = row_partition(self.N, self.world_size)
        self.row_begin, self.row_end = self.rows[self.rank]
        self.ncomp = 2 if self.include_angular else 1
        self.counts = [3 * (e - b) for b, e in self.rows]  # values per component
        self.n_local = self.ncomp * self.counts[self.rank]
        self.hard_limit = int(hard_limit)
        self.dtype = dtype
        self.device = torch.device(device)
        self.check_convergence_steps = 3
        self._pad = self.ncomp * max(self.counts)
        self._send = torch.zeros(self._pad, dtype=dtype, device=self.device)
        self._recv = [torch.zeros(self._pad, dtype=dtype, device=self.device)
                      for _ in range(self.world_size)]
        self._full = torch.zeros(self.ncomp * 3 * self.N, dtype=dtype, device=self.device)

    # -- collectives -------------------------------------------------------
    def _allreduce(self, x):
        """Sum of an FP64 tensor over the ranks (on the host for gloo)."""
        if self.world_size == 1:
            return x
        if self._host_comm and x.is_cuda:
            h = x.cpu()
            dist.all_reduce(h, group=self.group)
            return h.to(x.device)
        dist.all_reduce(x, group=self.group)
        return x

    def _dots(self, *pairs):
        """Global inner products sum_ranks a.b in FP64, one all-reduce."""
        v = torch.stack([torch.dot(a.double(), b.double()) for a, b in pairs])
        return self._allreduce(v).cpu().numpy()

    def local_rows(self, full):
        """This rank's piece of a whole vector [linear; angular]."""
        full = torch.as_tensor(full).reshape(-1)
        b, e = 3 * self.row_begin, 3 * self.row_end
        parts = [full[c * 3 * self.N + b: c * 3 * self.N + e] for c in range(self.ncomp)]
        return torch.cat(parts).to(device=self.device, dtype=self.dtype)

    def gather(self, local):
        """The whole vector [linear; angular] from every rank's piece."""
        n = self.counts[self.rank]
        if self.world_size == 1:
            self._full.copy_(local)
            return self._full
        self._send[: self.ncomp * n].copy_(local)
        if self._host_comm and self._send.is_cuda:
            send = self._send.cpu()
            recv = [torch.empty_like(send) for _ in range(self.world_size)]
            dist.all_gather(recv, send, group=self.group)
            recv = [t.to(self.device) for t in recv]
        else:
            dist.all_gather(self._recv, self._send, group=self.group)
            recv = self._recv
        off = 0
        for c in range(self.ncomp):
            for r, cnt in enumerate(self.counts):
                self._full[off: off + cnt].copy_(recv[r][c * cnt: (c + 1) * cnt])
                off += cnt
        return self._full

    def gather_positions(self, pos_local):
        """All N positions (N, 3) from every rank's own particles (its rows,
        shape (e_r - b_r, 3)): the all-gather a rank does once per
        setPositions when it holds only its own particles."""
        pos_local = torch.as_tensor(pos_local).reshape(-1, 3)
        n_r = self.row_end - self.row_begin
        if pos_local.shape[0] != n_r:
            raise RuntimeError("[libmobility_gb300] local positions must hold this rank's rows")
        if self.world_size == 1:
            return pos_local.clone()
        pad = max(e - b for b, e in self.rows)
        send = torch.zeros((pad, 3), dtype=pos_local.dtype, device=pos_local.device)
        send[:n_r] = pos_local
        host = self._host_comm and send.is_cuda
        if host:
            send = send.cpu()
        recv = [torch.empty_like(send) for _ in range(self.world_size)]
        dist.all_gather(recv, send, group=self.group)
        out = torch.cat([recv[r][: e - b] for r, (b, e) in enumerate(self.rows)])
        return out.to(pos_local.device) if host else out

    # -- the solve ---------------------------------------------------------
    def _register(self, steps):  # LanczosAlgorithm.cu:224-232
        if steps - 2 > self.check_convergence_steps:
            self.check_convergence_steps += 1
        else:
            self.check_convergence_steps = max(1, self.check_convergence_steps - 2)

    def run(self, matvec, z_local, tol, callback=None):
        """y = M^{1/2} z, rows of this rank; returns (y_local, iterations).

        matvec(v_whole) returns this rank's rows of M v (length n_local);
        z_local is this rank's piece of z."""
        dt, dev = self.dtype, self.device
        n = self.n_local
        z = torch.as_tensor(z_local).reshape(-1).to(device=dev, dtype=dt)
        if z.numel() != n:
            raise RuntimeError("[libmobility_gb300] the local noise vector has the wrong size")
        m_max = self.hard_limit
        V = torch.zeros((m_max + 1, n), dtype=dt, device=dev)
        hdiag = np.zeros(m_max + 1)
        hsup = np.zeros(m_max + 1)
        normz = math.sqrt(self._dots((z, z))[0])
        V[0] = z * (1.0 / normz)
        old = torch.zeros(n, dtype=dt, device=dev)
        k = min(self.check_convergence_steps, m_max - 2)
        for i in range(m_max):
            # KrylovSubspace::nextIteration, LanczosAlgorithm.cu:120-153
            w = torch.as_tensor(matvec(self.gather(V[i]))).reshape(-1).to(dtype=dt).clone()
            if i > 0:
                w -= hsup[i - 1] * V[i - 1]
            hdiag[i] = self._dots((w, V[i]))[0]
            w -= hdiag[i] * V[i]
            hsup[i] = math.sqrt(self._dots((w, w))[0])
            if hsup[i] < 1e-3 * hdiag[i] / normz:
                hsup[i] = 0.0
            if hsup[i] > 0:
                V[i + 1] = w * (1.0 / hsup[i])
            else:  # breakdown: the next vector is e_0, owned by rank 0
                V[i + 1].zero_()
                if self.rank == 0:
                    V[i + 1, 0] = 1
            if i >= k or callback is not None:
                # computeCurrentResultEstimation, LanczosAlgorithm.cu:158-167
                m = i + 1
                c = torch.as_tensor(_tridiag_sqrt_e1(hdiag[:m], hsup[:m]), dtype=dt, device=dev)
                y = normz * (V[:m].T @ c)
                if i > 0:
                    # computeError, LanczosAlgorithm.cu:202-222
                    d = old - y
                    pp, dd = self._dots((old, old), (d, d))
                    prev, diff = math.sqrt(pp), math.sqrt(dd)
                    if prev != 0:
                        err = abs(diff / prev)
                    else:
                        err = math.inf if diff > 0 else math.nan
                    if math.isnan(err):
                        raise RuntimeError("[Lanczos] Unknown error (found NaN in result guess)")
                    if callback is not None:
                        callback(i, float(err))
                    if err <= tol:
                        self._register(i)
                        return y, i
                old = y
        raise RuntimeError("[Lanczos] Could not converge")


class NBodyRows:
    """The matrix-vector product of one rank: its rows of M v through
    lmg_mdot_rows on an NBody handle whose positions hold all N particles
    (torch tensors on the handle's GPU)."""

    def __init__(self, solver, lanczos):
        self.solver = solver
        self.lz = lanczos

    def __call__(self, v):
        N, lz = self.lz.N, self.lz
        F = v[: 3 * N]
        T = v[3 * N:] if lz.include_angular else None
        U, W = self.solver.Mdot_rows(lz.row_begin, lz.row_end, F, T)
        if lz.include_angular:
            return torch.cat([U.reshape(-1), W.reshape(-1)])
        return U.reshape(-1)


def sqrt_mdot_w_rows(solver, lanczos, dW_local, tol, prefactor=1.0):
    """prefactor * M^{1/2} dW, rows of this rank: (linear (n_r, 3),
    angular (n_r, 3) or None, iterations).  dW_local is this rank's piece of
    the Gaussian vector [dW_F; dW_T] (``ShardedLanczos.local_rows``)."""
    y, it = lanczos.run(NBodyRows(solver, lanczos), dW_local, tol)
    y = y * prefactor
    n = lanczos.counts[lanczos.rank]
    lin = y[:n].reshape(-1, 3)
    ang = y[n:].reshape(-1, 3) if lanczos.include_angular else None
    return lin, ang, it
