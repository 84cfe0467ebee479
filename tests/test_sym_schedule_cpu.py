"""Host tables of the symmetric open-space kernel (no GPU needed).

The library's own planner (lmg_internal_sym_plan) builds the warp schedule,
the per-pair slot places and the per-tile slot ranges; these tests walk the
tables the way the kernel does and check that
  * every rotation step of every tile pair is taken by exactly one warp, and
    the warps' step counts differ by at most one;
  * every partial slot is written at most once, by a warp whose sums belong
    to the tile owning the slot's range (every tile owns the same number of
    slots; those never written stay zero, so the fold reads whole ranges);
  * on small systems, the rotation steps the kernel takes from these tables
    (slot l against slot l + k mod 32, the diagonal tile's own slots and
    distance-16 slot pairs) cover every unordered particle pair of each batch
    exactly once, the self pairs included.
"""
import ctypes

import numpy as np
import pytest

TILE = 128


@pytest.fixture(scope="module")
def lib():
    from libmobility_gb300 import _capi
    return _capi.load()


def plan(lib, N, nper, resident, warps=0):
    info = np.zeros(9, np.int64)
    ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    rc = lib.lmg_internal_sym_plan(N, nper, resident, warps, ptr(info), None, None, None, None)
    if rc == 2:
        return None
    assert rc == 0
    nw, npairs, ntiles = int(info[0]), int(info[1]), int(info[2])
    pairs = np.zeros((npairs, 4), np.int32)
    pseg = np.zeros(npairs, np.int32)
    wt = np.zeros((nw, 8), np.int32)
    tused = np.zeros(ntiles, np.int32)
    assert lib.lmg_internal_sym_plan(N, nper, resident, warps, ptr(info), ptr(pairs), ptr(pseg),
                                     ptr(wt), ptr(tused)) == 0
    return dict(nw=nw, slots=int(info[3]), rt=int(info[4]), grid=int(info[5]),
                steps=int(info[6]), tpb=int(info[7]), cmax=int(info[8]), pairs=pairs,
                pseg=pseg, warps=wt, tused=tused)


def walk(P):
    """The kernel's walk: yields (warp, pair, first step, steps)."""
    for w in range(P["nw"]):
        p, k0, left, ps = P["warps"][w, :4]
        assert np.array_equal(P["warps"][w, 4:], P["pairs"][p])
        assert ps == P["pseg"][p]
        while left > 0:
            tI, tJ = P["pairs"][p, :2]
            n = min((16 if tI == tJ else 32) - k0, left)
            yield w, p, k0, n
            left -= n
            p += 1
            k0 = 0


CASES = [(1, 1, 1, 0), (5, 5, 2, 0), (128, 128, 3, 0), (129, 129, 3, 0), (257, 257, 456, 0),
         (300, 100, 456, 0), (1000, 500, 456, 0), (1537, 1537, 456, 0), (4096, 4096, 304, 0),
         (4096, 4096, 304, 37), (16384, 16384, 304, 0), (640, 128, 304, 1000),
         (12000, 4000, 304, 0)]


@pytest.mark.parametrize("N,nper,resident,warps", CASES)
def test_steps_and_slots(lib, N, nper, resident, warps):
    P = plan(lib, N, nper, resident, warps)
    assert P is not None
    npairs = len(P["pairs"])
    length = np.where(P["pairs"][:, 0] == P["pairs"][:, 1], 16, 32)
    assert P["steps"] == int(length.sum())
    taken = [np.zeros(L, np.int32) for L in length]
    per_warp = np.zeros(P["nw"], np.int64)
    written = np.zeros(P["slots"], np.int32)
    owner = np.full(P["slots"], -1, np.int64)
    for w, p, k0, n in walk(P):
        taken[p][k0:k0 + n] += 1
        per_warp[w] += n
        first, nseg = P["pseg"][p] >> 8, P["pseg"][p] & 255
        seg = w - first
        assert 0 <= seg < nseg
        tI, tJ, sI, sJ = P["pairs"][p]
        written[sI + seg] += 1
        owner[sI + seg] = tI
        if tI != tJ:
            written[sJ + seg] += 1
            owner[sJ + seg] = tJ
    assert all(np.all(t == 1) for t in taken)
    assert per_warp.max() - per_warp.min() <= 1
    ntiles = len(P["tused"])
    assert P["slots"] == ntiles * P["cmax"] and P["cmax"] == P["tused"].max()
    assert np.all(written <= 1)
    for t in range(ntiles):
        rng_ = slice(t * P["cmax"], (t + 1) * P["cmax"])
        w_t = written[rng_]
        # the first tused slots of the range are written, by this tile's sums
        assert np.all(w_t[:P["tused"][t]] == 1) and np.all(w_t[P["tused"][t]:] == 0)
        assert np.all(owner[rng_][:P["tused"][t]] == t)
    assert npairs == (N // nper) * P["tpb"] * (P["tpb"] + 1) // 2
    assert 1 <= P["rt"] <= 32 and P["rt"] & (P["rt"] - 1) == 0


@pytest.mark.parametrize("N,nper,warps", [(1, 1, 5), (5, 5, 3), (129, 129, 7), (300, 100, 11),
                                          (384, 192, 4), (257, 257, 0)])
def test_rotation_covers_each_pair_once(lib, N, nper, warps):
    P = plan(lib, N, nper, 304, warps)
    tpb = P["tpb"]
    cov = np.zeros((N, N), np.int32)

    def tile(t):
        b, I = divmod(int(t), tpb)
        return b * nper + I * TILE, min(TILE, nper - I * TILE)

    lanes = np.arange(32)
    for w, p, k0, n in walk(P):
        tI, tJ = P["pairs"][p, :2]
        bI, vI = tile(tI)
        bJ, vJ = tile(tJ)
        for k in range(k0, k0 + n):
            if tI == tJ and k == 0:
                for q in range(4):
                    for r in range(q, 4):
                        ok = (4 * lanes + r) < vI
                        i = bI + 4 * lanes[ok] + q
                        j = bI + 4 * lanes[ok] + r
                        np.add.at(cov, (np.minimum(i, j), np.maximum(i, j)), 1)
                ls, ss = lanes[:16], (lanes[:16] + 16) & 31
            else:
                ls, ss = lanes, (lanes + k) & 31
            for q in range(4):
                for r in range(4):
                    ok = ((4 * ls + q) < vI) & ((4 * ss + r) < vJ)
                    i = bI + 4 * ls[ok] + q
                    j = bJ + 4 * ss[ok] + r
                    np.add.at(cov, (np.minimum(i, j), np.maximum(i, j)), 1)
    want = np.zeros((N, N), np.int32)
    for b in range(N // nper):
        blk = slice(b * nper, (b + 1) * nper)
        want[blk, blk] = np.triu(np.ones((nper, nper), np.int32))
    assert np.array_equal(cov, want)


def test_shapes_the_kernel_declines(lib):
    # several batches whose size is not a multiple of 4 (float4 slot loads)
    assert plan(lib, 33, 11, 456) is None
    assert plan(lib, 0, 1, 456) is None
    assert plan(lib, 10, 3, 456) is None  # N not a multiple of the batch
