"""SurfaceAreaHeuristic::generateBatches against a plain restatement of the
reference's algorithm (SurfaceAreaHeuristic.cpp:10-104), on inputs with
many equal centres and signed zeros: the library's sorts (a stable radix
sort for NaN-free keys, std::stable_sort otherwise) must give exactly the
reference's stable order.  CPU only; runs on any host."""
import numpy as np
import pytest

from rasterizer_gb300 import api

F = np.float32


def _area(lo, hi):
    """Aabb::surfaceArea (VectorMath.h:57-62): DPPS 0x7F of the extents with
    their yzx shuffle: (ex*ey + ey*ez) + (ez*ex + 0), float32."""
    e = (hi - lo).astype(F)
    p0, p1, p2 = F(e[0] * e[1]), F(e[1] * e[2]), F(e[2] * e[0])
    return F(F(p0 + p1) + F(p2 + F(0)))


def _split(lo, hi, ctr, idx, gran):
    n = len(idx)
    best, best_axis, best_index = F(np.inf), -1, -1
    for axis in range(3):
        idx = sorted(idx, key=lambda i: ctr[i, axis])  # stable, like std::stable_sort with `<`
        left, right = np.empty(n, F), np.empty(n, F)
        alo, ahi = np.full(4, np.inf, F), np.full(4, -np.inf, F)
        for k, i in enumerate(idx):
            alo, ahi = np.where(alo < lo[i], alo, lo[i]), np.where(ahi > hi[i], ahi, hi[i])
            left[k] = _area(alo, ahi)
        alo, ahi = np.full(4, np.inf, F), np.full(4, -np.inf, F)
        for k in range(n - 1, -1, -1):
            i = idx[k]
            alo, ahi = np.where(alo < lo[i], alo, lo[i]), np.where(ahi > hi[i], ahi, hi[i])
            right[k] = _area(alo, ahi)
        for s in range(gran, n - gran, gran):
            cost = F(F(left[s - 1] * F(s)) + F(right[s] * F(n - s)))
            if cost < best:
                best, best_axis, best_index = cost, axis, s
    if best_axis < 0:
        return -1, idx
    return best_index, sorted(idx, key=lambda i: ctr[i, best_axis])


def _batches(aabbs, target, gran):
    lo, hi = aabbs[:, :4], aabbs[:, 4:]
    ctr = (lo + hi).astype(F)
    out = []

    def rec(idx):
        split, idx = _split(lo, hi, ctr, idx, gran) if len(idx) > 2 * gran else (-1, idx)
        if split < 0:
            out.append(idx)
            return
        for part in (idx[:split], idx[split:]):
            if len(part) < target:
                out.append(part)
            else:
                rec(part)

    rec(list(range(len(aabbs))))
    return out


def _boxes(n, seed, snap):
    rng = np.random.default_rng(seed)
    lo = rng.uniform(-50, 50, (n, 4)).astype(F)
    if snap:
        lo = np.round(lo / snap) * snap  # many equal centres
    lo[:, 3] = 1.0
    hi = (lo + np.round(rng.uniform(0, 3, (n, 4)))).astype(F)
    hi[:, 3] = 1.0
    z = rng.integers(0, n, n // 10)
    lo[z[::2], 0], hi[z[::2], 0] = F(-0.0), F(-0.0)  # centres -0 and +0: equal under `<`
    lo[z[1::2], 0], hi[z[1::2], 0] = F(0.0), F(0.0)
    return np.ascontiguousarray(np.concatenate([lo, hi], axis=1), F)


@pytest.mark.parametrize("n,seed,snap", [(6000, 1, 8.0), (5000, 2, 0.0), (3000, 3, 25.0)])
def test_sah_matches_the_reference_order(n, seed, snap):
    aabbs = _boxes(n, seed, snap)
    got = api.SurfaceAreaHeuristic.generateBatches(aabbs, 512, 8)
    want = _batches(aabbs, 512, 8)
    assert len(got) == len(want)
    for g, w in zip(got, want):
        assert np.array_equal(np.asarray(g), np.asarray(w, np.uint32))
