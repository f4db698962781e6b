"""The FP32 bound of the 'nrst' neighbour selection (k_neb_nrst,
csrc/spi_nebs.cu) restated in numpy float32: once a cell holds k stations,
a station whose FP32 squared distance from coordinates relative to station
0 exceeds (thr * 1.00001 + 2^-20 (|x_s| + |y_s| + |x_c| + |y_c|))^2 is
skipped, thr the current k-th FP64 distance. The selection with the skip
must equal the (FP64 distance, index) selection of every station, with and
without a fused multiply-add in the squared distance, on lattices full of
exact ties, co-located stations, clusters and UTM-sized coordinates."""
import numpy as np
import pytest

f32 = np.float32
REL, ABS = f32(1.00001), f32(2.0 ** -20)


def exact(cx, cy, sx, sy, k):
    out = []
    for x, y in zip(cx, cy):
        dx, dy = x - sx, y - sy
        d = np.sqrt(dx * dx + dy * dy)
        out.append(np.sort(np.lexsort((np.arange(sx.size), d))[:k]))
    return np.array(out)


def bounded(cx, cy, sx, sy, k, fma):
    ox, oy = sx[0], sy[0]
    xs, ys = (sx - ox).astype(f32), (sy - oy).astype(f32)
    ss = (np.abs(xs) + np.abs(ys)).astype(f32)
    out, cand = [], 0
    for x, y in zip(cx, cy):
        xc, yc = f32(x - ox), f32(y - oy)
        sc = f32(abs(xc) + abs(yc))
        keys = []  # (d, index) ascending, at most k
        lim0 = f32(np.inf)
        for j in range(sx.size):
            ex, ey = f32(xs[j] - xc), f32(ys[j] - yc)
            if fma:
                d2 = f32(np.float64(ex) * ex + f32(ey * ey))
                lim = f32(np.float64(ABS) * f32(ss[j] + sc) + lim0)
            else:
                d2 = f32(f32(ex * ex) + f32(ey * ey))
                lim = f32(f32(ABS * f32(ss[j] + sc)) + lim0)
            if d2 > f32(lim * lim):
                continue
            cand += 1
            dx, dy = x - sx[j], y - sy[j]
            key = (np.sqrt(dx * dx + dy * dy), j)
            if len(keys) == k and not key < keys[-1]:
                continue
            keys = sorted(keys + [key])[:k]
            if len(keys) == k:
                lim0 = f32(f32(keys[-1][0]) * REL)
        out.append(np.sort([j for _, j in keys]))
    return np.array(out), cand


@pytest.mark.parametrize("case", range(8))
def test_bound_keeps_the_exact_selection(case):
    rng = np.random.default_rng(100 + case)
    n = int(rng.integers(20, 160))
    k = int(rng.integers(1, min(n, 64) + 1))
    off = [0.0, 5e5, 5.8e6, -3e6][case % 4]
    if case % 4 == 0:  # a lattice: many exact ties
        g = np.arange(int(np.sqrt(n)) + 1) * 1000.0
        sx, sy = (a.ravel()[:n] + off for a in np.meshgrid(g, g))
        cx = rng.integers(0, 30, 80) * 500.0 + off
        cy = rng.integers(0, 30, 80) * 500.0 + off
    else:
        sx, sy = rng.uniform(0, 2e5, n) + off, rng.uniform(0, 2e5, n) + off
        if case % 4 == 1:  # co-located pairs
            m = sx[1::3].size
            sx[1::3], sy[1::3] = sx[0::3][:m], sy[0::3][:m]
        if case % 4 == 2:  # one tight cluster
            sx, sy = rng.normal(1e5, 3e3, n) + off, rng.normal(1e5, 3e3, n) + off
        cx = rng.uniform(-5e4, 2.5e5, 80) + off
        cy = rng.uniform(-5e4, 2.5e5, 80) + off
    ref = exact(cx, cy, sx, sy, k)
    for fma in (False, True):
        got, cand = bounded(cx, cy, sx, sy, k, fma)
        assert np.array_equal(got, ref), fma
    if k < n // 4:
        assert cand < 0.8 * n * cx.size  # the bound skips stations
