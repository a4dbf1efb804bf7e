"""The fine z grid's argument, on the CPU, in float32 numpy.

The prediction count can walk a z grid f times finer than the grid
(trax_set_fine_rows; fine_walk in k_triplets.cu).  Its results equal the grid
walk's because:

1. a hit's fine row, h(z) = floor((z - minZ) * f / sZ) clamped into the block
   of its grid row, is non-decreasing in z and lies in that block, so every
   z row's hits keep their range of grid order in fine order;
2. walking, for each of a window's z rows and phi parts, the fine rows
   between fine_row(zl) and fine_row(zh) visits every hit that passes a z
   test in [zl, zh] and the grid walk visits, each as often (also for
   windows across +-pi and wider than 2 pi, whose parts overlap);
3. the captured candidates, sorted per (row, part) by grid index as they
   arrive in fine order, are the grid walk's first ones, also when the
   walk stops at the first (row, part) after the slots are full (the store
   pass's re-walks).

This file restates the grid walk (pred_row_parts), the fine walk and the
capture's insertion and replacement rules in Python and checks the three
points on random layers and windows.  The GPU tests
(tests/test_gpu_fine_grid.py) check the kernels themselves against the
oracle.
"""
import numpy as np
import pytest

f32 = np.float32
MIN_Z, MAX_Z = f32(-300.0), f32(300.0)
MIN_PHI, MAX_PHI = f32(-np.pi), f32(np.pi)
PI = f32(3.14159274101257324)  # TRAX_PI_F
U32 = 1 << 32


def f2u_sat(x):
    """Truncate to uint32, saturating, NaN -> 0 (the kernels' conversion)."""
    x = np.asarray(x, np.float64)
    return np.where(np.isnan(x), 0.0, np.clip(np.trunc(x), 0.0, U32 - 1.0)).astype(np.int64)


def f2i_sat(x):
    x = np.asarray(x, np.float64)
    return np.where(np.isnan(x), 0.0, np.clip(np.trunc(x), -2.0 ** 31, 2.0 ** 31 - 1)).astype(np.int64)


class Layer:
    """One (event, layer): its hits in grid order and in fine order."""

    def __init__(self, z, phi, n_z, n_p, f):
        self.n_z, self.n_p, self.f = n_z, n_p, f
        self.sZ = f32(f32(MAX_Z - MIN_Z) / f32(n_z))
        self.sP = f32(f32(MAX_PHI - MIN_PHI) / f32(n_p))
        self.scale = f32(f32(f) / self.sZ)
        row = self.row(z)
        col = np.minimum(f2u_sat(np.floor(f32(phi - MIN_PHI) / self.sP)), n_p)
        cell = row * (n_p + 1) + col
        order = np.argsort(cell, kind="stable")  # grid order: by cell, ties by input order
        self.z, self.phi, self.rowOf, self.col = z[order], phi[order], row[order], col[order]
        self.C = (n_z + 1) * (n_p + 1)
        self.off = np.searchsorted(np.sort(cell), np.arange(self.C), side="left")
        frow = self.fine_row(self.z, self.rowOf)
        fcell = frow * (n_p + 1) + self.col
        self.fine = np.argsort(fcell, kind="stable")  # fine position -> grid index, ties by grid order
        self.Cf = (f * n_z + 1) * (n_p + 1)
        self.foff = np.searchsorted(np.sort(fcell), np.arange(self.Cf), side="left")
        self.frow = frow

    def row(self, z):
        return np.minimum(f2u_sat(np.floor(f32(z - MIN_Z) / self.sZ)), self.n_z - 1)

    def fine_row(self, z, g):
        h = f2u_sat(np.floor(f32(f32(z - MIN_Z) * self.scale)))
        lo = np.asarray(g, np.int64) * self.f
        return np.minimum(np.maximum(h, lo), lo + self.f - 1)


def phi_window(L, centre, half):
    """pred_phi_window's tail: the wrap flag, the wrapped bounds and the columns."""
    lo, hi = f32(centre - half), f32(centre + half)
    wrap = bool(lo < -PI or hi > PI or lo > PI or hi < -PI)
    lo = f32(lo - f32(2 * PI)) if lo > PI else lo
    lo = f32(lo + f32(2 * PI)) if lo < -PI else lo
    hi = f32(hi - f32(2 * PI)) if hi > PI else hi
    hi = f32(hi + f32(2 * PI)) if hi < -PI else hi
    pL = int(f2u_sat(np.floor(f32(lo - MIN_PHI) / L.sP)))
    pH = min((int(f2u_sat(np.floor(f32(hi - MIN_PHI) / L.sP))) + 1) % U32, L.n_p)
    return lo, hi, wrap, pL, pH


def passes(L, j, zl, zh, plo, phi_hi, wrap):
    p, z = L.phi[j], L.z[j]
    a, b = plo <= p, p <= phi_hi
    return bool((a or b) if wrap else (a and b)) and bool(zl <= z <= zh)


def grid_walk(L, zLo, zHi, pL, pH, wrap):
    """The grid walk's visits (row, part, grid index): pred_row_parts."""
    cell = lambda k: int(L.off[min(k, L.C - 1)])
    out = []
    for zs in range(zLo, zHi):
        row = zs * (L.n_p + 1)
        zStart, zEnd = cell(row), cell(row + L.n_p + 1)
        length = zEnd - zStart
        J0 = cell(row + pL)
        end2 = (wrap * zEnd + cell(row + pH) - wrap * zStart) % U32
        a1, b1 = J0, max(min(end2, zEnd), J0)
        out += [(zs, 0, j) for j in range(a1, b1)]
        j2 = max(J0, zEnd)
        if j2 < end2:
            out += [(zs, 1, j) for j in range(j2 - length, end2 - length)]
    return out


def fine_walk(L, zl, zh, zLo, zHi, pL, pH, wrap):
    """fine_walk's visits, in its order: (row, part, grid index)."""
    F, nP1 = L.f, L.n_p + 1
    fLo = int(L.fine_row(zl, min(zLo, L.n_z - 1)))
    fHi = int(L.fine_row(zh, zHi - 1)) + 1 if zHi else 0
    cell = lambda k: int(L.foff[min(k, L.Cf - 1)])
    out = []
    for r in range(zLo, zHi):
        for part in range(int(wrap) + 1):
            ca = 0 if part else pL
            cb = nP1 if (wrap and not part) else pH
            for fr in range(max(F * r, fLo), min(F * r + F, fHi)):
                a = cell(fr * nP1 + ca)
                b = max(a, cell(fr * nP1 + cb))
                out += [(r, part, int(L.fine[s])) for s in range(a, b)]
    return out


def capture(chunks, n_keep):
    """fine_walk's capture: chunks of grid indices in arrival order."""
    slot, n_store = [None] * n_keep, 0
    for ch in chunks:
        cs, last = n_store, 0
        for j in ch:
            if n_store < n_keep:
                if n_store == cs or j > last:
                    slot[n_store], last = j, j
                else:
                    q = n_store
                    slot[q] = last
                    q -= 1
                    while q > cs and slot[q - 1] > j:
                        slot[q] = slot[q - 1]
                        q -= 1
                    slot[q] = j
            elif cs < n_keep and j < last:
                q, top = n_keep - 1, j
                while q > cs:
                    v = slot[q - 1]
                    if v <= j:
                        break
                    slot[q] = v
                    if q == n_keep - 1:
                        top = v
                    q -= 1
                slot[q], last = j, top
            n_store += 1
    return slot[:min(n_store, n_keep)], n_store


def random_layer(rng, n, n_z, n_p, f):
    z = rng.uniform(-299.9, 299.9, n).astype(f32)
    # hits on and next to the z rows' and the fine rows' edges
    sZ = f32(f32(MAX_Z - MIN_Z) / f32(n_z))
    edges = (MIN_Z + f32(sZ / f32(f)) * rng.integers(0, f * n_z, n // 4).astype(f32)).astype(f32)
    z[: edges.size] = np.nextafter(edges, edges + rng.choice([-1, 1], edges.size).astype(f32)).astype(f32)
    phi = rng.uniform(-np.pi, np.pi, n).astype(f32)
    phi[:8] = [MIN_PHI, MAX_PHI, PI, -PI, 0, f32(1e-7), f32(-1e-7), f32(3.1415)]
    return Layer(z, phi, n_z, n_p, f)


@pytest.mark.parametrize("n_z,n_p,f", [(80, 256, 8), (80, 256, 2), (40, 100, 16), (250, 48, 4), (7, 5, 8)])
def test_fine_order_keeps_each_z_rows_range(n_z, n_p, f):
    L = random_layer(np.random.default_rng(n_z * 7 + f), 6000, n_z, n_p, f)
    # the fine row lies in the block of the grid row, and is monotone in z
    assert np.all(L.frow // f == L.rowOf)
    zs = np.sort(L.z)
    fr = L.fine_row(zs, L.row(zs))
    assert np.all(np.diff(fr) >= 0)
    # each z row's hits keep their range of grid order in fine order
    pos = np.empty_like(L.fine)
    pos[L.fine] = np.arange(L.fine.size)
    starts = L.off[np.arange(n_z + 1) * (n_p + 1)]
    for r in range(n_z):
        a, b = starts[r], starts[r + 1]
        assert sorted(pos[a:b]) == list(range(a, b))


@pytest.mark.parametrize("n_z,n_p,f", [(80, 256, 8), (80, 256, 4), (40, 100, 16), (250, 48, 2), (7, 5, 8)])
def test_fine_walk_equals_grid_walk(n_z, n_p, f):
    rng = np.random.default_rng(1000 + n_z + f)
    L = random_layer(rng, 5000, n_z, n_p, f)
    checked = 0
    for _ in range(400):
        # the count variant's z bounds and the store variant's, a little apart
        c = f32(rng.uniform(-320, 320))
        w = f32(rng.choice([0.05, 0.3, 3.0, 40.0]) * rng.uniform(0.1, 1))
        zl0, zh0 = f32(c - w), f32(c + w)
        d = f32(rng.choice([0.0, 1e-5, 0.02]))
        zl1, zh1 = f32(zl0 + d), f32(zh0 - d / 2)
        zl, zh = min(zl0, zl1), max(zh0, zh1)
        zLo = int(max(f2i_sat(np.floor(f32(zl - MIN_Z) / L.sZ)), 0))
        zHi = int(min(f2u_sat(np.floor(f32(zh - MIN_Z) / L.sZ)) + 1, n_z))
        half = f32(rng.choice([0.01, 0.3, 1.5, 3.3]) * rng.uniform(0.2, 1))  # 3.3: windows wider than 2 pi
        plo, phi_hi, wrap, pL, pH = phi_window(L, f32(rng.uniform(-np.pi, np.pi)), half)
        if pL > n_p:
            continue  # the kernel keeps the grid walk for these
        g = grid_walk(L, zLo, zHi, pL, pH, wrap)
        fw = fine_walk(L, zl, zh, zLo, zHi, pL, pH, wrap)
        # the same hits pass, as often, for both variants (the counts)
        for lo_, hi_ in ((zl0, zh0), (zl1, zh1)):
            ok_g = sorted((r, p, j) for r, p, j in g if passes(L, j, lo_, hi_, plo, phi_hi, wrap))
            ok_f = sorted((r, p, j) for r, p, j in fw if passes(L, j, lo_, hi_, plo, phi_hi, wrap))
            assert ok_g == ok_f
        # the captured candidates: the grid walk's first store-valid visits
        valid = [(r, p, j) for r, p, j in fw if passes(L, j, zl1, zh1, plo, phi_hi, wrap)]
        chunks, key = [], None
        for r, p, j in valid:
            if (r, p) != key:
                chunks.append([])
                key = (r, p)
            chunks[-1].append(j)
        want = [j for r, p, j in g if passes(L, j, zl1, zh1, plo, phi_hi, wrap)]
        for n_keep in (1, 4, 16):
            got, n_store = capture(chunks, n_keep)
            assert n_store == len(want) and got == want[:n_keep]
        checked += bool(want)
    assert checked > 50


def test_capture_keeps_the_first_in_chunk_order():
    rng = np.random.default_rng(5)
    for _ in range(20000):
        n_keep = int(rng.choice([1, 2, 4, 8]))
        chunks, base = [], 0
        for _c in range(int(rng.integers(0, 5))):
            k = int(rng.integers(0, 7))
            chunks.append([int(v) for v in rng.permutation(np.arange(base, base + 20))[:k]])
            base = max(base + int(rng.integers(-10, 26)), 0)
        want = [j for ch in chunks for j in sorted(ch)]
        assert capture(chunks, n_keep) == (want[:n_keep], len(want))
        # the store pass's re-walk stops at the first (row, part) that starts
        # with n_keep captures made: what follows cannot change the slots
        kept, total = [], 0
        for ch in chunks:
            if total >= n_keep:
                break
            kept.append(ch)
            total += len(ch)
        assert capture(kept, n_keep)[0] == want[:n_keep]
