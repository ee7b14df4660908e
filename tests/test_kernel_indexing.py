"""CPU replay of the step kernels' strip and storage index arithmetic.

For edge-case geometries (no CPML, thin CPML, grids that are not multiples
of the tile or of 4, the minimum grid 2*d_pml) every memory-variable slot and
every field offset the TMA step kernel can touch is recomputed here, exactly
as the kernel computes it, and checked against the allocation sizes the
engine uses.  No GPU is involved.
"""
import itertools

import pytest

HZ, HZB, HX = 4, 4, 2
TMA_TZ, TMA_TX = 64, 16


def round_up(a, b):
    return (a + b - 1) // b * b


def geometry(nz, nx, d):
    ld = round_up(nz + HZ + HZB, 32)
    dpz = round_up(d + 6, 4)
    zb0 = (nz - d) & ~3
    return dict(ld=ld, S=ld * (nx + 2 * HX), dpz=dpz, zb0=zb0,
                mx_size=2 * 9 * d * ld if d > 0 else 0,
                mz_size=2 * 9 * nx * dpz if d > 0 else 0)


def strip_accesses(nz, nx, d, pz):
    """Yield (array, first, last) of every vector memory-variable access of a
    thread handling pz consecutive z points."""
    g = geometry(nz, nx, d)
    ld, dpz, zb0 = g["ld"], g["dpz"], g["zb0"]
    ntz, ntx = -(-nz // TMA_TZ), -(-nx // TMA_TX)
    for tz, tx, tzt, txt in itertools.product(range(ntz), range(ntx), range(TMA_TZ // pz), range(TMA_TX)):
        j = tz * TMA_TZ + tzt * pz
        i = tx * TMA_TX + txt
        if not (j < nz and i < nx):
            continue
        lean = i >= d and i < nx - d and j >= d and j + pz - 1 < nz - d
        if lean or d <= 0:
            continue
        if i < d or i >= nx - d:
            side = 0 if i < d else 1
            kx = i - (nx - d) if side else i
            for f, m in itertools.product(range(3), range(3)):
                off = ((side * 9 + f * 3 + m) * d + kx) * ld + j
                yield "mx", off, off + pz - 1
        for side in (0, 1):
            if side == 0 and not j < d:
                continue
            if side == 1 and not j + pz - 1 >= nz - d:
                continue
            k0 = j - zb0 if side else j
            for f, m in itertools.product(range(3), range(3)):
                off = ((side * 9 + f * 3 + m) * nx + i) * dpz + k0
                yield "mz", off, off + pz - 1


@pytest.mark.parametrize("pz", [2, 4])
@pytest.mark.parametrize("nz,nx,d", [(48, 64, 0), (37, 70, 9), (481, 1281, 40), (381, 681, 40), (80, 80, 40),
                                     (201, 201, 20), (45, 53, 1), (66, 47, 5), (19, 23, 2)])
def test_memory_variable_accesses_stay_in_bounds_and_aligned(nz, nx, d, pz):
    g = geometry(nz, nx, d)
    n = 0
    for arr, lo, hi in strip_accesses(nz, nx, d, pz):
        size = g["mx_size"] if arr == "mx" else g["mz_size"]
        assert size > 0, "strip storage touched although d_pml == 0"
        assert 0 <= lo and hi < size, (arr, lo, hi, size)
        assert lo % pz == 0, "vector access must be aligned to its width"
        n += 1
    assert (n == 0) == (d == 0)


@pytest.mark.parametrize("nz,nx", [(48, 64), (37, 70), (481, 1281), (201, 201)])
def test_field_offsets_of_active_groups_stay_in_the_column(nz, nx):
    g = geometry(nz, nx, 4)
    ld = g["ld"]
    for j in range(0, nz, 2):
        # rows j..j+3 (+4 halo) of an active group, and its stencil reach
        assert j + HZ + 3 < ld
        assert j + HZ - 2 >= 0 and j + HZ + 3 + 2 < ld
    # halo columns +-2 of every column stay inside nx + 2*HX columns
    assert (nx - 1) + HX + 2 < nx + 2 * HX


DIRECT_TZ, DIRECT_TX = 32, 8


def bucket_receivers(nz, nx, zr, xr):
    """The engine's receiver bucketing (per TMA tile, then per local column;
    stable counting sort): returns (tile_rec, col_rec, pt, id)."""
    ld = round_up(nz + HZ + HZB, 32)
    ntz, ntx = -(-nz // TMA_TZ), -(-nx // TMA_TX)
    nb = ntz * ntx * TMA_TX
    bucket = [((z // TMA_TZ) + (x // TMA_TX) * ntz) * TMA_TX + x % TMA_TX for z, x in zip(zr, xr)]
    cnt = [0] * (nb + 1)
    for b in bucket:
        cnt[b + 1] += 1
    for b in range(nb):
        cnt[b + 1] += cnt[b]
    fill = cnt[:-1]
    pt, ident = [0] * len(zr), [0] * len(zr)
    for k, b in enumerate(bucket):
        e = fill[b]
        fill[b] += 1
        pt[e] = (xr[k] + HX) * ld + (zr[k] + HZ)
        ident[e] = k
    tile_rec = [cnt[t * TMA_TX] for t in range(ntz * ntx + 1)]
    return tile_rec, cnt, pt, ident, ld, ntz


@pytest.mark.parametrize("nz,nx,nr,seed", [(48, 64, 40, 0), (37, 70, 200, 1), (201, 201, 500, 2), (66, 47, 1, 3),
                                           (130, 35, 0, 4), (481, 1281, 900, 5)])
def test_direct_kernel_finds_each_receiver_once_in_the_shared_buckets(nz, nx, nr, seed):
    """Replays the direct kernel's lookup: a DIRECT_TZ x DIRECT_TX block
    scans the DIRECT_TX bucket columns of its TMA tile and keeps the rows it
    owns (forward recording), and a point scans its own column (adjoint
    injection).  Every receiver, duplicates included, is found exactly once by
    each, and every bucket index stays inside the arrays."""
    import random
    rnd = random.Random(seed)
    zr = [rnd.randrange(nz) for _ in range(nr)]
    xr = [rnd.randrange(nx) for _ in range(nr)]
    if nr > 3:
        zr[1], xr[1] = zr[0], xr[0]          # a duplicated receiver
    tile_rec, col_rec, pt, ident, ld, bntz = bucket_receivers(nz, nx, zr, xr)
    dntz, dntx = -(-nz // DIRECT_TZ), -(-nx // DIRECT_TX)
    recorded, injected = [], []
    for tl in range(dntz * dntx):
        tz, tx = tl % dntz, tl // dntz
        j0, i0 = tz * DIRECT_TZ, tx * DIRECT_TX
        cb = (j0 // TMA_TZ + (i0 // TMA_TX) * bntz) * TMA_TX + i0 % TMA_TX
        assert 0 <= cb and cb + DIRECT_TX < len(col_rec)
        for k in range(col_rec[cb], col_rec[cb + DIRECT_TX]):
            row = pt[k] % ld - HZ
            if j0 <= row < j0 + DIRECT_TZ:
                recorded.append(ident[k])
        for ty in range(DIRECT_TX):
            for tzt in range(DIRECT_TZ):
                j, i = j0 + tzt, i0 + ty
                if j >= nz or i >= nx:
                    continue
                p = (i + HX) * ld + (j + HZ)
                c = cb + ty
                injected += [ident[k] for k in range(col_rec[c], col_rec[c + 1]) if pt[k] == p]
    assert sorted(recorded) == list(range(nr))
    assert sorted(injected) == list(range(nr))
