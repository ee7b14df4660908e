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
