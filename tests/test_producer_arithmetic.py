"""CPU replay of the persistent step kernels' producer arithmetic.

* Tile numbers are decoded without integer division (csrc/mnad_tile.cuh,
  div_small): q = trunc(float(n) * RN(1/d)) followed by two corrections each
  way.  Replayed here in float32 for tile numbers below 2^24 (the engine
  refuses larger launch groups) and every divisor class the engine produces.
* A CTA that gave up waits for the last fill it issued on each stage
  (drain_fills): from the total fill count F, stage k has had
  (F + NS - 1 - k) / NS fills, the last one completing phase fills - 1.
  Replayed against a simulation of the producer's fill sequence.
* A CTA's first NS tiles are b, b + grid, ... and later tiles are claimed
  from a counter offset by NS * grid: every tile is processed exactly once.
* The last warp to release a stage refills it with the tile thread 0
  claimed for that stage in the same iteration: replayed with warps moving
  at random rates, every warp computes every tile of the CTA once, in order.
No GPU is involved.
"""
import numpy as np
import pytest


def div_small(n, d):
    inv = np.float32(1.0) / np.float32(d)
    q = (np.asarray(n, dtype=np.int64).astype(np.float32) * inv).astype(np.int64)
    for _ in range(2):
        q -= (q * d > n)
    for _ in range(2):
        q += ((q + 1) * d <= n)
    return q


@pytest.mark.parametrize("d", [1, 2, 3, 7, 8, 9, 81, 255, 602, 648, 1023, 2048, 5355, 65535, 99991, 1 << 20])
def test_div_small_is_exact_below_2_24(d):
    rng = np.random.default_rng(d)
    n = np.concatenate([rng.integers(0, 1 << 24, 20000), np.arange(0, 4096),
                        np.array([(1 << 24) - 1, (1 << 24) - 2]),
                        np.clip(np.arange(1, 200) * d + np.array([[-1], [0], [1]]), 0, (1 << 24) - 1).ravel()])
    assert np.array_equal(div_small(n, d), n // d)


@pytest.mark.parametrize("ns", [2, 3])
@pytest.mark.parametrize("stop", [0, 1, 2, 5, 17])
def test_drain_counts_each_stage_fills(ns, stop):
    """The producer fills stages 0..ns-1, then refills stage n % ns after
    iteration n for n < stop; after any prefix of that sequence the formula
    gives each stage's fill count (and so the parity of its last phase)."""
    fills = [0] * ns
    seq = list(range(ns)) + [n % ns for n in range(stop)]
    for f, stage in enumerate(seq):
        fills[stage] += 1
        total = f + 1
        for k in range(ns):
            assert (total + ns - 1 - k) // ns == fills[k]


@pytest.mark.parametrize("ntiles,grid,ns", [(1, 1, 3), (5, 304, 3), (700, 304, 3), (912, 304, 3), (77000, 304, 3),
                                            (1000, 608, 2), (3, 2, 3)])
def test_static_first_tiles_and_claims_cover_every_tile_once(ntiles, grid, ns):
    grid = min(grid, ntiles)
    first = ns * grid
    seen = np.zeros(ntiles, dtype=int)
    for b in range(grid):
        for k in range(ns):
            t = b + k * grid
            if t < ntiles:
                seen[t] += 1
    counter = 0
    while first + counter < ntiles:        # claims in any interleaving hand out consecutive numbers
        seen[first + counter] += 1
        counter += 1
    assert np.all(seen == 1)


@pytest.mark.parametrize("nwarps,ns", [(8, 3), (4, 2)])
@pytest.mark.parametrize("seed", range(6))
def test_last_warp_refill_processes_each_claimed_tile_once_in_order(nwarps, ns, seed):
    """Replay of the refill protocol with warps progressing at random rates:
    thread 0 (warp 0) writes its claim for stage n % ns when it starts
    iteration n; the warp that completes the release count of a stage
    refills it with that claim; a warp may start iteration n only once the
    stage holds iteration n's tile.  Every tile is then computed by every warp
    exactly once, in claim order, and the stream ends with "no tile"."""
    rng = np.random.default_rng(seed)
    ntiles, grid, b = 50, 4, 1                       # one CTA (b) of a launch of `grid` CTAs
    first = ns * grid
    counter = iter(range(0, 10 ** 6))
    claims_made = []

    def claim():
        t = first + next(counter) * grid + b         # the other CTAs take the claims in between
        claims_made.append(t)
        return t

    stage_tile = [b + k * grid if b + k * grid < ntiles else -1 for k in range(ns)]
    stage_iter = list(range(ns))                     # which iteration each stage currently serves
    next_tile = [None] * ns
    released = [0] * ns
    next_claim = claim()
    it = [0] * nwarps                                # next iteration of each warp
    done = [False] * nwarps
    computed = [[] for _ in range(nwarps)]
    for _ in range(100000):
        if all(done):
            break
        w = int(rng.integers(nwarps))
        if done[w]:
            continue
        n = it[w]
        s = n % ns
        if stage_iter[s] != n:                       # the stage is not filled for this iteration yet
            continue
        t = stage_tile[s]
        if t < 0:
            done[w] = True
            continue
        if w == 0:                                   # thread 0: the claim for this stage's next fill
            next_tile[s] = next_claim
            next_claim = claim()
        computed[w].append(t)
        released[s] += 1
        if released[s] == nwarps:                    # the last warp to release refills
            assert next_tile[s] is not None          # written by warp 0 in this iteration
            released[s] = 0
            t2 = next_tile[s]
            stage_tile[s] = t2 if t2 < ntiles else -1
            stage_iter[s] = n + ns
        it[w] += 1
    assert all(done)
    expected = [t for t in range(ntiles) if t % grid == b]
    for w in range(nwarps):
        assert computed[w] == expected
