"""Index maps of the red-black half-sweeps, checked on the CPU.

The multigrid tiles (csrc/kc_mg_tile.cuh, ``mg_colour_cells``) hand each
thread cells of one colour only: AJ/2 threads share a staged row, thread m
taking column 2m or 2m + 1, whichever has the colour.  The blocked
Gauss-Seidel sweeps (csrc/kc_solver.cu, ``k_gs_block_sweeps``) give each
thread a column pair -- one cell of each colour -- in rows a0, a0 + RP, ...
These restate both maps and check, for every tile shape the kernels use,
that a half-sweep visits exactly the cells of its colour in its region, each
once, and that the pair map stages every cell of the tile exactly once.
"""
import itertools

import pytest


def colour_cells(nt, aj, col, a0, a1, b0, b1):
    """(thread, staged row, staged column) visited by mg_colour_cells."""
    hj = aj // 2
    rp = nt // hj
    assert nt % hj == 0
    out = []
    for t in range(nt):
        m = t & (hj - 1)
        a = a0 + t // hj
        while a < a1:
            b = 2 * m + ((a + col) & 1)
            if b0 <= b < b1:
                out.append((t, a, b))
            a += rp
    return out


# (TI, AJ, RY, H): level 0 (one sweep), MgTile3 (3-cell halo), the levels below level 0
# with one to three sweeps on the small and the large tiles
TILES = [(16, 64, 4, 2), (16, 64, 4, 3), (16, 64, 4, 4), (12, 64, 4, 4), (8, 64, 4, 6),
         (8, 32, 4, 2), (8, 32, 4, 4), (8, 32, 4, 6)]


@pytest.mark.parametrize("ti,aj,ry,h_halo", TILES)
def test_colour_map_visits_each_cell_of_the_colour_once(ti, aj, ry, h_halo):
    nt = aj * ry
    ai = ti + 2 * h_halo
    regions = [(h, h) for h in range(1, h_halo + 1)] + [(1, 1), (2, 2)]
    for (ra, rb), col in itertools.product(regions, (0, 1)):
        got = colour_cells(nt, aj, col, ra, ai - ra, rb, aj - rb)
        cells = [(a, b) for _, a, b in got]
        want = {(a, b) for a in range(ra, ai - ra) for b in range(rb, aj - rb) if (a + b) & 1 == col}
        assert len(cells) == len(set(cells)), "a cell visited twice"
        assert set(cells) == want
        # a warp's lanes share one row: every lane of a full row pass has a cell
        per_warp_rows = {}
        for t, a, _ in got:
            per_warp_rows.setdefault((t // 32, a), 0)
            per_warp_rows[(t // 32, a)] += 1
        assert all(v <= 32 for v in per_warp_rows.values())


def gs_pair_map(ti, aj, ry, nu):
    """Per thread: its rows and its red and black columns in k_gs_block_sweeps."""
    h = 2 * nu
    nt, hj = aj * ry, aj // 2
    rp = nt // hj
    ai = ti + 2 * h
    r_cnt = (ai + rp - 1) // rp
    assert rp % 2 == 0
    threads = []
    for t in range(nt):
        m, a0 = t & (hj - 1), t // hj
        bcol = (2 * m + (a0 & 1), 2 * m + 1 - (a0 & 1))   # red, black
        rows = [a0 + r * rp for r in range(r_cnt) if a0 + r * rp < ai]
        threads.append((rows, bcol))
    return threads, ai


@pytest.mark.parametrize("ti,aj,ry,nu", [(12, 64, 4, 2), (12, 32, 4, 2), (16, 64, 4, 1)])
def test_gs_pair_map(ti, aj, ry, nu):
    threads, ai = gs_pair_map(ti, aj, ry, nu)
    staged = [(a, b) for rows, bcol in threads for a in rows for b in bcol]
    assert len(staged) == len(set(staged)) == ai * aj      # every staged cell exactly once
    for rows, (red, black) in threads:
        for a in rows:
            assert (a + red) & 1 == 0 and (a + black) & 1 == 1
    for h in range(1, 2 * nu + 1):   # odd h: red, even h: black; region less h rings
        q = 0 if h & 1 else 1
        got = [(a, bcol[q]) for rows, bcol in threads if h <= bcol[q] < aj - h for a in rows if h <= a < ai - h]
        want = {(a, b) for a in range(h, ai - h) for b in range(h, aj - h) if (a + b) & 1 == q}
        assert len(got) == len(set(got)) and set(got) == want
