"""CPU check of the thread / block mapping of the fused dual kernel of schedule 2
(k_dual_walk in gt_kernels.cu; launch geometry walk_shape / launch_dual_fused):
every (pixel, slice pair, channel) is updated by exactly one thread, every global
index a thread reads or writes stays inside its field, every shared-memory index
stays inside the block, and the neighbours read from shared memory are the
voxels the update needs.  A restatement of the kernel's index arithmetic, run
before the kernel ever runs on a GPU."""
import itertools

import pytest


def walk_shape(N, Nz, C):
    cp = 1 if C <= 1 else (2 if C <= 2 else 4)
    nz2 = Nz // 2
    nch = (nz2 + 14) // 15
    zc = (nz2 + nch - 1) // nch
    colT = (zc + 1) * cp
    ncol = 512 // colT
    threads = (ncol * colT + 31) // 32 * 32
    return cp, zc, ncol, 32, nch, threads


@pytest.mark.parametrize("N,Nz,C", [(36, 8, 1), (36, 6, 2), (36, 10, 4), (36, 4, 3), (28, 6, 4), (40, 60, 4),
                                    (33, 64, 2), (17, 2, 1), (20, 32, 3)])
def test_walk_mapping_covers_every_voxel_once_in_bounds(N, Nz, C):
    cp, ZC, NCOL, R, nch, T = walk_shape(N, Nz, C)
    assert NCOL >= 2 and T <= 512
    S = C * Nz
    vol, rowS = N * N * S, N * S
    grid = ((N + NCOL - 2) // (NCOL - 1), (N + R - 1) // R, nch)
    colT = (ZC + 1) * cp
    seen = set()
    for bx, by, bz in itertools.product(range(grid[0]), range(grid[1]), range(grid[2])):
        for t in range(T):
            col, rr = divmod(t, colT)
            pl, c = divmod(rr, cp)
            x = bx * (NCOL - 1) - 1 + col
            z0 = bz * 2 * ZC + 2 * (pl - 1)
            pthr = col < NCOL and 0 <= x < N and 0 <= z0 < Nz and c < C
            dthr = pthr and col >= 1 and pl >= 1
            nbx, nbz = col + 1 < NCOL, pl < ZC
            hx, hz1 = x < N - 1, z0 + 1 < Nz - 1
            if nbx:
                assert t + colT < T and bx * (NCOL - 1) - 1 + col + 1 == x + 1  # the x successor's slot
            if pthr and nbz:
                assert t + cp < (col + 1) * colT  # the pair above is in the same column
            for s in range(R + 1):
                y = by * R - 1 + s
                if not (pthr and 0 <= y < N):
                    continue
                i = (y * N + x) * S + c * Nz + z0
                assert i % 2 == 0 and 0 <= i and i + 1 < vol  # float2 operands, 8-byte aligned
                if y < N - 1:
                    assert i + rowS + 1 < vol
                if not nbx and hx:
                    assert i + S + 1 < vol
                if not nbz and hz1:
                    assert i + 2 < vol and z0 + 2 < Nz
                if s >= 1 and dthr:
                    key = (x, y, z0, c)
                    assert key not in seen, key
                    seen.add(key)
                    if z0 > 0:  # the pair below (the halo pair for pl = 1) holds slice z0 - 1
                        assert bz * 2 * ZC + 2 * (pl - 2) == z0 - 2
    assert len(seen) == N * N * (Nz // 2) * C
