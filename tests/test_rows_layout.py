"""The row-tiled step kernel's data movement, emulated on the CPU (no GPU).

csrc/lbm_tma.cu moves whole grid rows between HBM and shared memory with one bulk copy per
population plane each way, and does bounce-back through mailbox slots fixed up by a pass over the
wall-cell list.  This test restates that index arithmetic in numpy -- the tile geometry
(rows_per_tile, RowGeom), the plane ranges p n + c0 + sh[p], the shared-memory offsets of the
reads and writes, the write-back of untouched slots, and the two mailbox passes of an odd step --
drives the numpy AA stepper's collision with it, and checks:
  - every bulk copy lies inside the distribution array and every shared-memory index a live cell
    uses lies inside its tile;
  - no global element is covered by two (tile, plane) ranges of one step (the kernel's blocks
    then never race);
  - the result equals the plain AA step (np_aa.aa_step) bit for bit over many steps, on masks with
    random solid cells, partial last tiles, and the 320-cell tile variant.
"""
import numpy as np
import pytest

import np_aa

CX, CY, CZ, OPP, W = np_aa.CX, np_aa.CY, np_aa.CZ, np_aa.OPP, np_aa.W


def rows_per_tile(nx, ny, nz, esize, ps):
    """Mirror of rows_per_tile() in csrc/lbm_tma.cu."""
    if nx > ps or (nx * esize) % 16 != 0 or nz < 3 or ny < 3:
        return 0
    R = max(1, 256 // nx)
    while R > 1 and R * nx > ps:
        R -= 1
    return R if R * nx <= ps else 0


def geometry(nx, ny, nz, esize):
    ps = 256
    R = rows_per_tile(nx, ny, nz, esize, 256)
    if R == 0:
        ps = 320
        R = rows_per_tile(nx, ny, nz, esize, 320)
    return R, ps


def wall_list(flags):
    """Mirror of wall_list_kernel: fluid cells with a link bit, planes 1..nz-2, 1 <= i <= nx-2."""
    nz, ny, nx = flags.shape
    fl = flags.reshape(-1).astype(np.int64)
    c = np.arange(fl.size)
    i, k = c % nx, c // (nx * ny)
    want = ((fl & 1) == 0) & (((fl >> 8) & 0x7FFFE) != 0) & (k >= 1) & (k + 1 < nz) & (i >= 1) & (i + 1 < nx)
    return c[want]


def mailbox(F, flags, cells, n, off, direction):
    """Mirror of bb_mailbox_kernel: DIR 0 (d + e_q, q) := (d, opp q); DIR 1 the reverse."""
    fl = flags.reshape(-1).astype(np.int64)
    flat = F.reshape(-1)
    for d in cells:
        links = (fl[d] >> 8) & 0x7FFFE
        for q in range(1, 19):
            if (links >> q) & 1:
                own = OPP[q] * n + d
                mb = q * n + d + off[q]
                assert 0 <= own < 19 * n and 0 <= mb < 19 * n
                if direction == 0:
                    flat[mb] = flat[own]
                else:
                    flat[own] = flat[mb]


def collide(fin, omega):
    """The BGK collision of np_aa.aa_step on fin [19, m] (same operations, same order)."""
    rho = fin.sum(0)
    ux = (CX[:, None] * fin).sum(0) / rho
    uy = (CY[:, None] * fin).sum(0) / rho
    uz = (CZ[:, None] * fin).sum(0) / rho
    usq = ux * ux + uy * uy + uz * uz
    out = np.empty_like(fin)
    for q in range(19):
        eu = CX[q] * ux + CY[q] * uy + CZ[q] * uz
        feq = W[q] * rho * (1 + 3 * eu + 4.5 * eu * eu - 1.5 * usq)
        out[q] = fin[q] - omega * (fin[q] - feq)
    return out


def rows_step(f, flags, t, omega, esize, cover=None):
    """One step of f [19, nz, ny, nx] in place, moved the way the row-tiled kernel moves it."""
    nz, ny, nx = flags.shape
    n = nx * ny * nz
    F = f.reshape(19, n)
    flat = F.reshape(-1)
    fl = flags.reshape(-1).astype(np.int64)
    off = CX + CY * nx + CZ * nx * ny
    R, ps = geometry(nx, ny, nz, esize)
    assert R > 0
    T = R * nx
    row0, nrows = ny, ny * (nz - 2)
    ntiles = (nrows + R - 1) // R
    parity = t % 2
    sh = (CY * nx + CZ * nx * ny) if parity else np.zeros(19, dtype=np.int64)
    cells = wall_list(flags)
    if parity:
        mailbox(F, flags, cells, n, off, 0)
    # all loads of the launch, then all stores: blocks run in any order, and the ranges are
    # disjoint, so this is one valid interleaving (the coverage check makes it the only one needed)
    tiles = []
    for tile in range(ntiles):
        rows = min(R, nrows - tile * R)
        c0 = (row0 + tile * R) * nx
        size = rows * nx
        smem = np.zeros((19, ps))
        for p in range(19):
            a = p * n + c0 + int(sh[p])
            assert 0 <= a and a + size <= 19 * n, "bulk copy out of the array"
            assert (a * esize) % 16 == 0 and (size * esize) % 16 == 0, "bulk copy not 16-byte aligned"
            if cover is not None:
                cover[a:a + size] += 1
            smem[p, :size] = flat[a:a + size]
        tiles.append((c0, size, smem))
    for c0, size, smem in tiles:
        tid = np.arange(size)
        i = tid % nx
        c = c0 + tid
        live = (i >= 1) & (i + 1 < nx) & ((fl[c] & 1) == 0)
        lt = tid[live]
        fin = np.empty((19, lt.size))
        for q in range(19):
            if parity == 0:
                idx = np.full(lt.size, q), lt
            else:
                idx = np.full(lt.size, OPP[q]), lt - CX[q]
            assert np.all((idx[1] >= 0) & (idx[1] < size)), "shared-memory read outside the tile"
            fin[q] = smem[idx]
        fout = collide(fin, omega)
        for q in range(19):
            if parity == 0:
                pl, pos = OPP[q], lt
            else:
                pl, pos = q, lt + CX[q]
            assert np.all((pos >= 0) & (pos < size)), "shared-memory write outside the tile"
            smem[pl, pos] = fout[q]
    for c0, size, smem in tiles:
        for p in range(19):
            a = p * n + c0 + int(sh[p])
            flat[a:a + size] = smem[p, :size]
    if parity:
        mailbox(F, flags, cells, n, off, 1)


def _case(nx, ny, nz, seed, density=0.1):
    rng = np.random.default_rng(seed)
    solid = rng.uniform(size=(nz, ny, nx)) < density
    solid[0] = solid[-1] = True
    solid[:, 0] = solid[:, -1] = True
    solid[:, :, 0] = solid[:, :, -1] = True
    flags = np_aa.link_flags(solid)
    f = np.zeros((19, nz, ny, nx))
    fluid = ~solid
    for q in range(19):
        f[q][fluid] = W[q] * (1.0 + 0.05 * rng.uniform(-1, 1, size=int(fluid.sum())))
        f[q][solid] = rng.uniform(-7, 7, size=int(solid.sum()))  # whatever a solid slot holds
    return flags, f


@pytest.mark.parametrize("nx,ny,nz,esize", [
    (24, 14, 17, 2),    # 10 rows per tile, 21 whole tiles
    (40, 13, 12, 2),    # 6 rows per tile, partial last tile
    (16, 9, 11, 4),     # FP32: 16 rows per tile
    (264, 5, 6, 2),     # one 264-cell row per tile: the 320-cell tile variant
])
def test_row_tiles_match_the_aa_step(nx, ny, nz, esize):
    flags, f0 = _case(nx, ny, nz, seed=nx + ny + nz)
    a, b = f0.copy(), f0.copy()
    n = nx * ny * nz
    fluid = (flags & 1) == 0
    for t in range(6):
        cover = np.zeros(19 * n, dtype=np.int32)
        np_aa.aa_step(a, flags, t, 1.3)
        rows_step(b, flags, t, 1.3, esize, cover)
        assert cover.max() <= 1, "two tiles' ranges overlap"
        # every fluid slot holds the same value (solid slots serve as mailboxes)
        for q in range(19):
            np.testing.assert_array_equal(a[q][fluid], b[q][fluid])


def test_tile_geometry_of_the_workloads():
    # rows per tile / tile capacity of the benchmark lattices (FP16S and FP32)
    assert geometry(256, 256, 256, 2) == (1, 256)
    assert geometry(128, 128, 128, 4) == (2, 256)
    assert geometry(64, 64, 64, 2) == (4, 256)
    assert geometry(96, 96, 96, 4) == (2, 256)
    assert geometry(320, 320, 384, 2) == (1, 320)
    assert rows_per_tile(330, 8, 8, 2, 320) == 0      # longer rows: register-staged kernel
    assert rows_per_tile(36, 8, 8, 2, 256) == 0       # 72-byte rows are not 16-byte multiples
