"""A small numpy AA-pattern stepper (BGK, no forcing) with the step kernel's conventions: cells
x fastest, slots f[q][c], 32-bit flag words with solid-neighbour link bits at bit 8 + q, cells
within one plane + row + 1 of either end never updated.  Test infrastructure for the slab halo
protocol on CPU: every cell is computed elementwise from its own inputs, so a decomposed run is
bit-identical to the undivided one exactly when the halo exchange is right."""
import numpy as np

CX = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0])
CY = np.array([0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1])
CZ = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1])
OPP = np.array([0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15])
W = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)


def link_flags(solid: np.ndarray) -> np.ndarray:
    """[nz, ny, nx] uint32 flag words (SOLID bit + link bits) of a boolean solid mask."""
    fl = solid.astype(np.uint32)
    for q in range(1, 19):
        nb = np.roll(solid, shift=(-CZ[q], -CY[q], -CX[q]), axis=(0, 1, 2))
        fl |= np.where(~solid & nb, np.uint32(1) << np.uint32(8 + q), np.uint32(0)).astype(np.uint32)
    return fl


def aa_step(f: np.ndarray, flags: np.ndarray, t: int, omega: float) -> None:
    """One AA step of f [19, nz, ny, nx] (float64) in place at time t."""
    nz, ny, nx = flags.shape
    n = nz * ny * nx
    F = f.reshape(19, n)
    fl = flags.reshape(n).astype(np.int64)
    c = np.arange(n)
    lo = nx * ny + nx + 1
    live = ((fl & 1) == 0) & (c >= lo) & (c <= n - 1 - lo)
    cells, flc = c[live], fl[live]
    off = CX + CY * nx + CZ * nx * ny
    fin = np.empty((19, cells.size))
    for q in range(19):
        if t % 2 == 0:
            fin[q] = F[q, cells]
        else:
            wall = (q != 0) & (((flc >> (8 + OPP[q])) & 1) == 1)
            fin[q] = np.where(wall, F[q, cells], F[OPP[q], cells - off[q]])
    rho = fin.sum(0)
    ux = (CX[:, None] * fin).sum(0) / rho
    uy = (CY[:, None] * fin).sum(0) / rho
    uz = (CZ[:, None] * fin).sum(0) / rho
    usq = ux * ux + uy * uy + uz * uz
    for q in range(19):
        eu = CX[q] * ux + CY[q] * uy + CZ[q] * uz
        feq = W[q] * rho * (1 + 3 * eu + 4.5 * eu * eu - 1.5 * usq)
        fout = fin[q] - omega * (fin[q] - feq)
        if t % 2 == 0:
            F[OPP[q], cells] = fout
        else:
            wall = (q != 0) & (((flc >> (8 + q)) & 1) == 1)
            flat = np.where(wall, OPP[q] * n + cells, q * n + cells + off[q])
            F.reshape(-1)[flat] = fout
