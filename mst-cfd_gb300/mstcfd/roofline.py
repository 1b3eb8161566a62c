"""Algorithmic bytes per kernel launch (the HBM-roofline numerator).

Rules, applied to the actual array sizes of a mesh:
  R1  every persistent array a kernel reads counts once per launch, at its
      stored width (neighbour states and faces read by two cells count once);
  R2  every array it writes counts once;
  R3  re-reads of neighbour data within one launch are free (cache);
  R4  intermediates kept on chip (face fluxes in shared memory) are free.
A cell-update is one residual evaluation plus one state update of one cell
(one Runge-Kutta stage), so an RK2 step is two cell-updates per cell.
"""


def _sizes(info, precision):
    s = 4 if precision == 2 else 8  # geometry / gradient width
    return dict(nC=info.n_cells, nF=info.n_faces, tot=info.n_cell_faces,
                nT=info.n_tiles, s=s)


def kernel_bytes(info, precision, order, kernel, stage=0, n_borrowed=None):
    """Algorithmic bytes of one launch of ``kernel`` on a mesh with
    mst_mesh_info ``info``."""
    z = _sizes(info, precision)
    nC, nF, tot, nT, s = z["nC"], z["nF"], z["tot"], z["nT"], z["s"]
    q = 32  # double4 state
    if kernel.startswith("k_flux_update"):
        faces = nF * (8 + 4 + 2 * s + (4 * s if order == 2 else 0))
        tiles = 8 * (nT + 1) + 4 * (n_borrowed or 0)
        cells = nC * (q + 4 + 8 + q) + 4 * tot + (nC * 8 * s if order == 2 else 0)
        if stage == 1:
            cells += nC * q
        return faces + tiles + cells + nT * 9 * 8
    if kernel.startswith("k_gradient"):
        # state (the FP32 path reads its 16-byte FP32 copy), CSR, 1/V,
        # gradient write, per cell-face neighbour index, weights and the
        # outward area vector
        qs = 16 if precision == 2 else q
        return nC * (qs + 4 + 8 + 8 * s) + tot * (4 + 2 * s + 2 * s)
    if kernel.startswith("k_spectral_dt"):
        return nC * (q + 4 + 8) + tot * 2 * s + 8 * ((nC + 255) // 256)
    return 0


def step_bytes(info, precision, order, rk2=True, cfl=True):
    """Algorithmic bytes of one time step (all launches)."""
    b = 0
    stages = (0, 1) if rk2 else (0,)
    for st in stages:
        b += kernel_bytes(info, precision, order, "k_flux_update", stage=st)
        if order == 2:
            b += kernel_bytes(info, precision, order, "k_gradient")
    if cfl:
        b += kernel_bytes(info, precision, order, "k_spectral_dt")
    return b
