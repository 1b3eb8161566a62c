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
    if kernel.startswith("k_flux_update") and kernel.endswith(",tg>"):
        # FP32 float pairs, gradients formed in the tile (no gradient array):
        # per face info, area vector and the two reconstruction offsets;
        # per tile face slot the local cell indices, per borrowed slot its
        # face id; per cell the FP32 state (hi, staged once; halo re-reads
        # are neighbour re-reads), lo part, 1/V pair, CSR, and per
        # cell-face the slot, the local neighbour, weights and outward area
        # vector; per distinct halo cell its cell-faces' neighbour and mode;
        # the new pair written; Q^n pair read on stage 1
        nB = getattr(info, "n_borrowed", 0)
        faces = nF * (4 + 8 + 16) + 4 * (nF + nB) + 4 * nB
        tiles = 12 * (nT + 1) + 4 * getattr(info, "n_halo", 0)
        cells = nC * (16 + 16 + 8 + 4 + 32) + tot * (4 + 4 + 8 + 8)
        cells += 4 * getattr(info, "n_halo_cell_faces", 0)
        if stage == 1:
            cells += nC * 32
        return faces + tiles + cells + nT * 9 * 8
    if kernel.startswith("k_cfl_dt_pairs"):
        return nC * (16 + 4 + 8) + tot * 8 + 8 * ((nC + 255) // 256)
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


def kernel_bytes3d(n_cells, n_faces, n_cell_faces, n_tiles, n_borrowed, precision, order,
                   viscous, kernel, stage=0):
    """Algorithmic bytes of one launch of a 3D kernel (kernels3d.inc) under
    R1-R4.  FP32 path (precision 2): geometry and gradient in FP32, the
    state as float pairs (20 B hi + 20 B lo per cell); FP64 paths: FP64
    geometry, gradient and state (40 B per cell)."""
    nC, nF, tot = n_cells, n_faces, n_cell_faces
    s = 4 if precision == 2 else 8
    if kernel.startswith("k3_flux_update"):
        # per face: c0/c1, info, area vector, and for order 2 the two
        # reconstruction offsets (+ eta0 when viscous); the FP32 copies are
        # packed as float4 (S, eta0), (r0, 0), (r1, 0)
        if precision == 2:
            faces = nF * (8 + 4 + 16 + (32 if order == 2 else 0))
        else:
            faces = nF * (8 + 4 + 3 * s + ((6 * s + (s if viscous else 0)) if order == 2 else 0))
        tiles = 8 * (n_tiles + 1) + 4 * n_borrowed
        if precision == 2:
            # state hi (reconstruction), lo (update), Q^n pair on stage 1,
            # new pair written; 1/V pair; CSR; gradient
            cells = nC * (20 + 20 + 40 + 8 + 4) + (nC * 40 if stage == 1 else 0)
        else:
            cells = nC * (40 + 40 + 8 + 4) + (nC * 40 if stage == 1 else 0)
        if order == 2:
            cells += nC * 16 * s  # gradient record: [3][5] + pad
        return faces + tiles + cells + 4 * tot
    if kernel.startswith("k3_gradient"):
        qs = 20 if precision == 2 else 40
        # per cell-face: neighbour, outward S and the two weights (FP32:
        # float4 (S, w0) + w1)
        return nC * (qs + 4 + 8 + 16 * s) + tot * (4 + 5 * s) + 8 * ((nC + 255) // 256)
    return 0


def step_bytes3d(n_cells, n_faces, n_cell_faces, n_tiles, n_borrowed, precision, order,
                 viscous):
    """Algorithmic bytes of one RK2 step of the 3D path (two stages)."""
    b = 0
    for st in (0, 1):
        b += kernel_bytes3d(n_cells, n_faces, n_cell_faces, n_tiles, n_borrowed, precision,
                            order, viscous, "k3_flux_update", stage=st)
        if order == 2:
            b += kernel_bytes3d(n_cells, n_faces, n_cell_faces, n_tiles, n_borrowed, precision,
                                order, viscous, "k3_gradient")
    return b
