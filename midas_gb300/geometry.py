"""Host-side scene preparation for the MIDAS hot path.

The GPU library takes cells (centroids, edge, permittivity) and a CBFM
partition as inputs, exactly as the reference's ``Compute_EFields_*`` receive
them from its L2 geometry layer.  This module builds those inputs:

* ``sphere_cells``     -- the reference's sphere voxeliser
  (src/Discretization.f90:246-310), restated with numpy.
* ``gaussian_sphere``  -- a seeded Gaussian random sphere (log-normal radial
  distance with a Gaussian angular correlation), voxelised on a cubic grid.
* ``cube_cells``       -- an inhomogeneous cube lattice.
* ``box_partition``    -- a bounding-box split into nx*ny*nz blocks; cells are
  reordered so each block is contiguous (as Division_blocks orders them,
  src/Division_blocks.f90:582).
* ``block_contours`` / ``extend_blocks`` -- SetBlockCtrs
  (src/Division_blocks.f90:1616-1662) and Extend_blocks
  (src/Extend_blocks.f90:46-151): neighbours by bounding-sphere distance, then
  every neighbour cell inside the block box grown by ExtLength + Sc/2.
* ``transmitters_un`` / ``init_nipws`` -- getTransmitters_CBFM 'un'
  (src/getParameters_CBFM.f90:34-75) and initializeNipws (:294-348).
"""
from __future__ import annotations

import math

import numpy as np

REF_PI = float(np.arccos(np.float32(-1.0)))   # Pi = Acos(-1.) in single precision (src/Initialization.f90:39)


def sphere_cells(dm: float, sc: float) -> np.ndarray:
    """Cell centroids of the reference sphere voxelisation, in the reference's order."""
    ap = dm / 2.0
    nd = int(math.floor(dm / sc + 0.5))
    q = float(np.float32(0.8)) * ap / float(np.sqrt(np.float32(3.0)))
    next_ = int(math.ceil((ap - q) / sc))
    nint_ = nd - 2 * next_
    api = (nint_ * sc) / 2.0
    sx = [-api, -ap, -ap, api, -api, -api, -ap]
    nx = [nint_, nd, next_, next_, nint_, nint_, nd]
    sy = [-api, -ap, -ap, -ap, -ap, api, -ap]
    ny = [nint_, nd, nd, nd, next_, next_, nd]
    sz = [-api, -ap, -api, -api, -api, -api, api]
    nz = [nint_, next_, nint_, nint_, nint_, nint_, next_]
    out = []
    for d in range(7):
        iz, iy, ix = np.meshgrid(np.arange(1, nz[d] + 1), np.arange(1, ny[d] + 1), np.arange(1, nx[d] + 1),
                                 indexing="ij")
        px = sx[d] + (ix.ravel() - 0.5) * sc
        py = sy[d] + (iy.ravel() - 0.5) * sc
        pz = sz[d] + (iz.ravel() - 0.5) * sc
        if d > 0:
            keep = np.sqrt(px * px + py * py + pz * pz) < ap
            px, py, pz = px[keep], py[keep], pz[keep]
        out.append(np.stack([px, py, pz], axis=1))
    return np.concatenate(out, axis=0)


def _legendre_coeffs(corr_angle_deg: float, lmax: int) -> np.ndarray:
    """Legendre coefficients of the Gaussian correlation exp(-2 sin^2(g/2)/ell^2),
    ell = 2 sin(corr/2), normalised to sum 1."""
    ell = 2.0 * math.sin(math.radians(corr_angle_deg) / 2.0)
    xg, wg = np.polynomial.legendre.leggauss(4 * lmax + 32)
    cg = np.exp(-(1.0 - xg) / ell ** 2)           # 2 sin^2(g/2) = 1 - cos g
    c = np.zeros(lmax + 1)
    for l in range(lmax + 1):
        pl = np.polynomial.legendre.Legendre.basis(l)(xg)
        c[l] = (2 * l + 1) / 2.0 * np.sum(wg * cg * pl)
    c[:2] = 0.0                                   # no translation/rescale modes
    c = np.clip(c, 0.0, None)
    return c / c.sum()


def _real_sph_harm(l: int, m: int, ct: np.ndarray, phi: np.ndarray) -> np.ndarray:
    from scipy.special import lpmv
    am = abs(m)
    norm = math.sqrt((2 * l + 1) / (4 * math.pi) * math.factorial(l - am) / math.factorial(l + am))
    p = lpmv(am, l, ct) * norm
    if m == 0:
        return p
    s = math.sqrt(2.0) * (-1) ** am
    return s * p * (np.cos(am * phi) if m > 0 else np.sin(am * phi))


def gaussian_sphere(a: float, sigma: float, corr_angle_deg: float, d: float, seed: int,
                    lmax: int = 24, ngrid: int = 181) -> np.ndarray:
    """Voxel centroids inside r(u) = a exp(s(u) - sigma^2/2), s a Gaussian field
    on the unit sphere with std sigma and the given correlation angle.

    s is a real spherical-harmonic series with seeded coefficients; r is
    evaluated on an (ngrid x 2 ngrid) theta-phi grid and interpolated bilinearly
    at each voxel direction."""
    rng = np.random.default_rng(seed)
    c = _legendre_coeffs(corr_angle_deg, lmax)
    tg = np.linspace(0.0, np.pi, ngrid)
    pg = np.linspace(-np.pi, np.pi, 2 * ngrid - 1)
    T, P = np.meshgrid(tg, pg, indexing="ij")
    ct, ph = np.cos(T).ravel(), P.ravel()
    s = np.zeros_like(ct)
    for l in range(lmax + 1):
        if c[l] <= 0:
            continue
        sd = sigma * math.sqrt(c[l] * 4 * math.pi / (2 * l + 1))
        for m in range(-l, l + 1):
            s += rng.normal(0.0, sd) * _real_sph_harm(l, m, ct, ph)
    R = (a * np.exp(s - sigma ** 2 / 2.0)).reshape(T.shape)
    rmax = float(R.max()) * 1.001
    n = int(math.ceil(rmax / d))
    g = (np.arange(-n, n) + 0.5) * d
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    p = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    r = np.linalg.norm(p, axis=1)
    p, r = p[r < rmax], r[r < rmax]
    th = np.arccos(np.clip(p[:, 2] / r, -1.0, 1.0))
    phi = np.arctan2(p[:, 1], p[:, 0])
    fi = th / np.pi * (ngrid - 1)
    fj = (phi + np.pi) / (2 * np.pi) * (2 * ngrid - 2)
    i0 = np.clip(np.floor(fi).astype(int), 0, ngrid - 2)
    j0 = np.clip(np.floor(fj).astype(int), 0, 2 * ngrid - 3)
    wi, wj = fi - i0, fj - j0
    rr = (R[i0, j0] * (1 - wi) * (1 - wj) + R[i0 + 1, j0] * wi * (1 - wj) + R[i0, j0 + 1] * (1 - wi) * wj
          + R[i0 + 1, j0 + 1] * wi * wj)
    return np.ascontiguousarray(p[r < rr])


def cube_cells(n_side: int, d: float, n_cells: int | None = None) -> np.ndarray:
    """Cubic lattice of n_side^3 cells of edge d centred on the origin, truncated
    to the first n_cells (x fastest) when given."""
    g = (np.arange(n_side) - (n_side - 1) / 2.0) * d
    Z, Y, X = np.meshgrid(g, g, g, indexing="ij")
    p = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    if n_cells is not None:
        p = p[:n_cells]
    return np.ascontiguousarray(p)


def box_partition(xyz: np.ndarray, nx: int, ny: int, nz: int):
    """Split the bounding box into nx*ny*nz equal boxes.  Returns (perm,
    blk_offsets): xyz[perm] is ordered by block; empty boxes are dropped."""
    lo = xyz.min(axis=0)
    hi = xyz.max(axis=0)
    span = np.where(hi > lo, hi - lo, 1.0)
    ns = np.array([nx, ny, nz])
    ijk = np.minimum(((xyz - lo) / span * ns).astype(int), ns - 1)
    bid = (ijk[:, 2] * ny + ijk[:, 1]) * nx + ijk[:, 0]
    perm = np.argsort(bid, kind="stable")
    counts = np.bincount(bid, minlength=nx * ny * nz)
    counts = counts[counts > 0]
    offs = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
    return perm.astype(np.int64), offs


def block_contours(xyz: np.ndarray, blk_offsets: np.ndarray):
    """SetBlockCtrs: box (min, max per axis) and bounding sphere (centre, radius)."""
    nb = len(blk_offsets) - 1
    box = np.zeros((nb, 2, 3))
    sph = np.zeros((nb, 4))
    for b in range(nb):
        p = xyz[blk_offsets[b]:blk_offsets[b + 1]]
        box[b, 0] = p.min(axis=0)
        box[b, 1] = p.max(axis=0)
        ctr = (box[b, 0] + box[b, 1]) / 2.0
        sph[b, :3] = ctr
        sph[b, 3] = np.sqrt(((p - ctr) ** 2).sum(axis=1)).max()
    return box, sph


def extend_blocks(xyz: np.ndarray, blk_offsets: np.ndarray, ext_length: float, sc: float):
    """Extend_blocks: global indices of the extension cells of each block."""
    nb = len(blk_offsets) - 1
    box, sph = block_contours(xyz, blk_offsets)
    ext = []
    for b in range(nb):
        lo = box[b, 0] - ext_length - sc / 2.0
        hi = box[b, 1] + ext_length + sc / 2.0
        cells = []
        for bp in range(nb):
            if bp == b:
                continue
            dis = math.sqrt(((sph[bp, :3] - sph[b, :3]) ** 2).sum())
            if dis > sph[b, 3] + sph[bp, 3] + ext_length:
                continue
            idx = np.arange(blk_offsets[bp], blk_offsets[bp + 1])
            p = xyz[idx]
            inside = np.all((lo <= p) & (p <= hi), axis=1)
            cells.append(idx[inside])
        ext.append(np.concatenate(cells).astype(np.int32) if cells else np.zeros(0, np.int32))
    return ext


def transmitters_un(niws: int):
    """getTransmitters_CBFM for the 'un' distribution: (theta_deg, phi_deg)."""
    df = np.float32(291600.0) + np.float32(4 * (niws - 1) * (360 * 180))
    delta = float(df)
    step = ((360.0 + 180.0) + math.sqrt(delta)) / (2.0 * (niws - 1))
    nth = int(math.floor(180.0 / step + 0.5)) + 1
    nph = int(math.floor(360.0 / step + 0.5)) + 1
    step_ph = 360.0 / (nph - 1)
    margin = math.cos(180.0 * REF_PI / 180.0) - math.cos(0.0)
    step_th = margin / (nth - 1)
    th, ph = [], []
    for i in range(nph):
        for k in range(nth):
            v = max(1.0 * k * step_th + 1.0, -1.0)
            th.append(math.acos(v) * 180.0 / REF_PI)
            ph.append(i * step_ph)
    return np.array(th), np.array(ph)


def init_nipws(r_lambda: float, niws_input: int = 0) -> int:
    """initializeNipws for the 'un' distribution (src/Initialization.f90:58)."""
    tab = [91, 190, 190, 231, 325, 496, 703, 861]
    niws = None
    for rr in range(1, 9):
        if r_lambda <= rr:
            niws = tab[rr - 1]
            break
    if niws is None:
        niws = tab[3]
    return max(niws_input, niws)


def random_directions(n: int, seed: int):
    """Seeded directions uniform on the sphere, in MIDAS angles (degrees)."""
    rng = np.random.default_rng(seed)
    u = rng.uniform(-1.0, 1.0, n)
    phi = rng.uniform(0.0, 360.0, n)
    return np.degrees(np.arccos(u)), phi


def uniform_directions(th0: float, th1: float, nth: int, ph0: float, ph1: float, nph: int):
    """Uniform-step direction grid in degrees, theta fastest (get_trans_Receiv,
    src/get_trans_Receiv.f90:249-270 for transmitters, :509-524 for receivers)."""
    sth = 0.0 if nth == 1 else (th1 - th0) / (nth - 1)
    sph = 0.0 if nph == 1 else (ph1 - ph0) / (nph - 1)
    th = th0 + np.arange(nth) * sth
    ph = ph0 + np.arange(nph) * sph
    return np.tile(th, nph), np.repeat(ph, nth)


def receivers_with_extras(rx_th, rx_ph, tr_th, tr_ph):
    """Append, for each transmitter, its forward and backward scattering
    direction when the receiver grid lacks it (src/get_trans_Receiv.f90:571-590:
    getTxRxIndex over the grid only, tolerance 1e-2 degree)."""
    rx_th, rx_ph = np.asarray(rx_th, np.float64), np.asarray(rx_ph, np.float64)
    eps = float(np.float32(1e-2))
    extra_th, extra_ph = [], []

    def on_grid(t, p):
        return bool(np.any((np.abs(rx_th - t) <= eps) & (np.abs(rx_ph - p) <= eps)))

    for t, p in zip(np.asarray(tr_th, np.float64), np.asarray(tr_ph, np.float64)):
        for a, b in ((t, p), (180.0 - t, math.fmod(p + 180.0, 360.0))):
            if not on_grid(a, b):
                extra_th.append(a)
                extra_ph.append(b)
    return np.concatenate([rx_th, extra_th]), np.concatenate([rx_ph, extra_ph])


def gauss_legendre_directions(th0: float, th1: float, nth: int, ph0: float, ph1: float, nph: int):
    """Gauss-Legendre direction grid in degrees (theta fastest) and its weights
    for the 'gl' rule: theta weights then phi weights on the radian intervals
    (the phi weight is 1 for a single phi, src/Compute_Scattering_Quantities.f90:279-283)."""
    def rule(n, a, b):
        x, w = np.polynomial.legendre.leggauss(n)
        return (a + b) / 2 + (b - a) / 2 * x, (b - a) / 2 * w
    xt, wt = rule(nth, math.radians(th0), math.radians(th1))
    if nph > 1:
        xp, wp = rule(nph, math.radians(ph0), math.radians(ph1))
    else:
        xp, wp = np.array([math.radians(ph0)]), np.array([1.0])
    th, ph = np.degrees(xt), np.degrees(xp)
    return np.tile(th, nph), np.repeat(ph, nth), np.concatenate([wt, wp])


def list_receivers_with_extras(rx_th, rx_ph, tr_th, tr_ph):
    """Receiver list of the 'sd' / 'lb' / 'rf' rules: the NRx directions, then the
    forward direction of every transmitter, then every backward direction
    (src/get_trans_Receiv.f90:527-550) -- the positional layout that
    Compute_Scattering_Quantities_2 indexes (NRx + t, NRx + NTr + t)."""
    tr_th, tr_ph = np.asarray(tr_th, np.float64), np.asarray(tr_ph, np.float64)
    return (np.concatenate([np.asarray(rx_th, np.float64), tr_th, 180.0 - tr_th]),
            np.concatenate([np.asarray(rx_ph, np.float64), tr_ph, np.fmod(tr_ph + 180.0, 360.0)]))


def _unit(rng) -> np.ndarray:
    v = rng.normal(size=3)
    return v / np.linalg.norm(v)


def fractal_aggregate(n_mono: int, a: float = 1.0, df: float = 1.8, kf: float = 1.3, seed: int = 0,
                      tries: int = 400) -> np.ndarray:
    """Monomer centres of a seeded aggregate of n_mono touching spheres of radius a,
    grown by tunable particle-cluster aggregation: each new monomer is placed at
    the distance Gamma from the cluster's centre of mass that keeps the fractal law
    N = kf (Rg / a)^df exact, touching one monomer and overlapping none.  With
    Rg_N^2 the mean squared distance of the N centres from their centroid, adding
    one centre at distance Gamma gives (N+1) Rg_{N+1}^2 = N Rg_N^2 + N Gamma^2/(N+1),
    so Gamma^2 = (N+1)/N ((N+1) Rg_{N+1}^2 - N Rg_N^2).  Where no touching position
    reaches Gamma (small N, or a crowded shell), the touching, non-overlapping
    position closest to it is taken."""
    rng = np.random.default_rng(seed)
    pos = [np.zeros(3), 2.0 * a * _unit(rng)]
    d_min = 2.0 * a * (1.0 - 1e-9)
    while len(pos) < n_mono:
        P = np.array(pos)
        N = len(P)
        c = P.mean(axis=0)
        rg2 = float(np.mean(np.sum((P - c) ** 2, axis=1)))
        target = a * a * ((N + 1) / kf) ** (2.0 / df)
        gamma = math.sqrt(max((N + 1) / N * ((N + 1) * target - N * rg2), 0.0))
        dist = np.linalg.norm(P - c, axis=1)
        cand = np.flatnonzero((np.abs(dist - gamma) <= 2.0 * a) & (dist > 1e-12))
        placed = None
        for _ in range(tries if cand.size else 0):
            j = int(rng.choice(cand))
            D = dist[j]
            e = (P[j] - c) / D
            h = (D * D + gamma * gamma - 4.0 * a * a) / (2.0 * D)   # circle of the two spheres
            rho = math.sqrt(max(gamma * gamma - h * h, 0.0))
            u = np.cross(e, _unit(rng))
            u /= np.linalg.norm(u)
            v = np.cross(e, u)
            phi = rng.uniform(0.0, 2.0 * math.pi)
            p = c + h * e + rho * (math.cos(phi) * u + math.sin(phi) * v)
            if np.min(np.linalg.norm(P - p, axis=1)) >= d_min:
                placed = p
                break
        if placed is None:   # closest feasible touching position
            best, best_err = None, math.inf
            for _ in range(tries):
                p = P[int(rng.integers(N))] + 2.0 * a * _unit(rng)
                if np.min(np.linalg.norm(P - p, axis=1)) < d_min:
                    continue
                err = abs(np.linalg.norm(p - c) - gamma)
                if err < best_err:
                    best, best_err = p, err
            placed = best
        if placed is None:
            raise RuntimeError("fractal_aggregate: no free touching position")
        pos.append(placed)
    P = np.array(pos)
    return P - P.mean(axis=0)


def voxelise_spheres(centres: np.ndarray, a: float, cells_per_diameter: int = 6):
    """Cubic cells of edge 2a / cells_per_diameter whose centres lie strictly inside
    one of the spheres (the reference's inside test for its sphere voxeliser,
    src/Discretization.f90:246-310).  Returns (xyz, edge)."""
    d = 2.0 * a / cells_per_diameter
    lo = centres.min(axis=0) - a
    dims = np.ceil((centres.max(axis=0) + a - lo) / d).astype(int) + 1
    mask = np.zeros(dims, bool)
    r = int(math.ceil(a / d)) + 1
    off = np.arange(-r, r + 1)
    for cen in centres:
        base = np.floor((cen - lo) / d).astype(int)
        idx = [np.clip(base[k] + off, 0, dims[k] - 1) for k in range(3)]
        gx, gy, gz = np.meshgrid(*idx, indexing="ij")
        px, py, pz = (lo[k] + (g + 0.5) * d for k, g in enumerate((gx, gy, gz)))
        inside = (px - cen[0]) ** 2 + (py - cen[1]) ** 2 + (pz - cen[2]) ** 2 < a * a
        mask[gx[inside], gy[inside], gz[inside]] = True
    ijk = np.argwhere(mask)
    return lo + (ijk + 0.5) * d, d
