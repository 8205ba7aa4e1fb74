"""Seeded synthetic ICON-like regional grids and terrain.

The reference is exercised on ICON grids and EXTPAR topography files
(verification.py:81-104) that are not public. This module generates inputs of
the same form -- FP64 cell circumcentres ``clon/clat`` [rad], vertices
``vlon/vlat`` [rad], ``cells_of_vertex`` (6, nvertex) int32 with -2 for a
missing neighbour, and cell elevations ``hsurf`` [m] -- for the domain shapes
the benchmarks name:

* the grid is a uniform n-section (``root * 2**bisections``) of one spherical
  icosahedron face whose centre lies at the domain centre, projected radially
  onto the unit sphere (ICON's RnBk construction without its per-level
  re-projection and spring smoothing), cropped to a lat/lon box;
* cells are the lattice triangles with all three vertices inside the box; a
  cell's centre is the circumcentre of its spherical triangle;
* ``cells_of_vertex`` lists a vertex's cells in rotational order with the
  valid entries first and -2 after them (the layout on which the reference's
  mesh builder is defined, mo_lradtopo_horayzon.cpp:246-271);
* elevation is a sum of spectral fractional-Brownian fields, Gaussian peaks,
  Gaussian ridges and ridged noise, evaluated at the ICON vertices and scaled
  to a target range; each cell gets the mean of its three vertices.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

R_EARTH = 6371229.0  # ICON/COSMO Earth radius [m] (mo_lradtopo_horayzon.cpp:584)

# Icosahedron on the unit sphere: edge chord and inradius (face-plane distance).
_ICO_EDGE = 4.0 / math.sqrt(10.0 + 2.0 * math.sqrt(5.0))
_ICO_INRADIUS = _ICO_EDGE * (3.0 + math.sqrt(5.0)) / (4.0 * math.sqrt(3.0))
_ICO_FACE_RHO = math.acos(_ICO_INRADIUS)  # face centre -> face vertex angle


@dataclass
class Domain:
    """One regional ICON-like domain in the reference's input layout."""

    clon: np.ndarray
    clat: np.ndarray
    hsurf: np.ndarray
    vlon: np.ndarray
    vlat: np.ndarray
    cells_of_vertex: np.ndarray
    vertex_of_cell: np.ndarray
    meta: dict = field(default_factory=dict)

    @property
    def ncell(self) -> int:
        return int(self.clon.size)

    @property
    def nvertex(self) -> int:
        return int(self.vlon.size)

    def inputs(self):
        """Positional inputs of ``horizon_svf_comp_py`` (pyx:15-20)."""
        return (self.clon, self.clat, self.hsurf, self.vlon, self.vlat,
                self.cells_of_vertex)


def _basis(lat0: float, lon0: float):
    c = np.array([math.cos(lat0) * math.cos(lon0), math.cos(lat0) * math.sin(lon0),
                  math.sin(lat0)])
    e = np.array([-math.sin(lon0), math.cos(lon0), 0.0])
    n = np.cross(c, e)
    return c, e, n


def choose_division(edge_km: float) -> tuple[int, int]:
    """(root, bisections) whose n-section of a face gives ~edge_km edges."""
    target = R_EARTH / 1000.0 * _ICO_EDGE / _ICO_INRADIUS / edge_km
    best = None
    for bis in range(0, 24):
        root = max(1, int(round(target / 2 ** bis)))
        if root > 48:
            continue
        err = abs(root * 2 ** bis - target) / target
        key = (err > 0.03, -bis if err <= 0.03 else err)
        if best is None or key < best[0]:
            best = (key, root, bis)
    return best[1], best[2]


def icon_like_grid(lat0_deg: float, lon0_deg: float, box_km: float,
                   edge_km: float, face_rotation_deg: float = 0.0) -> dict:
    """Lattice grid of one icosahedron face cropped to a lat/lon box.

    The box is ``box_km`` wide in latitude and, at the centre latitude, in
    longitude. Returns the grid arrays plus per-vertex local coordinates
    (x east, y north, in m on the tangent plane) for terrain evaluation.
    """
    lat0, lon0 = math.radians(lat0_deg), math.radians(lon0_deg)
    c, e, n = _basis(lat0, lon0)
    rho = _ICO_FACE_RHO
    th0 = math.radians(face_rotation_deg)
    face = [math.cos(rho) * c + math.sin(rho) * (math.cos(th0 + k * 2 * math.pi / 3) * n
                                                 + math.sin(th0 + k * 2 * math.pi / 3) * e)
            for k in range(3)]
    A, B, C = face
    root, bis = choose_division(edge_km)
    N = root * 2 ** bis

    half_lat = box_km * 1000.0 / R_EARTH / 2.0
    half_lon = half_lat / math.cos(lat0)
    lat_lo, lat_hi = lat0 - half_lat, lat0 + half_lat
    lon_lo, lon_hi = lon0 - half_lon, lon0 + half_lon

    # Barycentric range of the box boundary on the face plane.
    t = np.linspace(0.0, 1.0, 257)
    blat = np.concatenate([np.full_like(t, lat_lo), np.full_like(t, lat_hi),
                           lat_lo + t * (lat_hi - lat_lo), lat_lo + t * (lat_hi - lat_lo)])
    blon = np.concatenate([lon_lo + t * (lon_hi - lon_lo), lon_lo + t * (lon_hi - lon_lo),
                           np.full_like(t, lon_lo), np.full_like(t, lon_hi)])
    q = np.stack([np.cos(blat) * np.cos(blon), np.cos(blat) * np.sin(blon), np.sin(blat)], 1)
    fc = (A + B + C) / np.linalg.norm(A + B + C)
    qp = q * (np.dot(A, fc) / (q @ fc))[:, None]
    M = np.stack([B - A, C - A], 1)  # 3x2
    st, *_ = np.linalg.lstsq(M, (qp - A).T, rcond=None)
    imin = max(0, int(math.floor(st[0].min() * N)) - 2)
    imax = min(N, int(math.ceil(st[0].max() * N)) + 2)
    jmin = max(0, int(math.floor(st[1].min() * N)) - 2)
    jmax = min(N, int(math.ceil(st[1].max() * N)) + 2)
    if imin >= imax or jmin >= jmax:
        raise ValueError("box does not overlap the icosahedron face")

    ni, nj = imax - imin + 1, jmax - jmin + 1
    ii, jj = np.meshgrid(np.arange(imin, imax + 1), np.arange(jmin, jmax + 1))  # (nj, ni)
    valid = (ii + jj) <= N
    P = (A[None, None, :] + (ii[..., None] / N) * (B - A)[None, None, :]
         + (jj[..., None] / N) * (C - A)[None, None, :])
    P /= np.linalg.norm(P, axis=-1, keepdims=True)
    plat = np.arcsin(np.clip(P[..., 2], -1.0, 1.0))
    plon = np.arctan2(P[..., 1], P[..., 0])
    inbox = valid & (plat >= lat_lo) & (plat <= lat_hi) & (plon >= lon_lo) & (plon <= lon_hi)

    # Cells: up (i,j),(i+1,j),(i,j+1) and down (i+1,j),(i+1,j+1),(i,j+1).
    ok = np.zeros((nj + 1, ni + 1), dtype=bool)
    ok[:nj, :ni] = inbox
    up = ok[:-1, :-1] & ok[:-1, 1:] & ok[1:, :-1]
    dn = ok[:-1, 1:] & ok[1:, 1:] & ok[1:, :-1]
    up[-1, :] = False
    up[:, -1] = False
    dn[-1, :] = False
    dn[:, -1] = False

    # Cell numbering: row by row, up then down at each (i, j).
    kind = np.stack([up, dn], -1)  # (nj, ni, 2)
    cell_id = np.full(kind.shape, -1, dtype=np.int64)
    cell_id[kind] = np.arange(int(kind.sum()))
    ncell = int(kind.sum())
    if ncell == 0:
        raise ValueError("empty domain")

    # Vertices used by at least one cell, numbered row by row.
    used = up.copy()
    used[:, 1:] |= up[:, :-1] | dn[:, :-1]
    used[1:, :] |= up[:-1, :] | dn[:-1, :]
    used[1:, 1:] |= dn[:-1, :-1]
    vert_id = np.full((nj, ni), -1, dtype=np.int64)
    vert_id[used] = np.arange(int(used.sum()))
    nvert = int(used.sum())

    # vertex_of_cell (3, ncell)
    jc, ic, kc = np.nonzero(kind)
    order = np.argsort(cell_id[jc, ic, kc])
    jc, ic, kc = jc[order], ic[order], kc[order]
    v0 = np.where(kc == 0, vert_id[jc, ic], vert_id[jc, ic + 1])
    v1 = np.where(kc == 0, vert_id[jc, ic + 1], vert_id[jc + 1, ic + 1])
    v2 = vert_id[jc + 1, ic]
    vertex_of_cell = np.stack([v0, v1, v2]).astype(np.int32)

    Pv = P[used]
    vlat = np.arcsin(np.clip(Pv[:, 2], -1.0, 1.0))
    vlon = np.arctan2(Pv[:, 1], Pv[:, 0])

    # Circumcentres of the spherical triangles.
    a, b, cc = Pv[v0], Pv[v1], Pv[v2]
    cen = np.cross(b - a, cc - a)
    cen /= np.linalg.norm(cen, axis=1, keepdims=True)
    cen *= np.sign(np.einsum("ij,ij->i", cen, a))[:, None]
    clat = np.arcsin(np.clip(cen[:, 2], -1.0, 1.0))
    clon = np.arctan2(cen[:, 1], cen[:, 0])

    # cells_of_vertex in rotational order around (i, j).
    def cid(jo, io, k):
        jx, ix = jv + jo, iv + io
        inside = (jx >= 0) & (jx < nj) & (ix >= 0) & (ix < ni)
        out = np.full(jv.shape, -2, dtype=np.int64)
        out[inside] = cell_id[jx[inside], ix[inside], k]
        out[out < 0] = -2
        return out

    jv, iv = np.nonzero(used)
    ring = np.stack([cid(0, 0, 0), cid(0, -1, 1), cid(0, -1, 0),
                     cid(-1, -1, 1), cid(-1, 0, 0), cid(-1, 0, 1)])  # (6, nvert)
    # Valid entries first (stable), -2 after them.
    key = (ring == -2).astype(np.int8)
    perm = np.argsort(key, axis=0, kind="stable")
    cov = np.take_along_axis(ring, perm, axis=0).astype(np.int32)

    # Local tangent-plane coordinates [m] for terrain evaluation.
    vx = R_EARTH * (Pv @ e)
    vy = R_EARTH * (Pv @ n)
    return dict(clon=clon, clat=clat, vlon=vlon, vlat=vlat, cells_of_vertex=cov,
                vertex_of_cell=vertex_of_cell, vx=vx, vy=vy,
                meta=dict(root=root, bisections=bis, division=N,
                          lat0_deg=lat0_deg, lon0_deg=lon0_deg, box_km=box_km,
                          edge_km=edge_km))


# ----------------------------------------------------------------------------
# Terrain
# ----------------------------------------------------------------------------

def fbm_field(n: int, hurst: float, rng: np.random.Generator) -> np.ndarray:
    """Periodic spectral fBm on an n x n grid, zero mean, unit std."""
    kx = np.fft.fftfreq(n)
    ky = np.fft.rfftfreq(n)
    k = np.sqrt(kx[:, None] ** 2 + ky[None, :] ** 2)
    amp = np.zeros_like(k)
    amp[k > 0] = k[k > 0] ** (-(hurst + 1.0))
    spec = amp * (rng.standard_normal(k.shape) + 1j * rng.standard_normal(k.shape))
    f = np.fft.irfft2(spec, s=(n, n))
    f -= f.mean()
    f /= f.std() + 1e-30
    return f


def _sample(field_: np.ndarray, x: np.ndarray, y: np.ndarray, extent: float) -> np.ndarray:
    """Bilinear sample of a periodic field covering [-extent/2, extent/2]^2."""
    n = field_.shape[0]
    u = (x / extent + 0.5) * n
    v = (y / extent + 0.5) * n
    i0 = np.floor(u).astype(np.int64)
    j0 = np.floor(v).astype(np.int64)
    fu, fv = u - i0, v - j0
    i0 %= n
    j0 %= n
    i1, j1 = (i0 + 1) % n, (j0 + 1) % n
    return ((1 - fu) * (1 - fv) * field_[j0, i0] + fu * (1 - fv) * field_[j0, i1]
            + (1 - fu) * fv * field_[j1, i0] + fu * fv * field_[j1, i1])


def _rescale(h: np.ndarray, lo: float, hi: float) -> np.ndarray:
    a, b = float(h.min()), float(h.max())
    if b - a <= 0:
        return np.full_like(h, lo)
    return lo + (h - a) * ((hi - lo) / (b - a))


def terrain(vx: np.ndarray, vy: np.ndarray, box_m: float, kind: str,
            rng: np.random.Generator, hmin: float, hmax: float,
            hurst: float = 0.8, n_features: int = 0, field_n: int = 2048) -> np.ndarray:
    """Vertex elevations [m] for the terrain recipes of the benchmark configs.

    kind: ``"fbm_peaks"`` (fBm in [hmin, hmax] plus Gaussian peaks),
    ``"fbm_ridges"`` (fBm plus Gaussian ridges, rescaled), ``"fbm_ridged"``
    (fBm plus ridged noise, rescaled), ``"eroded"`` (fBm plus sharper ridged
    noise, rescaled).
    """
    extent = box_m * 1.25
    base = _sample(fbm_field(field_n, hurst, rng), vx, vy, extent)
    if kind == "fbm_peaks":
        h = _rescale(base, hmin, hmax)
        for _ in range(n_features):
            cx, cy = rng.uniform(-box_m / 2, box_m / 2, 2)
            sig = rng.uniform(5e3, 30e3)
            amp = rng.uniform(500.0, 1500.0)
            h = h + amp * np.exp(-((vx - cx) ** 2 + (vy - cy) ** 2) / (2 * sig * sig))
        return h
    if kind == "fbm_ridges":
        h = _rescale(base, 0.0, 1.0)
        for _ in range(n_features):
            cx, cy = rng.uniform(-box_m / 2, box_m / 2, 2)
            ang = rng.uniform(0, math.pi)
            length = rng.uniform(50e3, 300e3)
            sig = rng.uniform(3e3, 15e3)
            amp = rng.uniform(0.3, 1.0)
            dx, dy = math.cos(ang), math.sin(ang)
            s = np.clip((vx - cx) * dx + (vy - cy) * dy, -length / 2, length / 2)
            d2 = (vx - cx - s * dx) ** 2 + (vy - cy - s * dy) ** 2
            h = h + amp * np.exp(-d2 / (2 * sig * sig))
        return _rescale(h, hmin, hmax)
    if kind in ("fbm_ridged", "eroded"):
        g = _sample(fbm_field(field_n, 0.9, rng), vx, vy, extent)
        g = g / (np.abs(g).max() + 1e-30)
        power = 2.0 if kind == "fbm_ridged" else 3.0
        ridged = (1.0 - np.abs(g)) ** power
        h = 0.55 * _rescale(base, 0.0, 1.0) + 0.45 * _rescale(ridged, 0.0, 1.0)
        return _rescale(h, hmin, hmax)
    raise ValueError("unknown terrain kind %r" % kind)


# ----------------------------------------------------------------------------
# Benchmark configurations
# ----------------------------------------------------------------------------

CONFIGS = {
    # 2.5 km grid, 400 x 400 km, fBm H=0.8 in 0-3000 m + 20 Gaussian peaks.
    "c1": dict(edge_km=2.5, box_km=400.0, kind="fbm_peaks", hmin=0.0, hmax=3000.0,
               hurst=0.8, n_features=20),
    # 1 km grid, 1000 x 1000 km, fBm + 60 Gaussian ridges, 0-4500 m.
    "c2": dict(edge_km=1.0, box_km=1000.0, kind="fbm_ridges", hmin=0.0, hmax=4500.0,
               hurst=0.8, n_features=60),
    # 500 m grid, 600 x 600 km, fBm H=0.7 + ridged noise, 200-4800 m.
    "c3": dict(edge_km=0.5, box_km=600.0, kind="fbm_ridged", hmin=200.0, hmax=4800.0,
               hurst=0.7, n_features=0),
    # 100 m grid, 150 x 150 km, fBm + erosion-like ridged noise, 500-4200 m.
    "c4": dict(edge_km=0.1, box_km=150.0, kind="eroded", hmin=500.0, hmax=4200.0,
               hurst=0.8, n_features=0),
}


def make_domain(edge_km: float, box_km: float, kind: str = "fbm_peaks",
                hmin: float = 0.0, hmax: float = 3000.0, hurst: float = 0.8,
                n_features: int = 20, seed: int = 0, lat0_deg: float = 46.0,
                lon0_deg: float = 8.0, face_rotation_deg: float = 0.0,
                field_n: int | None = None) -> Domain:
    """Build one seeded synthetic domain (grid + terrain)."""
    g = icon_like_grid(lat0_deg, lon0_deg, box_km, edge_km, face_rotation_deg)
    rng = np.random.default_rng(seed)
    if field_n is None:
        # ~2 field samples per grid edge, between 256 and 4096 per side.
        field_n = int(2 ** np.clip(np.ceil(np.log2(1.25 * box_km / edge_km * 2)), 8, 12))
    hv = terrain(g["vx"], g["vy"], box_km * 1000.0, kind, rng, hmin, hmax, hurst,
                 n_features, field_n)
    voc = g["vertex_of_cell"]
    hsurf = (hv[voc[0]] + hv[voc[1]] + hv[voc[2]]) / 3.0
    meta = dict(g["meta"], kind=kind, hmin=hmin, hmax=hmax, hurst=hurst,
                n_features=n_features, seed=seed)
    return Domain(clon=g["clon"], clat=g["clat"], hsurf=hsurf, vlon=g["vlon"],
                  vlat=g["vlat"], cells_of_vertex=g["cells_of_vertex"],
                  vertex_of_cell=voc, meta=meta)


def make_config(name: str, seed: int = 0, **overrides) -> Domain:
    """Domain of a named benchmark configuration (``c1`` .. ``c4``)."""
    cfg = dict(CONFIGS[name])
    cfg.update(overrides)
    d = make_domain(seed=seed, **cfg)
    d.meta["config"] = name
    return d


def make_batch(n_domains: int = 64, seed: int = 0, min_cells: float = 1e4,
               max_cells: float = 5e5, scale: float = 1.0):
    """Uneven batch of independent regional domains.

    Sizes are log-uniform in [min_cells, max_cells] (times ``scale``), grid
    spacing uniform in 0.5-2.5 km, each domain with its own terrain seed,
    relief 1000-4500 m and num_hori drawn from {16, 24, 36}. Domain centres
    are spread over mid-latitudes. Returns a list of (Domain, args) with args
    = (num_hori, grid_type, dist_search, ray_org_elev, refine_factor, svf_type).
    """
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_domains):
        target = float(np.exp(rng.uniform(np.log(min_cells), np.log(max_cells)))) * scale
        edge = float(rng.uniform(0.5, 2.5))
        box = math.sqrt(target * (math.sqrt(3.0) / 4.0) * edge * edge)
        relief = float(rng.uniform(1000.0, 4500.0))
        hmin = float(rng.uniform(0.0, 800.0))
        kind = ["fbm_peaks", "fbm_ridged", "eroded"][int(rng.integers(3))]
        d = make_domain(edge_km=edge, box_km=box, kind=kind, hmin=hmin, hmax=hmin + relief,
                        hurst=float(rng.uniform(0.6, 0.9)), n_features=int(rng.integers(0, 20)),
                        seed=seed * 1000 + i + 1, lat0_deg=float(rng.uniform(-60, 60)),
                        lon0_deg=float(rng.uniform(-160, 160)),
                        face_rotation_deg=float(rng.uniform(0, 120)))
        nhori = int(rng.choice([16, 24, 36]))
        d.meta["config"] = "batch"
        out.append((d, (nhori, 1, 40000.0, 0.2, 1, 2)))
    return out
