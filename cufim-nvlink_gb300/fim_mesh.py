"""Synthetic tetrahedral meshes and conduction fields for the solver's
workloads (seeded, deterministic).

* ``kuhn_box``      -- a box of nx*ny*nz cubes, each cut into 6 Kuhn tets
                       (Freudenthal triangulation, conforming across cubes),
                       interior vertices jittered by U[-j*h, j*h] per axis.
* ``slab_case``     -- the anisotropic slab: fibres in the xy-plane rotating
                       with z, cf/ct per tet, a spherical slow scar and random
                       surface stimuli with t0 ~ U[0, 10].
* ``cube_case``     -- the unit cube, isotropic 0.6, one stimulus at the
                       origin with t0 = 0.
* ``batch_cases``   -- uneven Kuhn boxes with per-solve conduction draws.

Units: lengths in mm, speeds in mm/ms, times in ms (any consistent unit
system works; the reference's own files are in um, um/us and us).
"""
import math

import numpy as np

# the six Kuhn tets of the unit cube: corners as bit triples (x, y, z)
_KUHN_PATHS = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]


def kuhn_box(nx, ny, nz, lx=1.0, ly=1.0, lz=1.0, jitter=0.2, seed=1, origin=(0.0, 0.0, 0.0)):
    """Return (xyz float64 [nV,3], tets int32 [nT,4]) for a Kuhn box mesh."""
    hx, hy, hz = lx / nx, ly / ny, lz / nz
    ix = np.arange(nx + 1)
    iy = np.arange(ny + 1)
    iz = np.arange(nz + 1)
    Z, Y, X = np.meshgrid(iz, iy, ix, indexing="ij")
    xyz = np.stack([X.ravel() * hx, Y.ravel() * hy, Z.ravel() * hz], axis=1).astype(np.float64)
    xyz += np.asarray(origin, dtype=np.float64)
    if jitter > 0:
        rng = np.random.default_rng(seed)
        jit = rng.uniform(-jitter, jitter, size=xyz.shape) * np.array([hx, hy, hz])
        interior = ((X.ravel() > 0) & (X.ravel() < nx) & (Y.ravel() > 0) & (Y.ravel() < ny) &
                    (Z.ravel() > 0) & (Z.ravel() < nz))
        xyz[interior] += jit[interior]

    def vid(i, j, k):
        return i + (nx + 1) * (j + (ny + 1) * k)

    ci, cj, ck = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    ci, cj, ck = ci.ravel(order="F"), cj.ravel(order="F"), ck.ravel(order="F")
    tets = []
    for path in _KUHN_PATHS:
        corner = [np.zeros(3, dtype=np.int64)]
        c = np.zeros(3, dtype=np.int64)
        for ax in path:
            c = c.copy()
            c[ax] = 1
            corner.append(c)
        t = np.stack([vid(ci + cc[0], cj + cc[1], ck + cc[2]) for cc in corner], axis=1)
        tets.append(t)
    tets = np.stack(tets, axis=1).reshape(-1, 4).astype(np.int32)
    return xyz, tets


def tet_centroids(xyz, tets):
    return xyz[tets].mean(axis=1)


def surface_vertices(xyz, tol=1e-12):
    lo = xyz.min(axis=0)
    hi = xyz.max(axis=0)
    on = np.any((np.abs(xyz - lo) < tol) | (np.abs(xyz - hi) < tol), axis=1)
    return np.nonzero(on)[0].astype(np.int32)


def cube_case(n=20, jitter=0.2, seed=1, speed=0.6):
    """Unit cube, n^3 cubes x 6 Kuhn tets, isotropic speed, stimulus at (0,0,0), t0 = 0."""
    xyz, tets = kuhn_box(n, n, n, 1.0, 1.0, 1.0, jitter=jitter, seed=seed)
    nT = tets.shape[0]
    fib = np.tile(np.array([1.0, 0.0, 0.0]), (nT, 1))
    cf = np.full(nT, speed)
    ct = np.full(nT, speed)
    return dict(xyz=xyz, tets=tets, fib=fib, cf=cf, ct=ct,
                seed_v=np.array([0], dtype=np.int32), seed_t=np.array([0.0]),
                name=f"cube{n}")


def fibre_rotation(z, z0, z1, a0_deg, a1_deg):
    th = np.deg2rad(a0_deg + (a1_deg - a0_deg) * (z - z0) / max(z1 - z0, 1e-30))
    return np.stack([np.cos(th), np.sin(th), np.zeros_like(th)], axis=1)


def slab_case(cells=(266, 93, 40), size=(20.0, 7.0, 3.0), jitter=0.2, seed=2, cf=0.6, ct=0.24,
              scar_radius=2.0, scar_factor=0.1, n_stim=5, t0_max=10.0, angle=60.0):
    """Anisotropic slab (default 266x93x40 cells -> 1,029,018 vertices, 5,937,120 tets)."""
    nx, ny, nz = cells
    lx, ly, lz = size
    xyz, tets = kuhn_box(nx, ny, nz, lx, ly, lz, jitter=jitter, seed=seed)
    cen = tet_centroids(xyz, tets)
    fib = fibre_rotation(cen[:, 2], 0.0, lz, -angle, angle)
    nT = tets.shape[0]
    cfv = np.full(nT, cf)
    ctv = np.full(nT, ct)
    c = np.array([lx / 2, ly / 2, lz / 2])
    scar = np.sum((cen - c) ** 2, axis=1) < scar_radius ** 2
    cfv[scar] *= scar_factor
    ctv[scar] *= scar_factor
    rng = np.random.default_rng(seed + 1000)
    surf = surface_vertices(xyz)
    sv = rng.choice(surf, size=n_stim, replace=False).astype(np.int32)
    st = rng.uniform(0.0, t0_max, size=n_stim)
    return dict(xyz=xyz, tets=tets, fib=fib, cf=cfv, ct=ctv, seed_v=sv, seed_t=st,
                name=f"slab{nx}x{ny}x{nz}", scar=scar)


def batch_cases(n_meshes=32, n_solves=256, vmin=10_000, vmax=500_000, seed=3, jitter=0.2):
    """Uneven Kuhn boxes (vertex counts log-uniform in [vmin, vmax]) and
    per-solve conduction/stimulus draws.  Returns (meshes, solves) where each
    solve is a dict with the mesh index and its conduction and stimuli."""
    rng = np.random.default_rng(seed)
    meshes = []
    for m in range(n_meshes):
        target = math.exp(rng.uniform(math.log(vmin), math.log(vmax)))
        ax = np.array([1.0, rng.uniform(0.5, 1.0), rng.uniform(0.25, 0.6)])
        s = (target / np.prod(ax)) ** (1 / 3)
        nx, ny, nz = [max(2, int(round(s * a)) - 1) for a in ax]
        size = (nx * 0.1, ny * 0.1, nz * 0.1)
        xyz, tets = kuhn_box(nx, ny, nz, *size, jitter=jitter, seed=seed * 100 + m)
        meshes.append(dict(xyz=xyz, tets=tets, cells=(nx, ny, nz), size=size))
    solves = []
    for i in range(n_solves):
        m = i % n_meshes
        mesh = meshes[m]
        cen = tet_centroids(mesh["xyz"], mesh["tets"])
        cf = rng.uniform(0.4, 0.8)
        ct = cf * rng.uniform(0.3, 0.5)
        ang = rng.uniform(40.0, 70.0)
        lz = mesh["size"][2]
        fib = fibre_rotation(cen[:, 2], 0.0, lz, -ang, ang)
        nT = mesh["tets"].shape[0]
        ns = int(rng.integers(1, 9))
        surf = surface_vertices(mesh["xyz"])
        sv = rng.choice(surf, size=ns, replace=False).astype(np.int32)
        st = rng.uniform(0.0, 10.0, size=ns)
        solves.append(dict(mesh=m, fib=fib, cf=np.full(nT, cf), ct=np.full(nT, ct), seed_v=sv, seed_t=st))
    return meshes, solves


def _kuhn_grid_tets(n0, n1, n2, periodic1):
    """Kuhn tets of an n0 x n1 x n2 grid of cells over (n0+1) x m1 x (n2+1)
    vertices, vertex (i, j, k) -> i + (n0+1) * (j + m1 * k); with periodic1
    the second index wraps (m1 = n1), else m1 = n1 + 1."""
    m1 = n1 if periodic1 else n1 + 1

    def vid(i, j, k):
        return i + (n0 + 1) * ((j % m1) + m1 * k)

    ci, cj, ck = np.meshgrid(np.arange(n0), np.arange(n1), np.arange(n2), indexing="ij")
    ci, cj, ck = ci.ravel(order="F"), cj.ravel(order="F"), ck.ravel(order="F")
    tets = []
    for path in _KUHN_PATHS:
        corner = [np.zeros(3, dtype=np.int64)]
        c = np.zeros(3, dtype=np.int64)
        for ax in path:
            c = c.copy()
            c[ax] = 1
            corner.append(c)
        tets.append(np.stack([vid(ci + cc[0], cj + cc[1], ck + cc[2]) for cc in corner], axis=1))
    return np.stack(tets, axis=1).reshape(-1, 4).astype(np.int32)


def shell_case(n_wall=20, n_circ=630, n_long=320, inner=(20.0, 50.0), outer=(30.0, 60.0), apex_hole_deg=3.0,
               jitter=0.2, seed=5, cf=0.6, ct=0.24, angle=60.0, n_stim=8, t0_max=15.0):
    """Ventricle-like shell: the wall between two confocal-free prolate
    spheroids (inner semi-axes 20/20/50 mm, outer 30/30/60 mm, so a 10 mm
    wall), base cut at z = c/3 (2/3 of the height from the apex), a small
    hole at the apex instead of a degenerate pole.  Structured transmural x
    circumferential (periodic) x meridional grid cut into Kuhn tets; defaults
    give 21 x 630 x 321 = 4,246,830 vertices and 24,192,000 tets.  Fibres in
    the wall's tangent plane rotate transmurally from -angle (endocardium) to
    +angle (epicardium) against the circumferential direction; n_stim
    endocardial stimuli with t0 ~ U[0, t0_max]."""
    s = np.linspace(0.0, 1.0, n_wall + 1)
    phi = np.arange(n_circ) * (2 * math.pi / n_circ)
    t = np.linspace(0.0, 1.0, n_long + 1)
    S, P, T = np.meshgrid(s, phi, t, indexing="ij")          # (wall, circ, long)
    a = inner[0] + (outer[0] - inner[0]) * S
    c = inner[1] + (outer[1] - inner[1]) * S
    z_cut = outer[1] / 3.0
    th_base = np.arccos(np.clip(z_cut / c, -1.0, 1.0))
    th_apex = math.pi - math.radians(apex_hole_deg)
    if jitter > 0:
        rng = np.random.default_rng(seed)
        inner_pts = (S > 0) & (S < 1) & (T > 0) & (T < 1)
        S = S + np.where(inner_pts, rng.uniform(-jitter, jitter, S.shape) / n_wall, 0.0)
        P = P + rng.uniform(-jitter, jitter, P.shape) * (2 * math.pi / n_circ)
        T = T + np.where(inner_pts, rng.uniform(-jitter, jitter, T.shape) / n_long, 0.0)
        a = inner[0] + (outer[0] - inner[0]) * S
        c = inner[1] + (outer[1] - inner[1]) * S
        th_base = np.arccos(np.clip(z_cut / c, -1.0, 1.0))
    TH = th_base + T * (th_apex - th_base)
    xyz = np.stack([a * np.sin(TH) * np.cos(P), a * np.sin(TH) * np.sin(P), c * np.cos(TH)], axis=-1)
    # vertex order of _kuhn_grid_tets: i (wall) fastest, then circ, then long
    xyz = np.ascontiguousarray(xyz.transpose(2, 1, 0, 3).reshape(-1, 3))
    tets = _kuhn_grid_tets(n_wall, n_circ, n_long, periodic1=True)
    # fibre per tet from the centroid's wall depth and tangent frame
    sv = np.ascontiguousarray(S.transpose(2, 1, 0).reshape(-1))
    pv = np.ascontiguousarray(P.transpose(2, 1, 0).reshape(-1))
    thv = np.ascontiguousarray(TH.transpose(2, 1, 0).reshape(-1))
    s_t = sv[tets].mean(axis=1)
    # circular mean of the angles of the tet's vertices (the seam wraps)
    p_t = np.arctan2(np.sin(pv[tets]).mean(axis=1), np.cos(pv[tets]).mean(axis=1))
    th_t = thv[tets].mean(axis=1)
    e_circ = np.stack([-np.sin(p_t), np.cos(p_t), np.zeros_like(p_t)], axis=1)
    e_long = np.stack([np.cos(th_t) * np.cos(p_t), np.cos(th_t) * np.sin(p_t), -np.sin(th_t)], axis=1)
    alpha = np.deg2rad(-angle + 2 * angle * s_t)
    fib = np.cos(alpha)[:, None] * e_circ + np.sin(alpha)[:, None] * e_long
    fib /= np.linalg.norm(fib, axis=1)[:, None]
    nT = tets.shape[0]
    rng = np.random.default_rng(seed + 1000)
    endo = np.nonzero(np.abs(sv) < 1e-12)[0]
    seeds = rng.choice(endo, size=n_stim, replace=False).astype(np.int32)
    t0 = rng.uniform(0.0, t0_max, size=n_stim)
    return dict(xyz=xyz, tets=tets, fib=fib, cf=np.full(nT, cf), ct=np.full(nT, ct), seed_v=seeds, seed_t=t0,
                name=f"shell{n_wall}x{n_circ}x{n_long}")


def block_tags(xyz, tets, parts):
    """Geometric partition (this library's own, standing in for the
    reference's METIS-style .tags input): the bounding box is cut into
    parts[0] x parts[1] x parts[2] blocks and every tet takes the block of
    its centroid.  Returns int32 tags numbered x-fastest."""
    cen = tet_centroids(xyz, tets)
    lo, hi = xyz.min(axis=0), xyz.max(axis=0)
    idx = []
    for a in range(3):
        k = np.floor((cen[:, a] - lo[a]) / max(hi[a] - lo[a], 1e-300) * parts[a]).astype(np.int64)
        idx.append(np.clip(k, 0, parts[a] - 1))
    return (idx[0] + parts[0] * (idx[1] + parts[1] * idx[2])).astype(np.int32)
