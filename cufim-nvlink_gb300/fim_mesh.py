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
