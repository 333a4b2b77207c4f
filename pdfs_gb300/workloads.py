"""Seeded synthetic inputs for the FSM distance-field solve.

Every workload is a halo-padded float64 field of shape (nz+2, ny+2, nx+2)
(x fastest, the layout of the reference's ``Phi.distance``,
single_gpu_cuda/src/phi3D.c:66 and mpi_openacc/src/phi3D_fsm.c:112), plus a
uint8 mask of the same shape marking the frozen interface nodes.

Conventions (single_gpu_cuda/src/phi3D.h:37-40): the one-node halo holds +inf
(DEFAULT_BORDER_DISTANCE); nodes away from the interface start at a large
value (1e10 here); interface nodes hold their exact distance to the interface.
Interior node (i, j, k), 1-based, sits at physical position
((i-1)*dx, (j-1)*dy, (k-1)*dz).

The reference ships no data sets; these generators stand in for its inputs
and are reproducible from (name, seed).
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

FAR = 1.0e10
BORDER = math.inf


@dataclasses.dataclass
class Workload:
    name: str
    nx: int
    ny: int
    nz: int
    dx: float
    dy: float
    dz: float
    field: np.ndarray      # float64 (nz+2, ny+2, nx+2), halo = +inf
    frozen: np.ndarray     # uint8, same shape; 1 = interface node

    @property
    def interior(self) -> int:
        return self.nx * self.ny * self.nz

    @property
    def shape(self):
        return (self.nz + 2, self.ny + 2, self.nx + 2)


def empty_field(nx, ny, nz, far=FAR):
    f = np.full((nz + 2, ny + 2, nx + 2), far, dtype=np.float64)
    f[0, :, :] = BORDER
    f[-1, :, :] = BORDER
    f[:, 0, :] = BORDER
    f[:, -1, :] = BORDER
    f[:, :, 0] = BORDER
    f[:, :, -1] = BORDER
    return f


def _stamp_sphere(field, frozen, c, r, thr, dx, dy, dz):
    """Freeze nodes with |‖p-c‖-r| <= thr at that exact distance (min over spheres)."""
    nzp, nyp, nxp = field.shape
    nx, ny, nz = nxp - 2, nyp - 2, nzp - 2
    lo, hi = [], []
    for ax, (cc, h, n) in enumerate(zip(c, (dx, dy, dz), (nx, ny, nz))):
        a = max(1, int(math.floor((cc - r - thr) / h)) + 1)
        b = min(n, int(math.ceil((cc + r + thr) / h)) + 1)
        lo.append(a)
        hi.append(b)
    if any(h < l for l, h in zip(lo, hi)):
        return
    xs = (np.arange(lo[0], hi[0] + 1) - 1) * dx - c[0]
    ys = (np.arange(lo[1], hi[1] + 1) - 1) * dy - c[1]
    zs = (np.arange(lo[2], hi[2] + 1) - 1) * dz - c[2]
    d = np.abs(np.sqrt(zs[:, None, None] ** 2 + ys[None, :, None] ** 2 + xs[None, None, :] ** 2) - r)
    sub = field[lo[2]:hi[2] + 1, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1]
    fsub = frozen[lo[2]:hi[2] + 1, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1]
    near = d <= thr
    np.minimum(sub, np.where(near, d, FAR), out=sub)
    fsub |= near.astype(np.uint8)


def spheres(nx, ny, nz, dx, dy, dz, centres, radii, thr=None, name="spheres"):
    """Union-of-spheres interface: frozen where the distance to the nearest
    sphere surface is <= thr (default: the largest spacing)."""
    thr = max(dx, dy, dz) if thr is None else thr
    field = empty_field(nx, ny, nz)
    frozen = np.zeros(field.shape, dtype=np.uint8)
    for c, r in zip(centres, radii):
        _stamp_sphere(field, frozen, c, float(r), thr, dx, dy, dz)
    return Workload(name, nx, ny, nz, dx, dy, dz, field, frozen)


def random_spheres(nx, ny, nz, dx, dy, dz, count, rmin, rmax, seed, log_radii=True, name=None):
    rng = np.random.default_rng(seed)
    ext = np.array([(nx - 1) * dx, (ny - 1) * dy, (nz - 1) * dz])
    centres = rng.uniform(0.0, 1.0, size=(count, 3)) * ext
    if log_radii:
        radii = np.exp(rng.uniform(math.log(rmin), math.log(rmax), size=count))
    else:
        radii = rng.uniform(rmin, rmax, size=count)
    return spheres(nx, ny, nz, dx, dy, dz, centres, radii,
                   name=name or f"spheres{count}_{nx}x{ny}x{nz}_s{seed}")


def unit_sphere(n=64):
    """A single sphere r=0.25 at the centre of the unit cube, h = 1/(n-1);
    nodes within h of the sphere are frozen at the exact distance."""
    h = 1.0 / (n - 1)
    w = spheres(n, n, n, h, h, h, [(0.5, 0.5, 0.5)], [0.25], thr=h, name=f"sphere_{n}")
    return w


def heightmap(nx, ny, nz, dx, dy, dz, seed, bumps=8, base=10.0, amp=(5.0, 40.0), width=(20.0, 120.0),
              name=None):
    """z = base + sum of seeded Gaussian bumps.  Nodes within one z-cell of the
    surface are frozen at the vertical distance corrected by the local slope,
    |z - h| / sqrt(1 + |grad h|^2)."""
    rng = np.random.default_rng(seed)
    cx = rng.uniform(0.0, (nx - 1) * dx, size=bumps)
    cy = rng.uniform(0.0, (ny - 1) * dy, size=bumps)
    A = rng.uniform(amp[0], amp[1], size=bumps)
    W = rng.uniform(width[0], width[1], size=bumps)
    x = (np.arange(nx) * dx)[None, :]
    y = (np.arange(ny) * dy)[:, None]
    h = np.full((ny, nx), base)
    hx = np.zeros((ny, nx))
    hy = np.zeros((ny, nx))
    for i in range(bumps):
        g = A[i] * np.exp(-((x - cx[i]) ** 2 + (y - cy[i]) ** 2) / (2.0 * W[i] ** 2))
        h += g
        hx += g * (-(x - cx[i]) / W[i] ** 2)
        hy += g * (-(y - cy[i]) / W[i] ** 2)
    corr = 1.0 / np.sqrt(1.0 + hx ** 2 + hy ** 2)
    field = empty_field(nx, ny, nz)
    frozen = np.zeros(field.shape, dtype=np.uint8)
    for k in range(nz):
        dist = np.abs(k * dz - h)
        near = dist <= dz
        plane = field[k + 1, 1:-1, 1:-1]
        plane[near] = (dist * corr)[near]
        frozen[k + 1, 1:-1, 1:-1] = near
    return Workload(name or f"heightmap_{nx}x{ny}x{nz}_s{seed}", nx, ny, nz, dx, dy, dz, field, frozen)


def random_field(nx, ny, nz, seed, frac_known=0.05, scale=5.0):
    """Small random field for sweep-level parity: mostly FAR, some random
    known values; halo +inf.  No frozen nodes."""
    rng = np.random.default_rng(seed)
    f = empty_field(nx, ny, nz)
    inner = f[1:-1, 1:-1, 1:-1]
    known = rng.uniform(size=inner.shape) < frac_known
    inner[known] = rng.uniform(0.0, scale, size=int(known.sum()))
    return f


# ---- the benchmark configurations -------------------------------------------------

def config(name: str, seed: int = 0) -> Workload:
    """C1..C4 at their full sizes, and reduced variants for tests."""
    if name == "C1":
        return unit_sphere(64)
    if name == "C2":
        return heightmap(512, 512, 128, 1.0, 1.0, 0.5, seed=seed + 2, name="C2_heightmap_512x512x128")
    if name == "C3":
        return random_spheres(1024, 1024, 1024, 1.0, 1.0, 0.5, 200, 5.0, 60.0, seed=seed + 3,
                              name="C3_spheres200_1024^3")
    if name == "C4":
        return random_spheres(768, 768, 768, 1.0, 1.0, 1.0, 150, 4.0, 50.0, seed=seed + 4,
                              name="C4_spheres150_768^3")
    raise KeyError(name)


def batch_c5(count=256, seed=5, lo=32, hi=256):
    """C5: `count` independent grids, per-axis sizes log-uniform in [lo, hi],
    dx = 1, 1..20 spheres of radius uniform in [3, 30] each."""
    rng = np.random.default_rng(seed)
    out = []
    for g in range(count):
        n = np.exp(rng.uniform(math.log(lo), math.log(hi), size=3)).astype(int)
        k = int(rng.integers(1, 21))
        s = int(rng.integers(0, 2 ** 31 - 1))
        out.append(random_spheres(int(n[0]), int(n[1]), int(n[2]), 1.0, 1.0, 1.0, k, 3.0, 30.0, seed=s,
                                  log_radii=False, name=f"C5_{g}"))
    return out
