"""Seeded synthetic microstructures of the benchmark / test workloads.

The reference reads raw initial fields (``--init-mode raw_fields``); these
generators produce them.  Precipitates use the reference's seed profile
phi = 1/2 (1 + tanh((1 - r_eff) * min_axis / w)) with r_eff the ellipsoidal
radius in the particle frame and the maximum over particles
(init_phi_kernel, main_cuda.cu:2244-2312); w = ic_phi_iface_w.
"""
from __future__ import annotations

import math

import numpy as np


def _grid(shape):
    return [np.arange(n, dtype=np.float64) for n in shape]


def _periodic(d, L):
    return d - L * np.round(d / L)


def random_rotation(rng: np.random.Generator) -> np.ndarray:
    """Uniform rotation (Haar measure) from a random unit quaternion."""
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def ellipsoid_field(shape, centers, radii, rots, w, cutoff=8.0):
    """max over particles of the tanh seed profile; radii (n,3), rots (n,3,3).

    Each particle is evaluated inside a periodic box of half-width
    max(R) + cutoff*w around its centre (outside, the profile is below
    1e-13 and the field keeps its previous value)."""
    Nx, Ny, Nz = shape
    phi = np.zeros(shape)
    for c, R, M in zip(centers, radii, rots):
        half = max(R) + cutoff * w
        idx = []
        for a, n in enumerate(shape):
            lo = int(math.floor(c[a] - half))
            hi = int(math.ceil(c[a] + half))
            if hi - lo + 1 >= n:
                ii = np.arange(n)
            else:
                ii = np.arange(lo, hi + 1) % n
            idx.append(ii)
        rx = _periodic(idx[0] - c[0], Nx)[:, None, None]
        ry = _periodic(idx[1] - c[1], Ny)[None, :, None]
        rz = _periodic(idx[2] - c[2], Nz)[None, None, :]
        q = [M[a, 0] * rx + M[a, 1] * ry + M[a, 2] * rz for a in range(3)]
        reff = np.sqrt((q[0] / R[0]) ** 2 + (q[1] / R[1]) ** 2 + (q[2] / R[2]) ** 2)
        seed = 0.5 * (1.0 + np.tanh((1.0 - reff) * (min(R) / w)))
        sub = np.ix_(idx[0], idx[1], idx[2])
        phi[sub] = np.maximum(phi[sub], seed)
    return np.clip(phi, 0.0, 1.0)


def composition(phi, rng, c_matrix=0.03, c_precip=0.33, noise=1e-3):
    h = phi ** 3 * (6 * phi ** 2 - 15 * phi + 10)
    base = c_matrix + noise * rng.standard_normal(phi.shape)
    return (1.0 - h) * base + h * c_precip


def single_sphere(n=64, radius=8.0, w=2.5, seed=1234):
    """One centred sphere, c = 0.03 + N(0, 1e-3) outside, 0.33 inside."""
    rng = np.random.default_rng(seed)
    shape = (n, n, n)
    c = np.array([n / 2, n / 2, n / 2])
    phi = ellipsoid_field(shape, [c], [np.full(3, radius)], [np.eye(3)], w)
    return {"phi": phi, "xB": composition(phi, rng)}


def ellipsoid_population(n=246, count=60, median_r=6.0, sigma_ln=0.3, eta_sites=20, eta_r=3.0,
                         w=2.5, seed=2468, max_tries=200000, shape=None):
    """Non-overlapping ellipsoids (log-normal radii, aspect ratios U[0.5,1],
    uniform rotations, rejection placement) plus spherical GP-zone eta seeds.
    ``shape`` overrides the cubic n^3 grid."""
    rng = np.random.default_rng(seed)
    shape = tuple(shape) if shape else (n, n, n)
    L = np.array(shape, dtype=np.float64)
    centers, radii, rots = [], [], []
    tries = 0
    while len(centers) < count and tries < max_tries:
        tries += 1
        a = median_r * math.exp(sigma_ln * rng.standard_normal())
        R = np.array([a, a * rng.uniform(0.5, 1.0), a * rng.uniform(0.5, 1.0)])
        c = rng.uniform(0, 1, size=3) * L
        ok = True
        for c2, R2 in zip(centers, radii):
            d = _periodic(c - c2, L)
            if np.linalg.norm(d) < R.max() + R2.max() + 2 * w:
                ok = False
                break
        if ok:
            centers.append(c)
            radii.append(R)
            rots.append(random_rotation(rng))
    phi = ellipsoid_field(shape, centers, radii, rots, w)
    # eta sites in the matrix, away from precipitates
    ecs = []
    tries = 0
    while len(ecs) < eta_sites and tries < max_tries:
        tries += 1
        c = rng.uniform(0, 1, size=3) * L
        ok = all(np.linalg.norm(_periodic(c - c2, L)) > R2.max() + eta_r + 2 * w
                 for c2, R2 in zip(centers, radii))
        ok = ok and all(np.linalg.norm(_periodic(c - e, L)) > 2 * eta_r + 2 * w for e in ecs)
        if ok:
            ecs.append(c)
    eta = ellipsoid_field(shape, ecs, [np.full(3, eta_r)] * len(ecs), [np.eye(3)] * len(ecs), w)
    return {"phi": phi, "xB": composition(phi, rng), "eta": eta,
            "n_particles": len(centers), "n_eta": len(ecs)}


EIGEN_DIAG = (0.046, -0.022, -0.017)


def rotated_eigenstrain(rot, diag=EIGEN_DIAG):
    """R diag(e) R^T as the 6-vector xx, yy, zz, yz, xz, xy."""
    E = rot @ np.diag(diag) @ rot.T
    return [E[0, 0], E[1, 1], E[2, 2], E[1, 2], E[0, 2], E[0, 1]]


def sweep_cases(count=48, sizes=(64, 80, 96, 112, 128, 144, 160), ratios=(1.0, 0.6, 0.3),
                r_range=(10.0, 40.0), n_rot=8, w=2.5, seed=7):
    """The batched minimize sweep: cubic grids cycled through `sizes`, a
    sphere or oblate spheroid (semi-axes R, R, (c/a) R) of radius R in
    r_range (capped below n/2 - 2w), and the eigenstrain rotated by one of
    n_rot seeded rotations (the spheroid shares the rotation)."""
    rng = np.random.default_rng(seed)
    rots = [random_rotation(rng) for _ in range(n_rot)]
    cases = []
    for i in range(count):
        n = sizes[i % len(sizes)]
        ca = ratios[int(rng.integers(len(ratios)))]
        R = float(rng.uniform(*r_range))
        R = min(R, n / 2 - 2 * w - 1)
        k = int(rng.integers(n_rot))
        cases.append({"n": n, "ca": ca, "radius": R, "rot": rots[k], "rot_index": k,
                      "eps00": rotated_eigenstrain(rots[k]), "seed": int(rng.integers(1 << 30))})
    return cases


def spheroid_fields(case, w=2.5):
    """Centred spheroid seed (tanh profile of init_phi_kernel) and the
    composition of `composition`."""
    n, R, ca = case["n"], case["radius"], case["ca"]
    shape = (n, n, n)
    c = np.array([n / 2, n / 2, n / 2])
    phi = ellipsoid_field(shape, [c], [np.array([R, R, ca * R])], [case["rot"]], w)
    rng = np.random.default_rng(case["seed"])
    return {"phi": phi, "xB": composition(phi, rng)}
