"""Oracle for the seeded initial fields (test infrastructure only).

float64 numpy restatement of the reference's initialize_fields_cuda
(main_cuda.cu:15157-15430): seed radius and axes
(compute_seed_axes_from_radius :2430-2457), centres (one at the box centre,
several by srand(seed) / rand() inside a margin,
generate_seed_centers_uniform :2335-2383) with the centre shift, the tilt
frame (build_seed_rotation_from_normal :15627-15675), the tanh seed
profile (init_phi_kernel :2244-2312), the hashed phi noise
(apply_phi_noise_kernel :2386-2406) and xB from the diffuse-interface lever
rule (:15316-15356, init_xB_Y_from_phi_kernel :2314-2333).  rand() is the C
library's, called through ctypes, as the reference calls it.
"""
from __future__ import annotations

import ctypes
import ctypes.util
import math

import numpy as np

_LIBC = ctypes.CDLL(ctypes.util.find_library("c"))
_LIBC.rand.restype = ctypes.c_int
_LIBC.srand.argtypes = [ctypes.c_uint]
RAND_MAX = 2147483647   # glibc


def h_of(p):
    return p ** 3 * (6 * p * p - 15 * p + 10)


def seed_axes(p, R, is3d):
    if p.init_shape_mode <= 0:
        return R, R, R
    ax = p.init_axis_ratio_rx if p.init_axis_ratio_rx > 0 else 1.0
    ay = p.init_axis_ratio_ry if p.init_axis_ratio_ry > 0 else 1.0
    az = p.init_axis_ratio_rz if p.init_axis_ratio_rz > 0 else 1.0
    if is3d:
        sc = (ax * ay * az) ** (1.0 / 3.0)
        return R * ax / sc, R * ay / sc, R * az / sc
    sc = math.sqrt(ax * az)
    return R * ax / sc, R, R * az / sc


def tilt_frame(theta_deg, phi_deg):
    t, f = math.radians(theta_deg), math.radians(phi_deg)
    n = np.array([math.sin(t) * math.cos(f), math.sin(t) * math.sin(f), math.cos(t)])
    if np.linalg.norm(n) < 1e-8:
        return np.eye(3)
    n /= np.linalg.norm(n)
    r = np.array([0.0, 1.0, 0.0]) if abs(n[2]) > 0.9 else np.array([0.0, 0.0, 1.0])
    e1 = np.cross(r, n)
    if np.linalg.norm(e1) < 1e-12:
        return np.eye(3)
    e1 /= np.linalg.norm(e1)
    e2 = np.cross(n, e1)
    return np.stack([e1, e2, n])


def centres(p):
    n = p.ic_phi_num_seeds if p.ic_phi_num_seeds > 0 else 1
    L = np.array([p.Nx * p.dx, p.Ny * p.dy, p.Nz * p.dz])
    if n == 1:
        c = [0.5 * L]
    else:
        w = p.ic_phi_iface_w * p.dx if p.ic_phi_iface_w > 0 else p.dx
        R = p.ic_phi_seed_radius if p.ic_phi_seed_radius > 0 else 10.0 * p.dx
        m = np.minimum(R + 2.0 * w, 0.1 * L)
        _LIBC.srand(ctypes.c_uint(p.seed & 0xFFFFFFFF))
        c = []
        for _ in range(n):
            ux = _LIBC.rand() / RAND_MAX
            uy = _LIBC.rand() / RAND_MAX if p.Ny > 2 else 0.0
            uz = _LIBC.rand() / RAND_MAX
            y = m[1] + uy * (L[1] - 2 * m[1]) if p.Ny > 2 else 0.5 * L[1]
            c.append(np.array([m[0] + ux * (L[0] - 2 * m[0]), y, m[2] + uz * (L[2] - 2 * m[2])]))
    sh = np.array([p.init_center_shift_x, p.init_center_shift_y, p.init_center_shift_z])
    if np.any(sh != 0):
        out = []
        for v in c:
            v = v + sh
            v = np.where(v < 0, v + L, v)
            v = np.where(v >= L, v - L, v)
            out.append(v)
        c = out
    return np.array(c)


def _noise_u(N, seed):
    idx = np.arange(1, N + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        x = np.uint64(seed) ^ (idx * np.uint64(2862933555777941757))
        x ^= x >> np.uint64(33)
        x *= np.uint64(0xff51afd7ed558ccd)
        x ^= x >> np.uint64(33)
        x *= np.uint64(0xc4ceb9fe1a85ec53)
        x ^= x >> np.uint64(33)
    return (x & np.uint64(0xFFFFFFFF)).astype(np.float64) / float(0xFFFFFFFF)


def seed_fields(p):
    """phi, xB float64 [Nx][Ny][Nz] for the parameter struct p."""
    Nx, Ny, Nz = p.Nx, p.Ny, p.Nz
    is3d = Ny > 2
    n = p.ic_phi_num_seeds if p.ic_phi_num_seeds > 0 else 1
    L = np.array([Nx * p.dx, Ny * p.dy, Nz * p.dz])
    if p.ic_phi_seed_radius > 0:
        R = p.ic_phi_seed_radius
    else:
        vf = min(0.999, max(1e-6, p.ic_vf_init_phi))
        R = max(1.0, (vf * L.prod() / (n * 4.0 * math.pi / 3.0)) ** (1 / 3) if is3d
                else math.sqrt(vf * L[0] * L[2] / (n * math.pi)))
    Rx, Ry, Rz = seed_axes(p, R, is3d)
    min_axis = min(Rx, Ry, Rz) if is3d else min(Rx, Rz)
    w = p.ic_phi_iface_w * p.dx if p.ic_phi_iface_w > 0 else p.dx
    rot = p.init_use_rotation and (p.init_tilt_theta_deg != 0 or p.init_tilt_phi_deg != 0)
    Rm = tilt_frame(p.init_tilt_theta_deg, p.init_tilt_phi_deg) if rot else None
    x = np.arange(Nx)[:, None, None] * p.dx
    y = np.arange(Ny)[None, :, None] * p.dy
    z = np.arange(Nz)[None, None, :] * p.dz

    def pd(a, c, Lk):
        d = a - c
        d = np.where(d > 0.5 * Lk, d - Lk, d)
        return np.where(d < -0.5 * Lk, d + Lk, d)

    phi = np.zeros((Nx, Ny, Nz))
    for c in centres(p):
        rx, rz = pd(x, c[0], L[0]), pd(z, c[2], L[2])
        ry = pd(y, c[1], L[1]) if is3d else np.zeros_like(y)
        rx, ry, rz = np.broadcast_arrays(rx, ry, rz)
        qx, qy, qz = rx, ry, rz
        if rot:
            qx = Rm[0, 0] * rx + Rm[0, 1] * ry + Rm[0, 2] * rz
            qy = Rm[1, 0] * rx + Rm[1, 1] * ry + Rm[1, 2] * rz
            qz = Rm[2, 0] * rx + Rm[2, 1] * ry + Rm[2, 2] * rz
        r2 = qx * qx / (Rx * Rx) + qz * qz / (Rz * Rz)
        if is3d:
            r2 = r2 + qy * qy / (Ry * Ry)
        phi = np.maximum(phi, 0.5 * (1.0 + np.tanh((1.0 - np.sqrt(r2)) * (min_axis / w))))
    phi = np.clip(phi, 0.0, 1.0)
    if p.init_phi_noise_amp > 0:
        seed = p.init_phi_noise_seed if p.init_phi_noise_seed != 0 else p.seed
        u = _noise_u(phi.size, seed).reshape(phi.shape)
        phi = np.clip(phi + (2.0 * u - 1.0) * p.init_phi_noise_amp, 0.0, 1.0)
    h = h_of(phi)
    mh, mh2 = h.mean(), (h * h).mean()
    xeq, vB = p.xB_eq_matrix, p.v_B
    if p.ic_23d_xB_out > 0:
        xout = p.ic_23d_xB_out
    else:
        vft = min(0.999, max(1e-6, p.ic_vf_target_phi))
        if p.ic_phi_seed_radius > 0:
            sx, sy, sz = seed_axes(p, p.ic_phi_seed_radius, is3d)
            vft = (n * 4.0 * math.pi / 3.0 * sx * sy * sz / L.prod()) if is3d else (n * math.pi * sx * sz / (L[0] * L[2]))
            vft = min(0.999, max(1e-6, vft))
        target = vB * vft + (1.0 - vft) * xeq
        A, B, C = 1.0 - 2.0 * mh + mh2, mh - mh2, vB * mh
        xout = ((vft - mh) * vB + (1 - vft) * xeq) / max(1 - mh, 1e-12) if abs(A) < 1e-12 else (target - B * xeq - C) / A
    xout = min(max(xout, p.xB_eps), 1.0 - p.xB_eps)
    hb = h_of(np.clip(phi, 0.0, 1.0))
    xB = np.clip((1.0 - hb) * xout + hb * xeq, p.xB_eps, 1.0 - p.xB_eps)
    return phi, xB
