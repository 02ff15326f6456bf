"""Headless smoke and flame rendering: the host side of phx_vol_render.

camera() builds the shader's uniforms (phx_vol_params) for a look-at
perspective camera over a case's grid; fire_lights() picks the fire lights
the way Viewer::uploadVolume does (src/app/viewer.cpp:950-981);
write_ppm() stores an image. The ray march itself runs on the GPU
(Solver.vol_render).
"""
from __future__ import annotations

import math

import numpy as np

from ._lib import PhxVolParams


def _look_at(eye, target, up=(0.0, 0.0, 1.0)):
    eye, target, up = (np.asarray(v, np.float64) for v in (eye, target, up))
    f = target - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s, u, -f
    m[:3, 3] = -m[:3, :3] @ eye
    return m


def _perspective(fov_deg, aspect, near, far):
    f = 1.0 / math.tan(math.radians(fov_deg) / 2)
    m = np.zeros((4, 4))
    m[0, 0], m[1, 1] = f / aspect, f
    m[2, 2], m[2, 3] = (far + near) / (near - far), 2 * far * near / (near - far)
    m[3, 2] = -1.0
    return m


def camera(case, eye, target, width=640, height=360, fov_deg=60.0, near=0.05, far=500.0, smoke=True, fire=True,
           slice_z=None, t_range=(293.15, 1200.0), time=0.0, smoke_scale=1.0, sun_dir=(0.3, 0.2, 0.93),
           background=(0.55, 0.62, 0.70), lights=()) -> PhxVolParams:
    """Uniforms for a perspective camera at `eye` looking at `target` (m); the
    march step is 0.3 dx as the viewer sets it (src/render/renderer.cpp:515)."""
    vp = _perspective(fov_deg, width / height, near, far) @ _look_at(eye, target)
    inv = np.linalg.inv(vp)
    p = PhxVolParams()
    p.width, p.height = int(width), int(height)
    for i, v in enumerate(inv.T.reshape(-1)):      # column-major
        p.inv_vp[i] = float(v)
    for i in range(3):
        p.eye[i] = float(eye[i])
        p.background[i] = float(background[i])
    sd = np.asarray(sun_dir, np.float64)
    sd /= np.linalg.norm(sd)
    for i in range(3):
        p.sun_dir[i] = float(sd[i])
    p.step = 0.3 * case.dx
    p.clip_z = case.oz + case.nz * case.dx
    p.slice = 0 if slice_z is None else 1
    p.slice_z = 0.0 if slice_z is None else float(slice_z)
    p.t_min, p.t_max = float(t_range[0]), float(t_range[1])
    p.smoke, p.fire = int(bool(smoke)), int(bool(fire))
    p.time, p.smoke_scale = float(time), float(smoke_scale)
    p.n_lights = min(8, len(lights))
    for q in range(p.n_lights):
        for k in range(4):
            p.lights[q][k] = float(lights[q][k])
    return p


def fire_lights(case, hrr, time=0.0):
    """Up to 8 fire lights: the strongest burning cells (hrr > 100 kW/m3) at
    least 1.6 m apart, each carrying the heat release of the burning cells
    nearest it; intensity clamp(sqrt(kW) 0.16, 0, 5) with the viewer's flicker
    (src/app/viewer.cpp:950-981). Returns [(x, y, z, intensity)]."""
    nx, ny, dx = case.nx, case.ny, case.dx
    cells = np.nonzero(hrr > 1e5)[0]
    cells = cells[np.argsort(-hrr[cells], kind="stable")]

    def center(c):
        i, j, k = c % nx, (c // nx) % ny, c // (nx * ny)
        return np.array([case.ox + (i + 0.5) * dx, case.oy + (j + 0.5) * dx, case.oz + (k + 0.5) * dx])

    lp = []
    for c in cells:
        if len(lp) >= 8:
            break
        p = center(c)
        if all(np.linalg.norm(p - q) >= 1.6 for q in lp):
            lp.append(p)
    power = np.zeros(len(lp))
    V = dx ** 3
    for c in cells:
        if lp:
            d = [np.linalg.norm(center(c) - q) for q in lp]
            power[int(np.argmin(d))] += hrr[c] * V
    out = []
    for q, p in enumerate(lp):
        kw = power[q] / 1000.0
        flicker = 0.85 + 0.1 * math.sin(time * 13.0 + q * 2.3) + 0.05 * math.sin(time * 29.0 + q)
        out.append((p[0], p[1], p[2], min(max(math.sqrt(kw) * 0.16, 0.0), 5.0) * flicker))
    return out


def write_ppm(path: str, rgb: np.ndarray):
    """An (height, width, 3) image with rows from the bottom, as 8-bit PPM."""
    img = (np.clip(rgb[::-1], 0.0, 1.0) * 255.0 + 0.5).astype(np.uint8)
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (img.shape[1], img.shape[0]))
        f.write(img.tobytes())
