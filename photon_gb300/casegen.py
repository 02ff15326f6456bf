"""Seeded synthetic fire scenarios on Photon's staggered grid.

Photon builds its grid from a scene through its discretizer
(src/sim/discretize.cpp:10-494). The workloads here are synthetic instead: a
seeded generator writes the same arrays the discretizer would leave behind --
the solid-cell mask, face open fractions (`fx/fy/fz`), pressure-matrix
coefficients (`ax/ay/az`) and leak-face flags (`lx/ly/lz`) -- following the
face rule of Solver::updateFace (src/sim/solver.cpp:66-101): a face is closed
when either cell beside it is solid, the ground (k = 0 z-faces) is closed, and
every other face is open. Walls here are solid cells, so no face carries a
barrier and no face leaks.

Workloads (grid sizes in cells; dx in m):

* ``single_room``   36x24x24 at 0.1 m: a closed 3.6 x 2.4 x 2.4 m box with one
  0.8 x 2.0 m doorway in the x = 0 wall open to the atmosphere and a 100 kW
  burner on the floor centre.
* ``house(nx, ny, nz, dx, seed)``: a house of 4-8 rooms (1-cell solid
  partitions, 0.9 x 2.0 m door gaps, 2-6 windows in the exterior wall, a
  ceiling slab at 2.4 m) inside outdoor air whose domain sides and top are
  open; one burner of 10-500 kW (log-uniform) in a random room.
* ``batch_scenarios`` -- 64 houses of 20k-400k cells with log-uniform sizes,
  aspect ratios 1-3 and dx of 0.1 or 0.2 m.
* ``serving_requests`` -- a Poisson stream of houses of 20k-1.32M cells with
  simulated durations of 30-300 s.

All index orders follow the reference (src/sim/solver.h:216-220): cell
i + nx (j + ny k); x-face i + (nx+1)(j + ny k); y-face i + nx (j + (ny+1) k);
z-face i + nx (j + ny k).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

T0 = 293.15


@dataclass
class Burner:
    """A prescribed gas burner (src/sim/solver.h:115-127)."""
    x0: float
    y0: float
    x1: float
    y1: float
    z: float
    peakW: float
    rampS: float = 0.0
    start: float = 0.0
    duration: float = 1e9


@dataclass
class Profile:
    """Time-step and pressure-solve settings (src/sim/solver.h:82-104).

    ``tol`` is the reference's stopping test: the largest divergence error in
    1/s. ``rel_tol`` adds a relative test on max|r| / max|b| (0 = off)."""
    cfl: float = 0.5
    dtMax: float = 0.02
    maxIters: int = 400
    tol: float = 0.002
    rel_tol: float = 0.0

    @staticmethod
    def reference():
        return Profile(0.5, 0.02, 400, 0.002, 0.0)

    @staticmethod
    def realtime():
        return Profile(0.8, 0.05, 80, 0.02, 0.0)


@dataclass
class Case:
    name: str
    nx: int
    ny: int
    nz: int
    dx: float
    ox: float
    oy: float
    oz: float
    blocked: np.ndarray          # uint8 [N]
    fx: np.ndarray               # float64 [(nx+1) ny nz]
    fy: np.ndarray
    fz: np.ndarray
    ax: np.ndarray
    ay: np.ndarray
    az: np.ndarray
    lx: np.ndarray               # uint8, leak faces
    ly: np.ndarray
    lz: np.ndarray
    burners: list = field(default_factory=list)
    profile: Profile = field(default_factory=Profile.reference)
    radiationOn: bool = True
    adiabatic: bool = True
    wind: tuple = (0.0, 0.0, 0.25)
    duration: float = 60.0
    seed: int = 0

    @property
    def N(self) -> int:
        return self.nx * self.ny * self.nz

    @property
    def gas_cells(self) -> int:
        return int(self.N - int(self.blocked.sum()))


def faces_from_blocked(blocked3: np.ndarray):
    """Face open fractions for a solid mask [nz, ny, nx] with open domain sides and
    top and a closed ground (the no-barrier case of Solver::updateFace)."""
    b = blocked3.astype(bool)
    nz, ny, nx = b.shape
    fx = np.ones((nz, ny, nx + 1))
    fy = np.ones((nz, ny + 1, nx))
    fz = np.ones((nz + 1, ny, nx))
    fx[:, :, 1:nx][b[:, :, :-1] | b[:, :, 1:]] = 0
    fx[:, :, 0][b[:, :, 0]] = 0
    fx[:, :, nx][b[:, :, -1]] = 0
    fy[:, 1:ny, :][b[:, :-1, :] | b[:, 1:, :]] = 0
    fy[:, 0, :][b[:, 0, :]] = 0
    fy[:, ny, :][b[:, -1, :]] = 0
    fz[1:nz][b[:-1] | b[1:]] = 0
    fz[nz][b[-1]] = 0
    fz[0] = 0
    return fx, fy, fz


def _finish(name, blocked3, fx, fy, fz, dx, origin, burners, profile, duration, seed, radiationOn=True):
    nz, ny, nx = blocked3.shape
    N = nx * ny * nz
    lx = np.zeros(fx.size, np.uint8)
    ly = np.zeros(fy.size, np.uint8)
    lz = np.zeros(fz.size, np.uint8)
    fx = np.ascontiguousarray(fx.reshape(-1), dtype=np.float64)
    fy = np.ascontiguousarray(fy.reshape(-1), dtype=np.float64)
    fz = np.ascontiguousarray(fz.reshape(-1), dtype=np.float64)
    return Case(name=name, nx=nx, ny=ny, nz=nz, dx=dx, ox=origin[0], oy=origin[1], oz=origin[2],
                blocked=np.ascontiguousarray(blocked3.reshape(-1), dtype=np.uint8),
                fx=fx, fy=fy, fz=fz, ax=fx.copy(), ay=fy.copy(), az=fz.copy(), lx=lx, ly=ly, lz=lz,
                burners=burners, profile=profile, duration=duration, seed=seed, radiationOn=radiationOn)


def from_blocked(name: str, blocked3: np.ndarray, dx: float, origin=(0.0, 0.0, 0.0)) -> Case:
    """A case of the given solid mask [nz, ny, nx] with no barriers and no
    burners: faces open except next to solid cells and at the ground."""
    fx, fy, fz = faces_from_blocked(blocked3)
    return _finish(name, np.asarray(blocked3, np.uint8), fx, fy, fz, dx, origin, [], Profile.reference(), 60.0, 0)


def single_room(peakW: float = 100e3, profile: Profile | None = None) -> Case:
    """36x24x24 cells at 0.1 m: closed box, 0.8 x 2.0 m doorway in the x = 0 wall."""
    nx, ny, nz, dx = 36, 24, 24, 0.1
    blocked = np.zeros((nz, ny, nx), np.uint8)
    fx, fy, fz = faces_from_blocked(blocked)
    fx[:, :, 0] = 0
    fx[:, :, nx] = 0
    fy[:, 0, :] = 0
    fy[:, ny, :] = 0
    fz[nz] = 0
    fx[0:20, 8:16, 0] = 1.0          # doorway: j in [8, 16), k in [0, 20)
    # 3x3 floor cells nearest the centre (i 16-18, j 11-13); edges on cell faces
    burners = [Burner(1.6, 1.1, 1.9, 1.4, 0.0, peakW)]
    return _finish("single_room_36x24x24", blocked, fx, fy, fz, dx, (0.0, 0.0, 0.0), burners,
                   profile or Profile.reference(), 60.0, 0)


def _split_rooms(rng, x0, y0, x1, y1, nrooms, min_size):
    """Recursive guillotine split of a rectangle (cell units, exclusive ends) into
    nrooms rectangles; returns rooms and the partition walls (axis, pos, lo, hi)."""
    rooms = [(x0, y0, x1, y1)]
    walls = []
    tries = 0
    while len(rooms) < nrooms and tries < 200:
        tries += 1
        idx = int(np.argmax([(r[2] - r[0]) * (r[3] - r[1]) for r in rooms]))
        rx0, ry0, rx1, ry1 = rooms[idx]
        w, h = rx1 - rx0, ry1 - ry0
        axis = 0 if w >= h else 1
        span = w if axis == 0 else h
        if span < 2 * min_size + 1:
            break
        cut = int(rng.integers(min_size, span - min_size))
        if axis == 0:
            pos = rx0 + cut
            a, b = (rx0, ry0, pos, ry1), (pos + 1, ry0, rx1, ry1)
            walls.append((0, pos, ry0, ry1))
        else:
            pos = ry0 + cut
            a, b = (rx0, ry0, rx1, pos), (rx0, pos + 1, rx1, ry1)
            walls.append((1, pos, rx0, rx1))
        rooms[idx:idx + 1] = [a, b]
    return rooms, walls


def house(nx: int, ny: int, nz: int, dx: float, seed: int, profile: Profile | None = None,
          duration: float = 300.0, name: str | None = None) -> Case:
    """A seeded house in outdoor air. Sizes of walls, doors and windows are in
    metres, so one seed gives the same house at 0.2 m and 0.1 m cells when the
    domain has the same physical size."""
    rng = np.random.default_rng(seed)
    blocked = np.zeros((nz, ny, nx), np.uint8)
    m = lambda metres: max(1, int(round(metres / dx)))
    # house footprint inside a margin of outdoor air
    mxy = max(2, min(m(1.6), (min(nx, ny) - 8) // 4))
    hx0, hy0, hx1, hy1 = mxy, mxy, nx - mxy, ny - mxy          # exterior wall cells included
    kslab = min(m(2.4), nz - 3)
    wall_top = kslab                                            # walls span k in [0, kslab)
    # exterior walls and ceiling slab
    blocked[0:wall_top, hy0:hy1, hx0] = 1
    blocked[0:wall_top, hy0:hy1, hx1 - 1] = 1
    blocked[0:wall_top, hy0, hx0:hx1] = 1
    blocked[0:wall_top, hy1 - 1, hx0:hx1] = 1
    blocked[kslab, hy0:hy1, hx0:hx1] = 1
    # rooms inside
    nrooms = int(rng.integers(4, 9))
    min_size = max(2, m(1.8))
    rooms, walls = _split_rooms(rng, hx0 + 1, hy0 + 1, hx1 - 1, hy1 - 1, nrooms, min_size)
    for axis, pos, lo, hi in walls:
        if axis == 0:
            blocked[0:wall_top, lo:hi, pos] = 1
        else:
            blocked[0:wall_top, pos, lo:hi] = 1
    # door gaps: one per partition, 0.9 m wide, 2.0 m tall, at a random spot
    door_w, door_h = m(0.9), min(m(2.0), wall_top)
    for axis, pos, lo, hi in walls:
        span = hi - lo
        w = min(door_w, max(1, span - 2))
        s = lo + int(rng.integers(1, max(2, span - w)))
        if axis == 0:
            blocked[0:door_h, s:s + w, pos] = 0
        else:
            blocked[0:door_h, pos, s:s + w] = 0
    # windows: 2-6 gaps in the exterior wall, 1.0-1.5 m wide, sill 0.9 m, 1.2 m tall
    nwin = int(rng.integers(2, 7))
    k0 = min(m(0.9), wall_top - 2)
    k1 = min(k0 + m(1.2), wall_top)
    for _ in range(nwin):
        side = int(rng.integers(0, 4))
        w = m(float(rng.uniform(1.0, 1.5)))
        if side < 2:
            span = hy1 - hy0
            w = min(w, span - 4)
            s = hy0 + int(rng.integers(2, max(3, span - w - 1)))
            blocked[k0:k1, s:s + w, hx0 if side == 0 else hx1 - 1] = 0
        else:
            span = hx1 - hx0
            w = min(w, span - 4)
            s = hx0 + int(rng.integers(2, max(3, span - w - 1)))
            blocked[k0:k1, hy0 if side == 2 else hy1 - 1, s:s + w] = 0
    fx, fy, fz = faces_from_blocked(blocked)
    # burner: 0.4 m square on the floor of a random room, 10-500 kW log-uniform;
    # edges on cell faces so no cell centre ties with an edge
    room = rooms[int(rng.integers(0, len(rooms)))]
    rx0, ry0, rx1, ry1 = room
    bw = max(1, min(m(0.4), rx1 - rx0, ry1 - ry0))
    bi = rx0 + (rx1 - rx0 - bw) // 2
    bj = ry0 + (ry1 - ry0 - bw) // 2
    peak = float(math.exp(rng.uniform(math.log(10e3), math.log(500e3))))
    burners = [Burner(bi * dx, bj * dx, (bi + bw) * dx, (bj + bw) * dx, 0.0, peak)]
    return _finish(name or "house_%dx%dx%d_s%d" % (nx, ny, nz, seed), blocked, fx, fy, fz, dx, (0.0, 0.0, 0.0),
                   burners, profile or Profile.reference(), duration, seed)


def house_small(seed: int = 1) -> Case:
    """72x52x44 cells at 0.2 m (164,736 cells), 300 s simulated."""
    return house(72, 52, 44, 0.2, seed, duration=300.0)


def house_fine(seed: int = 1) -> Case:
    """144x104x88 cells at 0.1 m (1,317,888 cells): the same house at 10 cm."""
    return house(144, 104, 88, 0.1, seed, duration=60.0)


def _dims_for(rng, ncells: float):
    """Grid dims with a log-uniform aspect ratio of 1-3 between the longest and
    the shortest side, for about ncells cells."""
    ar = float(math.exp(rng.uniform(0.0, math.log(3.0))))
    a2 = float(math.exp(rng.uniform(0.0, math.log(ar))))
    # sides proportional to (ar, a2, 1); vertical side is the smallest
    base = (ncells / (ar * a2)) ** (1.0 / 3.0)
    nx, ny, nz = int(round(base * ar)), int(round(base * a2)), int(round(base))
    return max(nx, 16), max(ny, 16), max(nz, 16)


def batch_scenarios(n: int = 64, seed: int = 2024, lo: float = 20e3, hi: float = 400e3) -> list:
    """n seeded houses of lo-hi cells (log-uniform), dx of 0.1 or 0.2 m."""
    rng = np.random.default_rng(seed)
    out = []
    for s in range(n):
        N = float(math.exp(rng.uniform(math.log(lo), math.log(hi))))
        nx, ny, nz = _dims_for(rng, N)
        dx = 0.1 if rng.integers(0, 2) == 0 else 0.2
        out.append(house(nx, ny, nz, dx, seed * 1000 + s, name="batch%02d_%dx%dx%d" % (s, nx, ny, nz)))
    return out


def serving_requests(n: int, rate_hz: float, seed: int = 7, lo: float = 20e3, hi: float = 1.32e6):
    """A Poisson stream: list of (arrival_s, Case) with 30-300 s durations."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for r in range(n):
        t += float(rng.exponential(1.0 / rate_hz))
        N = float(math.exp(rng.uniform(math.log(lo), math.log(hi))))
        nx, ny, nz = _dims_for(rng, N)
        dx = 0.1 if rng.integers(0, 2) == 0 else 0.2
        c = house(nx, ny, nz, dx, seed * 100000 + r, name="req%03d_%dx%dx%d" % (r, nx, ny, nz))
        c.duration = float(rng.uniform(30.0, 300.0))
        out.append((t, c))
    return out


def tiny_room(nx=12, ny=10, nz=9, dx=0.2, peakW=60e3, doorway=True, seed=0) -> Case:
    """A small closed room for fast parity cases; one doorway in the x = 0 wall."""
    blocked = np.zeros((nz, ny, nx), np.uint8)
    fx, fy, fz = faces_from_blocked(blocked)
    fx[:, :, 0] = 0
    fx[:, :, nx] = 0
    fy[:, 0, :] = 0
    fy[:, ny, :] = 0
    fz[nz] = 0
    if doorway:
        fx[0:max(1, nz * 3 // 4), ny // 3:ny // 3 + max(2, ny // 3), 0] = 1.0
    ci, cj = nx // 2, ny // 2
    burners = [Burner((ci - 1) * dx, (cj - 1) * dx, (ci + 1) * dx, (cj + 1) * dx, 0.0, peakW)] if peakW > 0 else []
    return _finish("tiny_room_%dx%dx%d" % (nx, ny, nz), blocked, fx, fy, fz, dx, (0.0, 0.0, 0.0), burners,
                   Profile.reference(), 10.0, seed)


def rad_workload(case: Case, seed: int = 3, wall_frac: float = 0.02, porous_frac: float = 0.01) -> dict:
    """Seeded inputs of a radiation trace on `case`, shaped like what
    Solver::buildRadElements and the solid phase hand the trace
    (src/sim/radiation.cpp:104-164): a hot plume with flame cells over the
    first burner (or the domain centre); an element on every gas-facing side
    of every solid cell; a random share of the interior gas-gas faces as
    intact walls, with an element on each side; a random share of the gas
    cells as porous fuel (full-sphere elements that skip their own cell).
    Returns the gas fields (T Ys Yw Yc Pb hrr), elements (n x 11), walls
    (m x 4) and solidT (N)."""
    rng = np.random.default_rng(seed)
    nx, ny, nz, dx = case.nx, case.ny, case.nz, case.dx
    ox, oy, oz = case.ox, case.oy, case.oz
    b3 = case.blocked.reshape(nz, ny, nx).astype(bool)
    k3, j3, i3 = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    xc, yc, zc = ox + (i3 + 0.5) * dx, oy + (j3 + 0.5) * dx, oz + (k3 + 0.5) * dx
    if case.burners:
        b = case.burners[0]
        px, py = 0.5 * (b.x0 + b.x1), 0.5 * (b.y0 + b.y1)
    else:
        px, py = ox + 0.5 * nx * dx, oy + 0.5 * ny * dx
    r2 = (xc - px) ** 2 + (yc - py) ** 2
    plume = np.exp(-r2 / 0.5) * np.clip(1.2 - 0.25 * (zc - oz), 0.2, 1.0)
    layer = np.clip((zc - oz - 1.2) / 1.2, 0, 1) * 0.35
    heat = np.maximum(plume, layer)
    T = 293.15 + 900.0 * heat
    hrr = np.where(plume > 0.6, 2.0e6 * plume, 0.0)
    Ys = 0.004 * heat
    Yw = 0.0073 + 0.05 * heat
    Yc = 0.0006 + 0.08 * heat
    Pb = np.full(T.shape, 101325.0)
    for a in (T, hrr, Ys, Yw, Yc):
        a[b3] = 0.0 if a is not T else 293.15
    gas = {"T": T.ravel(), "Ys": Ys.ravel(), "Yw": Yw.ravel(), "Yc": Yc.ravel(), "Pb": Pb.ravel(), "hrr": hrr.ravel()}
    solidT = np.where(b3, 293.15 + 500.0 * heat + 50.0 * rng.random(b3.shape), 293.15).ravel()

    elems = []
    A = dx * dx
    # solid cell faces seen from gas (kind 1)
    for axis in range(3):
        for sgn in (-1, 1):
            sh = [0, 0, 0]
            sh[2 - axis] = sgn
            nb = np.zeros_like(b3)
            src = [slice(None)] * 3
            dst = [slice(None)] * 3
            if sgn > 0:
                src[2 - axis], dst[2 - axis] = slice(1, None), slice(0, -1)
            else:
                src[2 - axis], dst[2 - axis] = slice(0, -1), slice(1, None)
            nbb = np.ones_like(b3)            # outside the domain counts as no gas neighbour
            nbb[tuple(dst)] = b3[tuple(src)]
            exposed = b3 & ~nbb
            kk, jj, ii = np.nonzero(exposed)
            n = np.zeros((len(kk), 3))
            n[:, axis] = sgn
            o = np.stack([ox + (ii + 0.5) * dx, oy + (jj + 0.5) * dx, oz + (kk + 0.5) * dx], 1) + n * (0.5 * dx + 1e-3)
            t = solidT.reshape(nz, ny, nx)[kk, jj, ii]
            e = np.zeros((len(kk), 11))
            e[:, 0:3], e[:, 3:6], e[:, 6], e[:, 7], e[:, 8] = o, n, A, 0.9, t
            elems.append(e)
    # walls on interior gas-gas faces (kind 0 on each side)
    walls = []
    for axis, nf in ((0, (nz, ny, nx + 1)), (1, (nz, ny + 1, nx)), (2, (nz + 1, ny, nx))):
        lo = [slice(None)] * 3
        hi = [slice(None)] * 3
        lo[2 - axis], hi[2 - axis] = slice(0, -1), slice(1, None)
        both = ~b3[tuple(lo)] & ~b3[tuple(hi)]
        kk, jj, ii = np.nonzero(both & (rng.random(both.shape) < wall_frac))
        fi = [ii, jj, kk]
        fi[axis] = fi[axis] + 1                   # the face above the lower cell
        face = fi[0] + nf[2] * (fi[1] + nf[1] * fi[2])
        tl = 293.15 + 600.0 * heat[kk, jj, ii] * rng.random(len(kk))
        tu = 293.15 + 600.0 * heat[kk, jj, ii] * rng.random(len(kk))
        walls.append(np.stack([np.full(len(kk), axis), face, tl, tu], 1))
        for side, t in ((-1, tl), (1, tu)):
            n = np.zeros((len(kk), 3))
            n[:, axis] = side
            fc = np.stack([ox + (ii + 0.5) * dx, oy + (jj + 0.5) * dx, oz + (kk + 0.5) * dx], 1)
            fc[:, axis] += 0.5 * dx                 # the face plane
            e = np.zeros((len(kk), 11))
            e[:, 0:3], e[:, 3:6], e[:, 6], e[:, 7], e[:, 8] = fc + n * 1e-3, n, A, 0.85, t
            elems.append(e)
    # porous fuel in gas cells (kind 2)
    kk, jj, ii = np.nonzero(~b3 & (rng.random(b3.shape) < porous_frac))
    e = np.zeros((len(kk), 11))
    e[:, 0:3] = np.stack([ox + (ii + 0.5) * dx, oy + (jj + 0.5) * dx, oz + (kk + 0.5) * dx], 1)
    e[:, 6] = np.minimum(rng.uniform(0.2, 8.0, len(kk)) * A, 4 * A)
    e[:, 7], e[:, 8], e[:, 9], e[:, 10] = 0.8, T[kk, jj, ii], 1, 1
    elems.append(e)
    return {"gas": gas, "elements": np.concatenate(elems), "walls": np.concatenate(walls), "solidT": solidT}
