"""Seeded synthetic scan workloads with the shapes of the benchmark configs.

No public dataset is used: each config is a procedurally generated scene that
a simulated sensor scans. Points are float32 in the map frame, laid out as
pcl::PointXYZ (x, y, z, pad) rows of 16 bytes.

  small   seed 1: 40x40x6 m room with 20 random boxes; 64x1024 LiDAR beams
          (elevation -25..+15 deg, uniform azimuth); 10 scans from (0,0,1.5)
          stepping 0.2 m along x; range noise sigma 2 cm; 5% no-returns;
          voxel 0.1 m, max_range 30 m.
  dense   seed 2: 200x200x20 m street (buildings, cars as boxes, poles and
          trees as cylinders); 128x2048 beams; 100 scans stepping 1 m along
          the street; sigma 1 cm; 3% no-returns; voxel 0.05 m, max_range 60 m.
  stress  seed 3: 20 scans of 65,536 rays with uniform random directions and
          log-uniform ranges 0.5-200 m from (5000,-3000,40); 1% of endpoints
          on quantiser boundaries and DDA tie directions; voxel 0.02 m,
          max_range 250 m.
  batched seed 4: 32 independent maps, one scan each per step, 50 steps.
          Points per scan log-uniform over 2,000-307,200 (mean about 60.6k).
          A map is a depth camera (640x480 pixels, 90x60 deg field of view,
          subsampled to its point count, max_range 5 m) or a spinning LiDAR
          (rows x cols beams, max_range 30-60 m), in its own seeded room of
          boxes; voxel size drawn from {0.02, 0.05, 0.1, 0.2} m.

A no-return beam gets its endpoint at twice the max range along the beam, so
the reference's strict `length > max_range` clip turns it into free space.
All configs use prob_hit 0.7, prob_miss 0.4 and the thresholds 0.12/0.97.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .mapping import Config


def default_config(max_range: float) -> Config:
    return Config(max_range=max_range, fast_mode=False, accumulation_period=0.0, prob_hit=0.7,
                  prob_miss=0.4, prob_thres_min=0.12, prob_thres_max=0.97)


# ---------------------------------------------------------------------------
# Ray-scene intersection (float64, vectorised over rays)
# ---------------------------------------------------------------------------

def _hit_boxes(o, d, boxes, t_best):
    """Nearest entry of rays (origin o (3,), dirs d (N,3)) into axis-aligned
    boxes [(lo(3), hi(3)), ...]; updates t_best in place."""
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = 1.0 / d
    for lo, hi in boxes:
        t1 = (lo - o) * inv
        t2 = (hi - o) * inv
        tmin = np.nanmax(np.minimum(t1, t2), axis=1)
        tmax = np.nanmin(np.maximum(t1, t2), axis=1)
        ok = (tmax >= tmin) & (tmax > 0) & (tmin > 1e-6)
        t_best[ok] = np.minimum(t_best[ok], tmin[ok])


def _hit_room_inside(o, d, lo, hi, t_best):
    """Exit distance of rays from inside the box [lo, hi]."""
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = 1.0 / d
        t1 = (lo - o) * inv
        t2 = (hi - o) * inv
    tmax = np.nanmin(np.where(np.isfinite(np.maximum(t1, t2)), np.maximum(t1, t2), np.inf), axis=1)
    np.minimum(t_best, tmax, out=t_best)


def _hit_cylinders(o, d, cyls, t_best):
    """Vertical cylinders [(cx, cy, r, z0, z1), ...] (outer surface)."""
    a = d[:, 0] ** 2 + d[:, 1] ** 2
    for cx, cy, r, z0, z1 in cyls:
        ox, oy = o[0] - cx, o[1] - cy
        b = 2 * (ox * d[:, 0] + oy * d[:, 1])
        c = ox * ox + oy * oy - r * r
        disc = b * b - 4 * a * c
        ok = (disc >= 0) & (a > 1e-12)
        with np.errstate(invalid="ignore", divide="ignore"):
            t = (-b - np.sqrt(np.where(ok, disc, 0))) / (2 * a)
        z = o[2] + t * d[:, 2]
        ok &= (t > 1e-6) & (z >= z0) & (z <= z1)
        t_best[ok] = np.minimum(t_best[ok], t[ok])


def _azimuth_columns(o, ax, ay, half, cols):
    """Columns of a spinning-LiDAR grid (azimuth j * 2*pi/cols) within `half`
    radians (plus one column) of the direction (ax, ay) seen from o."""
    centre = np.arctan2(ay - o[1], ax - o[0])
    step = 2 * np.pi / cols
    j0 = int(np.floor((centre - half) / step)) - 1
    j1 = int(np.ceil((centre + half) / step)) + 1
    if j1 - j0 + 1 >= cols:
        return None
    return np.arange(j0, j1 + 1) % cols


def _lidar_subset(cols_idx, rows, cols):
    """Flat ray indices (row-major rows x cols grid) of the given columns."""
    return (np.arange(rows)[:, None] * cols + cols_idx[None, :]).reshape(-1)


def _hit_boxes_lidar(o, d, inv, boxes, t_best, rows, cols):
    """_hit_boxes for a rows x cols LiDAR grid, testing only the columns whose
    azimuth can reach each box (the same arithmetic per tested ray)."""
    for lo, hi in boxes:
        cx, cy = 0.5 * (lo[0] + hi[0]), 0.5 * (lo[1] + hi[1])
        rad = 0.5 * np.hypot(hi[0] - lo[0], hi[1] - lo[1])
        dist = np.hypot(cx - o[0], cy - o[1])
        idx = None
        if dist > rad * 1.01 + 1e-6:
            idx = _azimuth_columns(o, cx, cy, np.arcsin(min(1.0, rad / dist)) + 1e-3, cols)
        if idx is None:
            sub, isub = d, inv
        else:
            idx = _lidar_subset(idx, rows, cols)
            sub, isub = d[idx], inv[idx]
        t1 = (lo - o) * isub
        t2 = (hi - o) * isub
        tmin = np.nanmax(np.minimum(t1, t2), axis=1)
        tmax = np.nanmin(np.maximum(t1, t2), axis=1)
        ok = (tmax >= tmin) & (tmax > 0) & (tmin > 1e-6)
        if idx is None:
            t_best[ok] = np.minimum(t_best[ok], tmin[ok])
        else:
            sel = idx[ok]
            t_best[sel] = np.minimum(t_best[sel], tmin[ok])


def _hit_cylinders_lidar(o, d, cyls, t_best, rows, cols):
    """_hit_cylinders for a rows x cols LiDAR grid, column-culled likewise."""
    for cx, cy, r, z0, z1 in cyls:
        dist = np.hypot(cx - o[0], cy - o[1])
        idx = None
        if dist > r * 1.01 + 1e-6:
            idx = _azimuth_columns(o, cx, cy, np.arcsin(min(1.0, r / dist)) + 1e-3, cols)
        if idx is not None:
            idx = _lidar_subset(idx, rows, cols)
        sub = d if idx is None else d[idx]
        a = sub[:, 0] ** 2 + sub[:, 1] ** 2
        ox, oy = o[0] - cx, o[1] - cy
        b = 2 * (ox * sub[:, 0] + oy * sub[:, 1])
        c = ox * ox + oy * oy - r * r
        disc = b * b - 4 * a * c
        ok = (disc >= 0) & (a > 1e-12)
        with np.errstate(invalid="ignore", divide="ignore"):
            t = (-b - np.sqrt(np.where(ok, disc, 0))) / (2 * a)
        z = o[2] + t * sub[:, 2]
        ok &= (t > 1e-6) & (z >= z0) & (z <= z1)
        if idx is None:
            t_best[ok] = np.minimum(t_best[ok], t[ok])
        else:
            sel = idx[ok]
            t_best[sel] = np.minimum(t_best[sel], t[ok])


def _hit_ground(o, d, t_best, z=0.0):
    with np.errstate(divide="ignore", invalid="ignore"):
        t = (z - o[2]) / d[:, 2]
    ok = (d[:, 2] < 0) & (t > 0)
    t_best[ok] = np.minimum(t_best[ok], t[ok])


def lidar_directions(rows: int, cols: int, el_min=-25.0, el_max=15.0) -> np.ndarray:
    el = np.deg2rad(np.linspace(el_min, el_max, rows))
    az = np.arange(cols) * (2 * np.pi / cols)
    ce, se = np.cos(el)[:, None], np.sin(el)[:, None]
    d = np.stack([np.broadcast_to(ce * np.cos(az)[None, :], (rows, cols)),
                  np.broadcast_to(ce * np.sin(az)[None, :], (rows, cols)),
                  np.broadcast_to(se, (rows, cols))], axis=-1)
    return d.reshape(-1, 3)


def _to_pcl(o, d, r) -> np.ndarray:
    pts = np.empty((d.shape[0], 4), np.float32)
    pts[:, :3] = (o[None, :] + d * r[:, None]).astype(np.float32)
    pts[:, 3] = 1.0
    return pts


# ---------------------------------------------------------------------------
# Workloads
# ---------------------------------------------------------------------------

@dataclass
class Workload:
    name: str
    resolution: float
    max_range: float
    n_scans: int
    points_per_scan: int
    seed: int
    config: Config = field(default=None)

    def __post_init__(self):
        if self.config is None:
            self.config = default_config(self.max_range)

    def scan(self, k: int):
        """(points (N,4) float32, origin (3,) float64) of scan k."""
        raise NotImplementedError

    def describe(self) -> dict:
        return {"workload": self.name, "points_per_scan": self.points_per_scan, "scans": self.n_scans,
                "voxel_m": self.resolution, "max_range_m": self.max_range, "seed": self.seed}


class RoomWorkload(Workload):
    def __init__(self, name="small", seed=1, rows=64, cols=1024, n_scans=10, resolution=0.1,
                 max_range=30.0, sigma=0.02, no_return=0.05, n_boxes=20):
        super().__init__(name, resolution, max_range, n_scans, rows * cols, seed)
        rng = np.random.default_rng(seed)
        self.lo, self.hi = np.array([-20.0, -20.0, 0.0]), np.array([20.0, 20.0, 6.0])
        self.boxes = []
        while len(self.boxes) < n_boxes:
            c = rng.uniform([-18, -18], [18, 18])
            size = rng.uniform([0.3, 0.3, 0.5], [3.0, 3.0, 3.0])
            lo = np.array([c[0] - size[0] / 2, c[1] - size[1] / 2, 0.0])
            hi = np.array([c[0] + size[0] / 2, c[1] + size[1] / 2, size[2]])
            # keep the sensor path (x in [-1, 3], |y| < 1) clear
            if hi[0] > -1.5 and lo[0] < 3.5 and hi[1] > -1.5 and lo[1] < 1.5:
                continue
            self.boxes.append((lo, hi))
        self.dirs = lidar_directions(rows, cols)
        self.sigma, self.no_return, self.seed = sigma, no_return, seed

    def origin(self, k):
        return np.array([0.2 * k, 0.0, 1.5])

    def scan(self, k):
        o = self.origin(k)
        d = self.dirs
        t = np.full(d.shape[0], np.inf)
        _hit_room_inside(o, d, self.lo, self.hi, t)
        _hit_boxes(o, d, self.boxes, t)
        rng = np.random.default_rng([self.seed, k])
        r = t + rng.normal(0.0, self.sigma, t.shape)
        lost = (rng.random(t.shape) < self.no_return) | ~np.isfinite(t)
        r = np.where(lost, 2.0 * self.max_range, r)
        return _to_pcl(o, d, r), o


class StreetWorkload(Workload):
    def __init__(self, name="dense", seed=2, rows=128, cols=2048, n_scans=100, resolution=0.05,
                 max_range=60.0, sigma=0.01, no_return=0.03):
        super().__init__(name, resolution, max_range, n_scans, rows * cols, seed)
        rng = np.random.default_rng(seed)
        boxes, cyls = [], []
        # Buildings along both sides of a 20 m wide street running along x.
        for side in (-1, 1):
            x = -100.0
            while x < 100.0:
                w = rng.uniform(8, 25)
                depth = rng.uniform(10, 30)
                h = rng.uniform(5, 20)
                setback = rng.uniform(10, 14)
                y0 = side * setback
                y1 = side * (setback + depth)
                boxes.append((np.array([x, min(y0, y1), 0.0]), np.array([x + w, max(y0, y1), h])))
                x += w + rng.uniform(1, 6)
        # Parked cars.
        for _ in range(60):
            cx = rng.uniform(-100, 100)
            cy = rng.choice([-1, 1]) * rng.uniform(5.5, 8.0)
            boxes.append((np.array([cx - 2.2, cy - 0.9, 0.0]), np.array([cx + 2.2, cy + 0.9, 1.5])))
        # Poles and trees on the sidewalks.
        for _ in range(80):
            cx = rng.uniform(-100, 100)
            cy = rng.choice([-1, 1]) * rng.uniform(8.5, 9.8)
            r = rng.uniform(0.08, 0.5)
            cyls.append((cx, cy, r, 0.0, rng.uniform(3, 9)))
        self.boxes, self.cyls = boxes, cyls
        self.dirs = lidar_directions(rows, cols)
        self.rows, self.cols = rows, cols
        with np.errstate(divide="ignore"):
            self.inv_dirs = 1.0 / self.dirs
        self.sigma, self.no_return = sigma, no_return
        self.bounds_lo, self.bounds_hi = np.array([-100.0, -100.0, 0.0]), np.array([100.0, 100.0, 20.0])

    def origin(self, k):
        return np.array([-50.0 + 1.0 * k, 0.0, 1.8])

    def scan(self, k):
        o = self.origin(k)
        d = self.dirs
        t = np.full(d.shape[0], np.inf)
        _hit_ground(o, d, t)
        # Only primitives within reach of this scan.
        reach = 2.0 * self.max_range
        near_boxes = [b for b in self.boxes
                      if (b[0][0] - o[0] < reach) and (o[0] - b[1][0] < reach)]
        near_cyls = [c for c in self.cyls if abs(c[0] - o[0]) < reach]
        # Each primitive is tested against the beams whose azimuth reaches it.
        _hit_boxes_lidar(o, d, self.inv_dirs, near_boxes, t, self.rows, self.cols)
        _hit_cylinders_lidar(o, d, near_cyls, t, self.rows, self.cols)
        # The scene ends at its 200x200x20 m bounds: no return beyond.
        exit_t = np.full(d.shape[0], np.inf)
        _hit_room_inside(o, d, self.bounds_lo, self.bounds_hi, exit_t)
        t = np.where(t <= exit_t, t, np.inf)
        rng = np.random.default_rng([self.seed, k])
        r = t + rng.normal(0.0, self.sigma, t.shape)
        lost = (rng.random(t.shape) < self.no_return) | ~np.isfinite(t)
        r = np.where(lost, 2.0 * self.max_range, r)
        return _to_pcl(o, d, r), o


class StressWorkload(Workload):
    def __init__(self, name="stress", seed=3, n_rays=65536, n_scans=20, resolution=0.02, max_range=250.0,
                 origin=(5000.0, -3000.0, 40.0), special_frac=0.01):
        super().__init__(name, resolution, max_range, n_scans, n_rays, seed)
        self.base_origin = np.array(origin, np.float64)
        self.special_frac = special_frac

    def origin(self, k):
        return self.base_origin + np.array([0.37 * k, -0.21 * k, 0.05 * k])

    def scan(self, k):
        rng = np.random.default_rng([self.seed, k])
        n = self.points_per_scan
        o = self.origin(k)
        v = rng.normal(size=(n, 3))
        v /= np.linalg.norm(v, axis=1, keepdims=True)
        r = np.exp(rng.uniform(np.log(0.5), np.log(200.0), n))
        pts = _to_pcl(o, v, r)
        res = self.resolution
        n_sp = int(round(self.special_frac * n))
        idx = rng.choice(n, size=n_sp, replace=False)
        half = n_sp // 2
        # Quantiser boundaries: coordinates at (k - 1/2) * res (float32 nearest).
        for i in idx[:half]:
            axes = rng.random(3) < 0.6
            axes[rng.integers(3)] = True
            for a in np.nonzero(axes)[0]:
                kk = np.round(pts[i, a] / res)
                pts[i, a] = np.float32((kk - 0.5) * res)
        # DDA tie directions: voxel deltas with equal or small-ratio components.
        ovox = np.floor(o / res + 0.5)
        patterns = [(1, 1, 0), (1, 1, 1), (1, 3, 0), (2, 6, 0), (1, 1, 2), (3, 5, 0), (1, 3, 5), (2, 2, 1)]
        for i in idx[half:]:
            p = np.array(patterns[rng.integers(len(patterns))], np.float64)
            p = p[rng.permutation(3)] * rng.choice([-1, 1], 3)
            scale = rng.integers(1, max(2, int(150.0 / res / max(1.0, np.abs(p).sum()))))
            vox = ovox + p * scale
            pts[i, :3] = (vox * res).astype(np.float32)  # voxel centre
        return pts, o


def depth_directions(n: int, fov_h=90.0, fov_v=60.0, yaw=0.0, pitch=0.0) -> np.ndarray:
    """Unit rays of a pinhole depth camera subsampled to about n pixels of a
    640x480 image (4:3 grid), looking along yaw/pitch (degrees)."""
    w = max(4, min(640, int(round(np.sqrt(n * 4.0 / 3.0)))))
    h = max(3, min(480, int(np.ceil(n / w))))
    tx = np.tan(np.deg2rad(fov_h / 2)) * np.linspace(-1, 1, w)
    ty = np.tan(np.deg2rad(fov_v / 2)) * np.linspace(-1, 1, h)
    gx, gy = np.meshgrid(tx, ty)
    d = np.stack([np.ones_like(gx), gx, gy], axis=-1).reshape(-1, 3)[:n]
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    cy, sy, cp, sp = np.cos(np.deg2rad(yaw)), np.sin(np.deg2rad(yaw)), np.cos(np.deg2rad(pitch)), np.sin(np.deg2rad(pitch))
    rot = np.array([[cy * cp, -sy, -cy * sp], [sy * cp, cy, -sy * sp], [sp, 0.0, cp]])
    return d @ rot.T


class BatchedWorkload:
    """Independent maps of mixed sensors, one scan per map per step."""

    VOXELS = (0.02, 0.05, 0.1, 0.2)

    def __init__(self, name="batched", seed=4, n_maps=32, n_steps=50, n_min=2000, n_max=307200):
        self.name, self.seed, self.n_maps, self.n_steps = name, seed, n_maps, n_steps
        rng = np.random.default_rng(seed)
        self.maps = []
        for i in range(n_maps):
            n = int(round(np.exp(rng.uniform(np.log(n_min), np.log(n_max)))))
            depth = bool(rng.random() < 0.5)
            res = float(rng.choice(self.VOXELS))
            if depth:
                max_range = 5.0
                room = RoomWorkload(seed=1000 + i, n_boxes=20)
                dirs = depth_directions(n, yaw=rng.uniform(0, 360), pitch=rng.uniform(-20, 5))
            else:
                max_range = float(rng.uniform(30.0, 60.0))
                room = RoomWorkload(seed=1000 + i, n_boxes=30)
                room.lo, room.hi = np.array([-45.0, -45.0, 0.0]), np.array([45.0, 45.0, 12.0])
                rows = int(rng.choice([16, 32, 64, 128]))
                cols = max(8, n // rows)
                dirs = lidar_directions(rows, cols)[:n]
            self.maps.append(dict(n=dirs.shape[0], depth=depth, resolution=res, max_range=max_range, room=room,
                                  dirs=dirs, sigma=0.01, no_return=0.03, speed=rng.uniform(0.02, 0.2),
                                  heading=rng.uniform(0, 2 * np.pi)))
        self.resolutions = [m["resolution"] for m in self.maps]
        self.configs = [default_config(m["max_range"]) for m in self.maps]
        self.points_per_step = sum(m["n"] for m in self.maps)

    def origin(self, i, k):
        m = self.maps[i]
        step = m["speed"] * k
        return np.array([step * np.cos(m["heading"]), step * np.sin(m["heading"]), 1.2 + 0.01 * (i % 7)])

    def scan(self, i, k):
        """(points (N,4) float32, origin (3,) float64) of map i at step k."""
        m = self.maps[i]
        o = self.origin(i, k)
        d = m["dirs"]
        room = m["room"]
        t = np.full(d.shape[0], np.inf)
        _hit_room_inside(o, d, room.lo, room.hi, t)
        _hit_boxes(o, d, room.boxes, t)
        rng = np.random.default_rng([self.seed, i, k])
        r = t + rng.normal(0.0, m["sigma"], t.shape)
        lost = (rng.random(t.shape) < m["no_return"]) | ~np.isfinite(t)
        r = np.where(lost, 2.0 * m["max_range"], r)
        return _to_pcl(o, d, r), o

    def step(self, k):
        """[(points, origin)] of every map at step k (maps generated on
        several threads; numpy releases the interpreter lock)."""
        from concurrent.futures import ThreadPoolExecutor

        with ThreadPoolExecutor(max_workers=8) as ex:
            return list(ex.map(lambda i: self.scan(i, k), range(self.n_maps)))

    def describe(self) -> dict:
        return {"workload": self.name, "maps": self.n_maps, "steps": self.n_steps,
                "points_per_step": self.points_per_step, "seed": self.seed,
                "depth_maps": sum(m["depth"] for m in self.maps),
                "voxels_m": sorted(set(self.resolutions))}


class ServingWorkload:
    """Sensor streams for the serving loop: 8 LiDARs at 10 Hz (65k-262k
    points, 0.05 m voxels, max_range 30-60 m) and 8 depth cameras at 30 Hz
    (640x480 = 307,200 points, 0.02 m voxels, max_range 5 m), each in its own
    seeded room, moving along a heading. Arrivals are Poisson per stream."""

    def __init__(self, name="serving", seed=5, n_lidar=8, n_depth=8, lidar_hz=10.0, depth_hz=30.0,
                 distinct_scans=2):
        self.name, self.seed = name, seed
        rng = np.random.default_rng(seed)
        self.streams = []
        for i in range(n_lidar + n_depth):
            depth = i >= n_lidar
            if depth:
                n, res, max_range, hz = 307200, 0.02, 5.0, depth_hz
                room = RoomWorkload(seed=2000 + i, n_boxes=20)
                dirs = depth_directions(n, yaw=rng.uniform(0, 360), pitch=rng.uniform(-20, 5))
            else:
                rows = int(rng.choice([32, 64, 128]))
                n = int(rng.integers(65536, 262144 + 1)) // rows * rows
                res, max_range, hz = 0.05, float(rng.uniform(30.0, 60.0)), lidar_hz
                room = RoomWorkload(seed=2000 + i, n_boxes=30)
                room.lo, room.hi = np.array([-45.0, -45.0, 0.0]), np.array([45.0, 45.0, 12.0])
                dirs = lidar_directions(rows, n // rows)
            self.streams.append(dict(depth=depth, n=dirs.shape[0], resolution=res, max_range=max_range, hz=hz,
                                     room=room, dirs=dirs, speed=rng.uniform(0.02, 0.1),
                                     heading=rng.uniform(0, 2 * np.pi)))
        self.resolutions = [s["resolution"] for s in self.streams]
        self.configs = [default_config(s["max_range"]) for s in self.streams]
        self.distinct_scans = distinct_scans

    def origin(self, i, k):
        s = self.streams[i]
        step = s["speed"] * k
        return np.array([step * np.cos(s["heading"]), step * np.sin(s["heading"]), 1.3])

    def scan(self, i, k):
        s = self.streams[i]
        o = self.origin(i, k)
        d, room = s["dirs"], s["room"]
        t = np.full(d.shape[0], np.inf)
        _hit_room_inside(o, d, room.lo, room.hi, t)
        _hit_boxes(o, d, room.boxes, t)
        rng = np.random.default_rng([self.seed, i, k])
        r = t + rng.normal(0.0, 0.01, t.shape)
        lost = (rng.random(t.shape) < 0.03) | ~np.isfinite(t)
        r = np.where(lost, 2.0 * s["max_range"], r)
        return _to_pcl(o, d, r), o

    def arrivals(self, duration_s, seed=None):
        """Sorted [(time_s, stream)] of Poisson arrivals over duration_s."""
        rng = np.random.default_rng(self.seed if seed is None else seed)
        out = []
        for i, s in enumerate(self.streams):
            t = rng.exponential(1.0 / s["hz"])
            while t < duration_s:
                out.append((t, i))
                t += rng.exponential(1.0 / s["hz"])
        return sorted(out)

    def describe(self) -> dict:
        return {"workload": self.name, "streams": len(self.streams),
                "lidar": {"count": sum(not s["depth"] for s in self.streams), "hz": self.streams[0]["hz"],
                          "points": [s["n"] for s in self.streams if not s["depth"]], "voxel_m": 0.05},
                "depth": {"count": sum(s["depth"] for s in self.streams), "hz": self.streams[-1]["hz"],
                          "points": 307200, "voxel_m": 0.02, "max_range_m": 5.0},
                "seed": self.seed}


def get(name: str) -> Workload:
    if name == "small":
        return RoomWorkload()
    if name == "dense":
        return StreetWorkload()
    if name == "stress":
        return StressWorkload()
    if name == "batched":
        return BatchedWorkload()
    if name == "serving":
        return ServingWorkload()
    raise KeyError(name)
