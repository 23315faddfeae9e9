"""Seeded synthetic lidar workloads (they stand in for the reference's private
AirSim recordings, which are not available).

Each config fixes the lidar, the scene generator, the trajectory and the TSDF
parameters.  Scans come from libscangen.so (analytic ray casting, C++).

  plain_small    16x64 lidar, 200x200 m plane + 40 boxes, circle r=40 m at
                 z=5 m, 1 m/s, 4 Hz; vs 0.5, T 4.0, W 1000, pub d2 2500,
                 gc d2 250000.  371 scans.
  multimap32     32 maps with plain_small parameters, each with its own
                 scene / trajectory seeds and a lidar of {16,32,64} channels x
                 {64,256,1024} azimuths drawn per map (1k-65k points).
  large_stream   64x1024 lidar (-25..+15 deg, 100 m); 400x400 m urban block
                 (400 boxes 2-30 m, 200 spheres r 0.3-2 m); random walk
                 10 m/s at z=2 m, 10 Hz; vs 0.1, T 0.4, pub d2 900,
                 gc d2 40000; 2M-block heap.  1000 scans.
  serving64      64 clients, Poisson 10 Hz each, scenes as large_stream,
                 lidar in {16x64, 32x512, 64x1024, 128x2048}, vs in
                 {0.05, 0.1, 0.2, 0.5}, T = 4 vs.
  stress8        128x2048 lidar (120 m, sigma 0.01) over a 1x1 km scene
                 (2000 boxes, 1000 spheres), 20 m/s, 10 Hz; vs 0.05, T 0.2,
                 gc d2 22500, pub d2 2500; 8 maps.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, replace

import numpy as np

from .engine import TsdfParams
from ._lib import LIB_DIR


class SceneCfg(C.Structure):
    _fields_ = [("half_extent", C.c_double), ("n_boxes", C.c_int), ("box_lo", C.c_double), ("box_hi", C.c_double),
                ("n_spheres", C.c_int), ("sphere_lo", C.c_double), ("sphere_hi", C.c_double), ("seed", C.c_uint64)]


class LidarCfg(C.Structure):
    _fields_ = [("channels", C.c_int), ("azimuths", C.c_int), ("elev_lo_deg", C.c_double),
                ("elev_hi_deg", C.c_double), ("max_range", C.c_double), ("sigma", C.c_double)]


class TrajCfg(C.Structure):
    _fields_ = [("kind", C.c_int), ("radius", C.c_double), ("height", C.c_double), ("speed", C.c_double),
                ("rate_hz", C.c_double), ("seed", C.c_uint64)]


_gen = None


def _lib():
    global _gen
    if _gen is None:
        p = LIB_DIR / "libscangen.so"
        if not p.exists():
            raise RuntimeError(f"{p} is missing: run __graft_entry__.build()")
        g = C.CDLL(str(p))
        g.sg_scene_create.restype = C.c_void_p
        g.sg_scene_create.argtypes = [C.POINTER(SceneCfg)]
        g.sg_scene_destroy.argtypes = [C.c_void_p]
        g.sg_pose.argtypes = [C.POINTER(TrajCfg), C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        g.sg_scan.restype = C.c_int64
        g.sg_scan.argtypes = [C.c_void_p, C.POINTER(LidarCfg), C.POINTER(C.c_double), C.c_double, C.c_uint64,
                              C.c_int, C.c_void_p, C.c_int64, C.c_int]
        _gen = g
    return _gen


@dataclass(frozen=True)
class Lidar:
    channels: int
    azimuths: int
    elev_lo: float
    elev_hi: float
    max_range: float
    sigma: float


@dataclass(frozen=True)
class Scene:
    half_extent: float
    n_boxes: int
    box_lo: float
    box_hi: float
    n_spheres: int = 0
    sphere_lo: float = 0.0
    sphere_hi: float = 0.0


@dataclass(frozen=True)
class Traj:
    kind: int  # 0 circle, 1 random walk
    radius: float
    height: float
    speed: float
    rate_hz: float


@dataclass(frozen=True)
class MapSpec:
    lidar: Lidar
    scene: Scene
    traj: Traj
    params: TsdfParams
    heap_blocks: int
    seed: int


class ScanSource:
    """Scans of one map: scan(k) -> (xyz (n,3) float32, origin (3,) float32)."""

    def __init__(self, spec: MapSpec, threads: int | None = None):
        g = _lib()
        self.spec = spec
        s = spec.scene
        self._scene_cfg = SceneCfg(s.half_extent, s.n_boxes, s.box_lo, s.box_hi, s.n_spheres, s.sphere_lo,
                                   s.sphere_hi, spec.seed)
        self._scene = g.sg_scene_create(C.byref(self._scene_cfg))
        l = spec.lidar
        self._lidar = LidarCfg(l.channels, l.azimuths, l.elev_lo, l.elev_hi, l.max_range, l.sigma)
        t = spec.traj
        self._traj = TrajCfg(t.kind, t.radius, t.height, t.speed, t.rate_hz, spec.seed * 7919 + 17)
        self.threads = threads or min(16, os.cpu_count() or 1)
        self.rays = l.channels * l.azimuths

    def pose(self, k: int):
        pos = (C.c_double * 3)()
        yaw = C.c_double()
        _lib().sg_pose(C.byref(self._traj), int(k), pos, C.byref(yaw))
        return np.array(pos[:], np.float64), yaw.value

    def scan(self, k: int):
        pos, yaw = self.pose(k)
        out = np.empty((self.rays, 3), np.float32)
        n = _lib().sg_scan(self._scene, C.byref(self._lidar), (C.c_double * 3)(*pos), yaw,
                           self.spec.seed * 104729 + 3, int(k), out.ctypes.data, self.rays, self.threads)
        return out[:n].copy(), pos.astype(np.float32)

    def __del__(self):
        try:
            _lib().sg_scene_destroy(self._scene)
        except Exception:
            pass


# ---- named configs ----------------------------------------------------------
LIDAR_SMALL = Lidar(16, 64, -15.0, 15.0, 50.0, 0.02)
SCENE_SMALL = Scene(100.0, 40, 1.0, 10.0)
TRAJ_CIRCLE = Traj(0, 40.0, 5.0, 1.0, 4.0)
PARAMS_SMALL = TsdfParams(0.5, 4.0, 1000.0, 2500.0, 250000.0)

SCENE_URBAN = Scene(200.0, 400, 2.0, 30.0, 200, 0.3, 2.0)
LIDAR_LARGE = Lidar(64, 1024, -25.0, 15.0, 100.0, 0.02)
TRAJ_WALK10 = Traj(1, 200.0, 2.0, 10.0, 10.0)
PARAMS_LARGE = TsdfParams(0.1, 0.4, 1000.0, 900.0, 40000.0)

LIDAR_STRESS = Lidar(128, 2048, -25.0, 15.0, 120.0, 0.01)
SCENE_STRESS = Scene(500.0, 2000, 2.0, 30.0, 1000, 0.3, 2.0)
TRAJ_WALK20 = Traj(1, 500.0, 2.0, 20.0, 10.0)
PARAMS_STRESS = TsdfParams(0.05, 0.2, 1000.0, 2500.0, 22500.0)


def plain_small(seed: int = 0, heap_blocks: int = 65536) -> MapSpec:
    return MapSpec(LIDAR_SMALL, SCENE_SMALL, TRAJ_CIRCLE, PARAMS_SMALL, heap_blocks, seed)


def multimap32(n_maps: int = 32, base_seed: int = 1000, heap_blocks: int = 65536) -> list[MapSpec]:
    rng = np.random.default_rng(base_seed)
    out = []
    for m in range(n_maps):
        ch = int(rng.choice([16, 32, 64]))
        az = int(rng.choice([64, 256, 1024]))
        lid = replace(LIDAR_SMALL, channels=ch, azimuths=az)
        out.append(MapSpec(lid, SCENE_SMALL, TRAJ_CIRCLE, PARAMS_SMALL, heap_blocks, base_seed + m))
    return out


def large_stream(seed: int = 2000, heap_blocks: int = 2 * 1024 * 1024) -> MapSpec:
    return MapSpec(LIDAR_LARGE, SCENE_URBAN, TRAJ_WALK10, PARAMS_LARGE, heap_blocks, seed)


def serving64(n_clients: int = 64, base_seed: int = 3000, heap_blocks: int | None = None) -> list[MapSpec]:
    rng = np.random.default_rng(base_seed)
    shapes = [(16, 64), (32, 512), (64, 1024), (128, 2048)]
    out = []
    for c in range(n_clients):
        ch, az = shapes[int(rng.integers(0, 4))]
        vs = float(rng.choice([0.05, 0.1, 0.2, 0.5]))
        params = TsdfParams(vs, 4 * vs, 1000.0, 900.0, 40000.0)
        lid = replace(LIDAR_LARGE, channels=ch, azimuths=az)
        hb = heap_blocks or (1 << 18)
        out.append(MapSpec(lid, SCENE_URBAN, TRAJ_WALK10, params, hb, base_seed + c))
    return out


def stress8(n_maps: int = 8, base_seed: int = 4000, heap_blocks: int = 1 << 22) -> list[MapSpec]:
    return [MapSpec(LIDAR_STRESS, SCENE_STRESS, TRAJ_WALK20, PARAMS_STRESS, heap_blocks, base_seed + m)
            for m in range(n_maps)]
