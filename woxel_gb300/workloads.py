"""Seeded synthetic workloads standing in for the benchmark configurations.

The reference renders .vdb level sets (teapot, ISS, ...) that are not
available here; these generators reproduce the shapes, sizes and value
distributions the benchmark names:
  sphere    one f32 narrow-band sphere, r=64 voxels at the origin, band +-3,
            camera (0,0,200) -> origin, 60 deg, 640x480
  spheres   union of 2000 spheres, r ~ U[4,40], centres U[-1024,1024)^3, band +-3,
            seed 2; 16 orbit cameras at radius 3000, 1920x1080, 60 deg
  noise     4096^3 domain [-2048,2048)^3, 8^3 leaves where 3-octave value noise
            exceeds the 98th percentile (2.0% leaves), voxels active with p=0.5;
            8 views at radius 3500, 3840x2160, first active voxel (mode 0)
  mixed     256 requests over {sphere, spheres}, resolution uniform over
            {256x256, 640x480, 1280x720, 1920x1080, 3840x2160}, orbit poses at
            radius 200 (sphere) or 3000 (spheres)
Render mode 3 (Lambert, the reference app's default) except for `noise`.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import Topology, orbit_eyes, state_build

RESOLUTIONS = [(256, 256), (640, 480), (1280, 720), (1920, 1080), (3840, 2160)]


@dataclass
class Frame:
    grid: str
    width: int
    height: int
    eye: tuple
    mode: int = 3
    fovy: float = 60.0

    @property
    def rays(self) -> int:
        return (self.width // 8) * 8 * (self.height // 4) * 4

    def state(self):
        return state_build(eye=self.eye, target=(0.0, 0.0, 0.0), aspect=self.width / self.height, fovy=self.fovy,
                           width=float(self.width), mode=self.mode)


@dataclass
class Workload:
    name: str
    grids: dict = field(default_factory=dict)  # name -> zero-arg Topology factory
    frames: list = field(default_factory=list)

    @property
    def rays(self) -> int:
        return sum(f.rays for f in self.frames)


def sphere_topology(seed: int = 0) -> Topology:
    """Config-1 generator; seed > 0 moves the centre and radius (distinct resident grids)."""
    if seed == 0:
        return Topology.sphere((0.0, 0.0, 0.0), 64.0, 3.0)
    rng = np.random.default_rng(seed)
    c = rng.uniform(-512, 512, 3)
    return Topology.sphere(tuple(float(x) for x in c), float(rng.uniform(48, 96)), 3.0)


def spheres_topology(seed: int = 2) -> Topology:
    return Topology.spheres(2000, 4.0, 40.0, -1024.0, 1024.0, 3.0, seed)


def sphere_values(topo: Topology) -> np.ndarray:
    """Level-set values of sphere_topology's grid (zero-crossing mode)."""
    return topo.sphere_values((0.0, 0.0, 0.0), 64.0, 3.0)


def spheres_values(topo: Topology, seed: int = 2) -> np.ndarray:
    """Level-set values of spheres_topology's grid (zero-crossing mode)."""
    return topo.spheres_values(2000, 4.0, 40.0, -1024.0, 1024.0, 3.0, seed)


def noise_topology(seed: int = 3) -> Topology:
    return Topology.noise_leaves(-2048, 4096, 0.02, 0.5, seed)


def sphere_frames() -> list:
    return [Frame("sphere", 640, 480, (0.0, 0.0, 200.0))]


def spheres_frames(count: int = 16, seed: int = 16) -> list:
    return [Frame("spheres", 1920, 1080, tuple(float(x) for x in e)) for e in orbit_eyes(count, 3000.0, seed)]


def noise_frames(count: int = 8, seed: int = 8) -> list:
    return [Frame("noise", 3840, 2160, tuple(float(x) for x in e), mode=0) for e in orbit_eyes(count, 3500.0, seed)]


def mixed_frames(count: int = 256, seed: int = 4) -> list:
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        g = "sphere" if rng.integers(0, 2) == 0 else "spheres"
        w, h = RESOLUTIONS[int(rng.integers(0, len(RESOLUTIONS)))]
        radius = 200.0 if g == "sphere" else 3000.0
        eye = orbit_eyes(1, radius, int(rng.integers(0, 2**62)))[0]
        out.append(Frame(g, w, h, tuple(float(x) for x in eye)))
    return out


def workload(name: str) -> Workload:
    if name == "sphere":
        return Workload(name, {"sphere": sphere_topology}, sphere_frames())
    if name == "spheres":
        return Workload(name, {"spheres": spheres_topology}, spheres_frames())
    if name == "noise":
        return Workload(name, {"noise": noise_topology}, noise_frames())
    if name == "mixed":
        return Workload(name, {"sphere": sphere_topology, "spheres": spheres_topology}, mixed_frames())
    raise ValueError(f"unknown workload {name!r}")
