"""The benchmark workloads of this path, with synthetic geometry of the named shapes.

cube_config   plain FP32 half tunnel 128x64x64, symmetry plane z=0, inlet u=0.08,
              sponge outlet over the last 16 cells, moving belt at inlet speed,
              tau0=0.51, Cs=0.1, axis-aligned cube of edge 22 cells centred at
              x=40 resting on the floor and cut by the symmetry plane.
f1_config     generic analytic F1 (src/engine/f1.ts:283-320) voxelized at 4.5 cm into
              a 256x96x80 half tunnel; wing angles seeded uniformly in 5-25 deg, ride
              heights in 10-60 mm; heat sources (brakes, exhaust, radiator) at T=1.
Both use the same collision parameters (u_in 0.08, tau0 0.51, Cs 0.1, sponge 16).
"""
import math

import numpy as np

from . import _abi
from .engine import DEG, ORIGIN_X, make_sim

CONFIG_SIM = dict(u_in=0.08, tau0=0.51, smag=0.1, sponge_cells=16.0)


def box_scene(center, half):
    s = _abi.Shape()
    s.kind = _abi.KIND_BOX
    s.pw, s.ph = 256, 128
    for k in range(3):
        s.box_center[k] = center[k]
        s.box_half[k] = half[k]
    return s


def cube_config(dims=(128, 64, 64), edge=22, center_x=40, h=0.045, storage="f32"):
    """Returns (dims, origin, h, sim, shape)."""
    origin = (0.0, 0.0, 0.0)
    half = edge / 2.0
    shape = box_scene((center_x * h, half * h, 0.0), (half * h, half * h, half * h))
    return tuple(dims), origin, h, make_sim(storage=storage, **CONFIG_SIM), shape


def config_f1_shape(seed=0, ride=None, rear_ride=None):
    """F1 Shape uniform with seeded wing angles (5-25 deg) and ride heights (10-60 mm)."""
    rng = np.random.default_rng(seed)
    ff, rm, rf = (rng.uniform(5.0, 25.0, 3) * DEG).tolist()
    r0, r1 = rng.uniform(0.010, 0.060, 2).tolist()
    s = _abi.Shape()
    s.kind = _abi.KIND_F1
    s.pw, s.ph = 256, 128
    s.front_flap, s.rear_main, s.rear_flap = ff, rm, rf
    s.ride_h = r0 if ride is None else ride
    s.rear_ride = r1 if rear_ride is None else rear_ride
    s.aoa = 6 * DEG
    s.width, s.axis_y, s.p_scale = 0.5, 1.0, 0.02
    s.heat_brakes = s.heat_engine = s.heat_rad = 1.0
    s.duct = 1.0
    return s


def f1_config(dims=(256, 96, 80), h=0.045, seed=0, storage="f32"):
    """Returns (dims, origin, h, sim, shape)."""
    return tuple(dims), (ORIGIN_X, 0.0, 0.0), h, make_sim(storage=storage, **CONFIG_SIM), config_f1_shape(seed)


def half_area_cells(solid, dims):
    """Projected frontal area of the full (mirrored) body in cells: 2x the (y, z)
    columns of the half domain that contain a solid cell."""
    nx, ny, nz = dims
    s = np.asarray(solid).reshape(nz, ny, nx)
    return 2 * int((s != 0).any(axis=2).sum())


def drag_coefficient(fx_per_step, u_in, area_cells):
    """Cd = 2 * Fx(half body) / (0.5 * rho0 * u^2 * A_full), lattice units, rho0 = 1."""
    return 2.0 * fx_per_step / (0.5 * u_in * u_in * area_cells)


def lift_coefficient(fy_per_step, u_in, area_cells):
    """Cl with the reference's sign convention (downforce = -Fy)."""
    return 2.0 * (-fy_per_step) / (0.5 * u_in * u_in * area_cells)


def cells_per_second_to_mlups(cells, steps, seconds):
    return cells * steps / seconds / 1e6


def bytes_per_lup(storage):
    """Algorithmic bytes per lattice update of the collide-stream kernel:
    19 loads + 19 stores of the storage type + the 4-byte cell word."""
    return 19 * 2 * (4 if storage in ("f32", 0) else 2) + 4


HEAT_BYTES_PER_CELL = 28  # fields 16 + emit 4 + tin 4 read, tout 4 written


def f1_large_config(storage="f32", seed=0):
    """The precision-sweep lattice: the same F1 at 512x192x160 (15.7 M cells), h = 2.25 cm."""
    return f1_config(dims=(512, 192, 160), h=0.0225, seed=seed, storage=storage)


AEROMAP_RIDE_MM = (10.0, 22.5, 35.0, 47.5, 60.0)


def aeromap_cases(seed=0, uneven=8):
    """The batched aero map: 25 lattices 256x96x80 (front x rear ride height in
    10-60 mm, serpentine order of src/ui/aeromap.ts:79-84, re-voxelized per case)
    plus `uneven` lattices whose sizes run linearly from 128x48x40 to 384x144x120
    over the same 11.52 m tunnel.  Returns [(dims, origin, h, shape, label)]."""
    from .sweep import aero_map_points
    out = []
    for p in aero_map_points(AEROMAP_RIDE_MM, AEROMAP_RIDE_MM):
        shape = config_f1_shape(seed, ride=p.front, rear_ride=p.rear)
        out.append(((256, 96, 80), (ORIGIN_X, 0.0, 0.0), 0.045, shape, f"front {p.front*1e3:.1f} mm rear {p.rear*1e3:.1f} mm"))
    for k in range(uneven):
        t = k / max(1, uneven - 1)
        nx = int(round((128 + t * 256) / 8)) * 8
        ny, nz = nx * 3 // 8, nx * 5 // 16
        out.append(((nx, ny, nz), (ORIGIN_X, 0.0, 0.0), 11.52 / nx, config_f1_shape(seed), f"uneven {nx}x{ny}x{nz}"))
    return out
