"""Helpers shared by the parity tests: paired oracle/GPU simulations on one scene."""
from __future__ import annotations

import numpy as np

from garm import capi, scenes

STATE_FIELDS = [capi.FIELD_VELOCITY, capi.FIELD_LEVEL_SET, capi.FIELD_REF_MAP, capi.FIELD_REF_MAP_GRAD,
                capi.FIELD_REF_LEVEL_SET, capi.FIELD_REF_LEVEL_SET_GRAD, capi.FIELD_ADV_REGION,
                capi.FIELD_ORI_LEVEL_SET, capi.FIELD_TMP_LEVEL_SET]


def host_default_config(**kw) -> capi.Config:
    """garm_config_default restated on the host (checked against the library in test_capi_abi)."""
    c = capi.Config()
    c.precision = capi.PRECISION_FP64
    c.reinit_iters = 30
    c.reinit_cfl = 0.9
    c.reinit_interval = 1
    c.cg_tolerance = 1e-8
    c.cg_max_iters = 2000
    c.boundary_extrap_radius = 6.0
    c.air_extrap_radius = 15.0
    c.rm_threshold = 0.883022221559489
    c.rm_band = 4.0
    c.rm_ratio = 1e-5
    c.enable_gravity = 1
    c.mixed_residual_drop = 0.1
    c.mixed_replace_interval = 0
    c.cg_cells_per_block = 0
    c.record_volume = 0
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def load_scene(sim, scene: scenes.Scene) -> None:
    sim.upload(capi.FIELD_LEVEL_SET, scene.phi.ravel())
    sim.upload(capi.FIELD_VELOCITY, scene.velocity)


def copy_state(dst, src) -> None:
    for f in STATE_FIELDS:
        dst.upload(f, src.download(f))


def linf(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if a.size == 0:
        return 0.0
    return float(np.max(np.abs(a - b)))


def rel(a, b) -> float:
    scale = max(float(np.max(np.abs(np.asarray(b, dtype=np.float64)))), 1e-300)
    return linf(a, b) / scale


def velocity_check(g_u, o_u, fraction, rtol: float):
    """Compare staggered velocities.  Faces of the fluid domain (fraction < 1)
    must agree to `rtol` of max|u|.  On solid faces (fraction == 1) the wall
    condition of Boundary::enforce (Boundary.cpp:98-110) branches on the sign of
    the normal velocity vn; where vn is zero up to rounding the two sides may take
    different branches, which leaves one at u and the other at 0.2·u (the 0.8
    tangential damping).  Those faces are counted, every other solid-face
    mismatch fails.  Returns (interior relative error, number of tie faces)."""
    g_u = np.asarray(g_u, dtype=np.float64)
    o_u = np.asarray(o_u, dtype=np.float64)
    scale = max(float(np.max(np.abs(o_u))), 1e-300)
    diff = np.abs(g_u - o_u)
    fluid = fraction < 1
    inner = float(np.max(diff[fluid], initial=0.0)) / scale
    bad = (~fluid) & (diff > rtol * scale)
    ties = 0
    for gv, ov in zip(g_u[bad], o_u[bad]):
        if abs(gv - 0.2 * ov) <= rtol * scale + 1e-6 * abs(ov) or abs(ov - 0.2 * gv) <= rtol * scale + 1e-6 * abs(gv):
            ties += 1
        else:
            raise AssertionError(f"solid-face velocity mismatch not explained by the wall-condition tie: {gv} vs {ov}")
    return inner, ties


def band_error(a, b, ref_phi, dx: float, band: float = 3.0) -> float:
    """L∞ of a-b over cells with |ref_phi| <= band·dx (the accuracy band of the
    reference's own error measure, TestReinit.cpp:162-171 and TestAdvect2D.cpp:250-264)."""
    m = np.abs(np.asarray(ref_phi)) <= band * dx
    if not np.any(m):
        return 0.0
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))[m]))


# --- Rotation case of the reference's GA advection test (TestAdvect2D.cpp:32-59, 256-290) ---
ROT_LENGTH, ROT_DT, ROT_FRAMES_PER_TURN = 10.0, 0.02, 314


def zalesak_phi(x, y):
    """Slotted disk: circle (0, 2.5) r 1.5 minus the box [-0.25, 0.25] x [0, 3.5]
    (TestAdvect2D.cpp:33-41, 57-58, lengths x 10)."""
    circle = np.sqrt(x * x + (y - 2.5) ** 2) - 1.5
    box = scenes.box_sdf([x, y], [-0.25, 0.0], [0.5, 3.5])
    return np.maximum(circle, -box)


def rotation_case(s: int):
    """Grid (s^2 cells on [-5, 5]^2, no solid ring), cell φ, face velocity (.sav layout) and the
    angular speed of one turn per ROT_FRAMES_PER_TURN steps of ROT_DT."""
    dx = ROT_LENGTH / s
    grid = capi.grid_desc(2, [s, s], dx, [0.0, 0.0], boundary_width=0)
    c = -ROT_LENGTH / 2 + (np.arange(s) + 0.5) * dx
    f = -ROT_LENGTH / 2 + np.arange(s + 1) * dx
    omega = 2 * np.pi / (ROT_FRAMES_PER_TURN * ROT_DT)
    Y, X = np.meshgrid(c, c, indexing="ij")
    phi = np.ascontiguousarray(zalesak_phi(X, Y))
    yx, xx = np.meshgrid(c, f, indexing="ij")     # x-faces: shape (s, s+1)
    yy, xy = np.meshgrid(f, c, indexing="ij")     # y-faces: shape (s+1, s)
    u = np.concatenate([(-yx * omega).ravel(), (xy * omega).ravel()])
    return grid, phi, u, omega


def rotation_truth(s: int, steps: int):
    """The initial shape rotated by steps·ROT_DT·ω, at the cell centres."""
    dx = ROT_LENGTH / s
    c = -ROT_LENGTH / 2 + (np.arange(s) + 0.5) * dx
    Y, X = np.meshgrid(c, c, indexing="ij")
    a = 2 * np.pi * steps / ROT_FRAMES_PER_TURN
    return zalesak_phi(np.cos(a) * X + np.sin(a) * Y, -np.sin(a) * X + np.cos(a) * Y)


def run_rotation(sim, s: int, steps: int) -> np.ndarray:
    """GA advection of ξ and Π in the steady rotation (velocity re-uploaded each step),
    then φ = φ0(ξ) by the compose stage; returns φ."""
    grid, phi, u, _ = rotation_case(s)
    sim.upload(capi.FIELD_LEVEL_SET, phi.ravel())
    sim.upload(capi.FIELD_VELOCITY, u)
    sim.initialize()
    sim.stage("restart")
    sim.upload(capi.FIELD_ADV_REGION, np.ones(s * s, dtype=np.uint8))  # no air clamp
    for _ in range(steps):
        sim.upload(capi.FIELD_VELOCITY, u)
        sim.stage("advect", ROT_DT)
    sim.stage("compose")
    return sim.download(capi.FIELD_LEVEL_SET).reshape(s, s)


def band_l1(phi, truth, dx, band: float = 3.0) -> float:
    """Mean |φ - truth| over cells with |truth| <= band·dx (TestAdvect2D.cpp:236-251)."""
    m = np.abs(truth) <= band * dx
    return float(np.mean(np.abs(phi - truth)[m]))
