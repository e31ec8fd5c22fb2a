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
