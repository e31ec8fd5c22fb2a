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
    c.mixed_inner_tolerance = 1e-4
    c.mixed_max_refinements = 12
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
