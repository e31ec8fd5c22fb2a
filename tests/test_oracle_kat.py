"""Known-answer tests of the CPU oracle, taken from the behaviour the
reference's own test programs check (Source/Test/): analytic reinitialisation
(TestReinit.cpp:89-171), polynomial reproduction of the interpolants, rigid
rotation of the reference map (TestAdvect2D.cpp:32-63), plus invariants of
the full step (divergence-free projection, restart resets ξ and Π)."""
from __future__ import annotations

import numpy as np
import pytest

from garm import capi, scenes
from helpers import host_default_config, load_scene, linf


def test_hermite_reproduces_tricubic_polynomials(oracle_mod):
    # p(x,y,z) = x^3 + y^2 z + x y z - 2 y^3 + z^2: cubic per axis, so tricubic
    # Hermite with exact values and gradients (mixed derivatives by central
    # differences of the gradient are exact here) reproduces it.
    n, dx = 10, 0.1
    c = (np.arange(n) + 0.5) * dx
    Z, Y, X = np.meshgrid(c, c, c, indexing="ij")
    p = X**3 + Y**2 * Z + X * Y * Z - 2 * Y**3 + Z**2
    g = np.stack([3 * X**2 + Y * Z, 2 * Y * Z + X * Z - 6 * Y**2, Y**2 + X * Y + 2 * Z], axis=-1)
    rng = np.random.default_rng(1)
    pts = rng.uniform(0.2 + dx / 2, 0.7, size=(200, 3))
    v, gr = oracle_mod.hermite_eval(p, g, dx, [dx / 2] * 3, pts)
    x, y, z = pts[:, 0], pts[:, 1], pts[:, 2]
    exact = x**3 + y**2 * z + x * y * z - 2 * y**3 + z**2
    assert np.max(np.abs(v - exact)) < 1e-12
    ex_g = np.stack([3 * x**2 + y * z, 2 * y * z + x * z - 6 * y**2, y**2 + x * y + 2 * z], axis=-1)
    assert np.max(np.abs(gr - ex_g)) < 1e-10


def test_cubic_lagrange_reproduces_cubics(oracle_mod):
    n, dx = 12, 0.5
    c = np.arange(n) * dx
    Y, X = np.meshgrid(c, c, indexing="ij")
    f = X**3 - 2 * X * Y**2 + Y**3 + 1
    rng = np.random.default_rng(2)
    pts = rng.uniform(2 * dx, (n - 3) * dx, size=(100, 2))
    out = oracle_mod.cubic_eval(f, dx, [0.0, 0.0], pts)
    x, y = pts[:, 0], pts[:, 1]
    assert np.max(np.abs(out - (x**3 - 2 * x * y**2 + y**3 + 1))) < 1e-10


@pytest.mark.parametrize("case", [0, 1, 3])
def test_weno5_reinit_converges_to_sdf(oracle_mod, case):
    """TestReinit cases 0, 1, 3 (distorted circles): the band-limited L1 error
    to the exact SDF drops far below its initial value."""
    n, length = 100, 10.0
    dx = length / n
    x = (np.arange(n) + 0.5) * dx - length / 2
    X, Y = np.meshgrid(x, x, indexing="xy")
    r = np.sqrt(X * X + Y * Y)
    if case == 0:
        r0 = 0.2313 * length
        maxd = length / np.sqrt(2) - r0
        phi = (np.exp(r - r0) - 1) * (maxd / (np.exp(maxd) - 1))
    elif case == 1:
        r0 = length / 4
        f = (X - r0) ** 2 + (Y - r0) ** 2 + 0.1 * r0 * r0
        phi = f * (r - r0) / (2 * (length / 2 + r0) ** 2 + 0.1 * r0 * r0)
    else:
        r0 = 0.2313 * length
        phi = (r - r0) * 2.0
    sdf = r - r0

    def err(ph):
        m = np.abs(ph) <= 3 * dx
        return np.mean(np.abs(ph - sdf)[m])

    e0 = err(phi)
    out = oracle_mod.reinit(phi, dx, 100, 0.5)
    assert err(out) < 0.1 * e0
    assert err(out) < 0.05 * dx


def test_weno5_keeps_a_planar_sdf(oracle_mod):
    # the clamped edges are not a plane; 2 iterations of 3 sub-stages reach 18 cells in
    n, dx = 48, 0.025
    c = (np.arange(n) + 0.5) * dx
    Z, Y, X = np.meshgrid(c, c, c, indexing="ij")
    phi = 0.3 * X + 0.4 * Y + np.sqrt(1 - 0.25) * Z - 0.5
    out = oracle_mod.reinit(phi, dx, 2, 0.9)
    inner = (slice(19, -19),) * 3
    assert np.max(np.abs(out - phi)[inner]) < 1e-10


def test_weno5_reinit_amplifies_rounding_along_3d_diagonals(oracle_mod):
    """A property of the reference's constants, not of any port: Reinitialization::solve<5>
    with dτ = 0.9·dx (LevelSetLiquid.cpp:1156) amplifies small perturbations of level sets
    whose normal lies near a 3D diagonal.  Dimension by dimension, the TVD-RK3/WENO5 step
    moves information at 0.9·(|n_x| + |n_y| + |n_z|) cells per step, 1.56 along (1,1,1)
    against 0.9 along an axis.  A planar distance function is a fixed point, so the oracle
    run twice, once on it and once on it times 1 + 1e-12·noise, shows the growth directly:
    along (1,1,1) at dτ = 0.9·dx the 30 iterations amplify the difference 20-60 times
    (also at 0.7·dx); along an axis they damp it, and at dτ = 0.5·dx it stays near its
    size.  Away from the interface (beyond the reach of its
    information, |φ| > 15·dx in a scene) FP32 and FP64 runs therefore differ by amplified
    rounding, while inside the band they agree."""
    n = 40
    dx = 1.0 / n
    c = (np.arange(n) + 0.5) * dx
    Z, Y, X = np.meshgrid(c, c, c, indexing="ij")
    noise = 1 + 1e-12 * np.random.default_rng(0).standard_normal((n, n, n))
    inner = (slice(8, -8),) * 3

    def gain(phi, cfl):
        d_in = np.max(np.abs(phi * noise - phi)[inner])
        d_out = np.max(np.abs(oracle_mod.reinit(phi * noise, dx, 30, cfl) - oracle_mod.reinit(phi, dx, 30, cfl))[inner])
        return d_out / d_in

    diag = (X + Y + Z) / np.sqrt(3) - 0.1
    assert gain(diag, 0.9) > 10
    assert gain(diag, 0.5) < 3
    assert gain(X - 0.1, 0.9) < 1


def test_far_field_does_not_feed_back_into_the_band(oracle_mod):
    """The cells beyond the level-set band (|φ| > 15·dx) are where the reinitialisation
    amplifies rounding (previous test).  Perturbing all of them by up to 0.1·dx, the size
    of the FP32/FP64 difference there at 128^3, and restarting (φ0 = φ takes the perturbed
    values into the state that later steps read) moves φ inside the band by at most
    1e-3·dx and the velocity by at most 1e-4 of max|u| over the next three steps."""
    from helpers import LEVEL_SET_BAND
    sc = scenes.dam_break(3, 36)
    dx = sc.grid.spacing

    def evolved():
        o = oracle_mod.OracleSim(sc.grid, host_default_config())
        load_scene(o, sc)
        o.initialize()
        o.stage("restart")
        for dt in scenes.frame_time_steps(o.max_speed, 3, 25, 1.0, dx):
            o.advance(dt)
        return o

    a, b = evolved(), evolved()
    phi = b.download(capi.FIELD_LEVEL_SET)
    far = np.abs(phi) > LEVEL_SET_BAND * dx
    assert far.sum() > phi.size // 4
    b.upload(capi.FIELD_LEVEL_SET, phi + far * np.random.default_rng(1).uniform(-0.1, 0.1, phi.shape) * dx)
    a.stage("restart")
    b.stage("restart")
    for dt in scenes.frame_time_steps(a.max_speed, 3, 25, 1.0, dx):
        a.advance(dt)
        b.advance(dt)
        pa, pb = a.download(capi.FIELD_LEVEL_SET), b.download(capi.FIELD_LEVEL_SET)
        band = np.abs(pa) <= LEVEL_SET_BAND * dx
        assert np.max(np.abs(pa - pb)[band]) <= 1e-3 * dx
        ua, ub = a.download(capi.FIELD_VELOCITY), b.download(capi.FIELD_VELOCITY)
        assert np.max(np.abs(ua - ub)) <= 1e-4 * np.max(np.abs(ua))
    a.close()
    b.close()


def test_restart_resets_reference_map(oracle_mod):
    sc = scenes.dam_break(2, 24)
    o = oracle_mod.OracleSim(sc.grid, host_default_config())
    load_scene(o, sc)
    o.initialize()
    o.advance(0.02)
    o.stage("restart")
    xi = o.download(capi.FIELD_REF_MAP).reshape(-1, 2)
    pi = o.download(capi.FIELD_REF_MAP_GRAD).reshape(-1, 4)
    pos = scenes.cell_positions(sc.grid)
    assert np.array_equal(xi[:, 0], np.broadcast_to(pos[0], sc.phi.shape).ravel())
    assert np.array_equal(xi[:, 1], np.broadcast_to(pos[1], sc.phi.shape).ravel())
    assert np.array_equal(pi, np.tile([1.0, 0.0, 0.0, 1.0], (len(pi), 1)))
    assert np.array_equal(o.download(capi.FIELD_REF_LEVEL_SET), o.download(capi.FIELD_LEVEL_SET))


def discrete_divergence(sc, u_flat, phi, frac, bvel):
    """Divergence of Projector::buildLinearSystem's rhs (Projector.cpp:34-62) per liquid cell."""
    g = sc.grid
    sh = capi.field_shapes(g)
    faces, off = [], 0
    for s in sh["faces"]:
        m = int(np.prod(s))
        faces.append((u_flat[off:off + m].reshape(s), frac[off:off + m].reshape(s), bvel[off:off + m].reshape(s)))
        off += m
    div = np.zeros(sh["cell"])
    dim = g.dim
    for a in range(dim):
        u, f, b = faces[a]
        w = 1 - f
        flux = np.where(w > 0, w * u, 0) + np.where(w < 1, (1 - w) * b, 0)
        ax = dim - 1 - a
        hi = [slice(None)] * dim; lo = [slice(None)] * dim
        hi[ax] = slice(1, None); lo[ax] = slice(0, -1)
        div += flux[tuple(hi)] - flux[tuple(lo)]
    return div


def test_projection_makes_liquid_divergence_free(oracle_mod):
    sc = scenes.drop(24, seed=5)
    o = oracle_mod.OracleSim(sc.grid, host_default_config())
    load_scene(o, sc)
    o.initialize()
    o.stage("restart")
    o.advance(0.01)
    phi = o.download(capi.FIELD_LEVEL_SET).reshape(sc.phi.shape)
    u = o.download(capi.FIELD_VELOCITY).copy()
    # apply gravity and project once more from this state
    o.stage("body_force", 0.01)
    u0 = o.download(capi.FIELD_VELOCITY)
    st = o.stage("project")
    assert st["cg_residual"] <= 1e-8
    frac = o.download(capi.FIELD_FRACTION)
    bvel = o.download(capi.FIELD_BOUNDARY_VELOCITY)
    div0 = discrete_divergence(sc, u0, phi, frac, bvel)
    div1 = discrete_divergence(sc, o.download(capi.FIELD_VELOCITY), phi, frac, bvel)
    p = o.download(capi.FIELD_PRESSURE).reshape(sc.phi.shape)
    interior = (p != 0)
    # cells fully surrounded by unknowns have no ghost-fluid term: divergence ~ 0
    assert np.max(np.abs(div1[interior])) < 1e-5 * max(1.0, np.max(np.abs(div0[interior])))
    assert u is not None


def test_dam_break_steps_are_deterministic_and_bounded(oracle_mod):
    sc = scenes.dam_break(2, 32)
    res = []
    for threads in (1, 4):
        oracle_mod.set_threads(threads)
        o = oracle_mod.OracleSim(sc.grid, host_default_config())
        load_scene(o, sc)
        o.initialize()
        o.stage("restart")
        for dt in scenes.frame_time_steps(o.max_speed, 5, 25, 1.0, sc.grid.spacing):
            st = o.advance(dt)
            assert st["status"] == capi.OK
        res.append(o.download(capi.FIELD_LEVEL_SET))
    oracle_mod.set_threads(0)
    assert np.array_equal(res[0], res[1])  # fixed-order reductions: thread-count independent
    assert np.all(np.isfinite(res[0]))


def test_oracle_reports_not_converged(oracle_mod):
    sc = scenes.drop(12, seed=2)
    o = oracle_mod.OracleSim(sc.grid, host_default_config(cg_max_iters=1))
    load_scene(o, sc)
    assert o.initialize() == capi.NOT_CONVERGED


def test_ga_advection_rotation_converges(oracle_mod):
    """Known-answer test after the reference's GA advection program (TestAdvect2D.cpp,
    Rotation case, Hermite + reference map): the slotted disk turned half a revolution
    by the hot path's own stages (velocity re-uploaded each step so it stays the steady
    rotation; ξ, Π advected; φ = φ0(ξ) composed).  The band L1 error against the
    rotated shape is small and falls about 4x from 50 to 100 cells per axis; beyond
    that the RK2 backtrace's time error (|x|(ω dt)^3/6 per step) sets a floor."""
    from helpers import ROT_LENGTH, band_l1, rotation_case, rotation_truth, run_rotation, host_default_config
    errs = {}
    for s in (50, 100):
        grid, *_ = rotation_case(s)
        o = oracle_mod.OracleSim(grid, host_default_config())
        phi = run_rotation(o, s, 157)
        errs[s] = band_l1(phi, rotation_truth(s, 157), ROT_LENGTH / s)
        o.close()
    assert errs[50] < 0.1 * (ROT_LENGTH / 50)
    assert errs[100] < 0.04 * (ROT_LENGTH / 100)
    assert errs[100] < errs[50] / 4


def half_space_cube_volume(n, d0) -> float:
    """Exact volume of {x in [0,1]^3 : n.(x - 1/2) + d0 < 0} (inclusion-exclusion over the
    cube's corners of the simplex volumes max(b - a.v, 0)^3 / (6 a1 a2 a3), a > 0)."""
    import itertools
    a = np.array(n, dtype=float)
    b = -d0 + 0.5 * a.sum()          # a.x < b
    for k in range(3):                # reflect axes so every a_k > 0
        if a[k] < 0:
            b -= a[k]
            a[k] = -a[k]
    tot = 0.0
    for v in itertools.product((0, 1), repeat=3):
        tot += (-1) ** sum(v) * max(b - float(np.dot(a, v)), 0.0) ** 3
    return tot / (6 * a[0] * a[1] * a[2])


def test_volume_diagnostic_known_answers(oracle_mod):
    """calculateVolume (LevelSetLiquid.cpp:1162-1190).  Cell pieces: empty and full
    cells, a planar cut (exact for any plane: the surface is then the plane itself),
    the marching-squares saddle rule; whole fields: a ball and a disk converge to
    4/3 pi r^3 and pi r^2."""
    import itertools
    O = oracle_mod
    assert O.mc_tables_ok()
    assert O.mc_cube_volume([1.0] * 8) == 0.0 and O.mc_cube_volume([-1.0] * 8) == 1.0
    corners = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    rng = np.random.default_rng(4)
    for _ in range(500):
        n = rng.normal(size=3)
        d0 = rng.uniform(-0.6, 0.6)
        vals = [float(np.dot(n, np.array(c) - 0.5) + d0) for c in corners]
        assert abs(O.mc_cube_volume(vals) - half_space_cube_volume(n, d0)) < 1e-12
    # marching squares: a planar cut is a polygon; a saddle joins through the centre iff the mean <= 0
    assert abs(O.ms_square_area([-1.0, 1.0, -1.0, 1.0]) - 0.5) < 1e-15
    assert abs(O.ms_square_area([-1.0, 1.0, 1.0, -0.5]) - (0.5 * 0.5 * 0.5 + 0.5 * (0.5 / 1.5) * (0.5 / 1.5))) < 1e-15
    joined = O.ms_square_area([-1.0, 0.5, 0.5, -1.0])
    assert joined > 0.5
    # balls and disks.  The reference passes each cube to the evaluator in x-fastest
    # order, which swaps two pairs of corners: its volumes converge at first order.
    # In the evaluator's own order they converge at second order.
    ref_err, own_err, disk_err = [], [], []
    for s in (32, 64, 128):
        dx = 1.0 / s
        g = (np.arange(s) + 0.5) * dx
        X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
        phi = np.ascontiguousarray((np.sqrt((X - .5) ** 2 + (Y - .5) ** 2 + (Z - .5) ** 2) - 0.3).transpose(2, 1, 0))
        exact = 4 / 3 * np.pi * 0.3 ** 3
        ref_err.append(abs(O.field_volume(phi, dx) / exact - 1))
        own_err.append(abs(O.field_volume(phi, dx, evaluator_order=True) / exact - 1))
        Y2, X2 = np.meshgrid(g, g, indexing="ij")
        phi2 = np.sqrt((X2 - .5) ** 2 + (Y2 - .5) ** 2) - 0.3
        disk_err.append(abs(O.field_volume(np.ascontiguousarray(phi2), dx) / (np.pi * 0.3 ** 2) - 1))
    assert ref_err[0] < 2.5e-2 and ref_err[2] < 5e-3
    assert ref_err[0] / ref_err[1] > 1.8 and ref_err[1] / ref_err[2] > 1.8      # first order
    assert own_err[0] / own_err[1] > 3.2 and own_err[1] / own_err[2] > 3.2      # second order
    assert disk_err[0] < 1e-2 and disk_err[1] / disk_err[2] > 3.0


@pytest.mark.parametrize("dim,n", [(3, 24), (2, 48)])
def test_newton_restart_redistances_a_sphere(oracle_mod, dim, n):
    """Newton configuration restart (HybridNewton without FMM, LevelSetLiquid.cpp:1290-1308)
    on φ = (|x-c|² - r0²)/(2 r0), whose zero set is a sphere but which is not a distance
    function: the reference level set it produces is the signed distance (closest points
    by Newton next to the interface, eikonal advection beyond), ψ0 has unit length, and
    ξ = x, Π = I afterwards."""
    from helpers import newton_sphere_case
    grid, phi, grad, sdf = newton_sphere_case(n, dim)
    o = oracle_mod.OracleSim(grid, host_default_config(restart_newton=1))
    o.upload(capi.FIELD_LEVEL_SET, phi.ravel())
    o.upload(capi.FIELD_ORI_LEVEL_SET, phi.ravel())
    o.upload(capi.FIELD_LEVEL_SET_GRAD, grad.ravel())
    o.stage("restart")
    dx = 1.0 / n
    ref = o.download(capi.FIELD_REF_LEVEL_SET)
    s = sdf.ravel()
    near, band = np.abs(s) <= 1.5 * dx, np.abs(s) <= 6 * dx
    assert np.mean(np.abs(ref - s)[near]) < 1e-5 * dx
    assert np.max(np.abs(ref - s)[band]) < 1e-3 * dx
    assert np.max(np.abs(phi.ravel() - s)[band]) > 0.1 * dx  # the input was far from a distance function
    norms = np.linalg.norm(o.download(capi.FIELD_REF_LEVEL_SET_GRAD).reshape(-1, dim), axis=1)
    assert np.max(np.abs(norms - 1)) < 1e-12
    assert np.array_equal(o.download(capi.FIELD_LEVEL_SET_GRAD), o.download(capi.FIELD_REF_LEVEL_SET_GRAD))
    assert np.array_equal(o.download(capi.FIELD_ORI_LEVEL_SET), ref)
    pi = o.download(capi.FIELD_REF_MAP_GRAD).reshape(-1, dim * dim)
    assert np.array_equal(pi, np.tile(np.eye(dim).ravel(), (len(pi), 1)))


def test_newton_initialize_takes_psi0_from_the_level_set(oracle_mod):
    """initialize in the Newton configuration: ∇φ by the 4th-order difference of the
    level set before reinitialisation becomes ψ0 (LevelSetLiquid.cpp:546-558); the field
    is absent without it."""
    sc = scenes.drop(16, seed=4)
    o = oracle_mod.OracleSim(sc.grid, host_default_config(restart_newton=1))
    load_scene(o, sc)
    o.initialize()
    lg = o.download(capi.FIELD_LEVEL_SET_GRAD).reshape(-1, 3)
    assert np.array_equal(lg.ravel(), o.download(capi.FIELD_REF_LEVEL_SET_GRAD))
    # interior cells: (f(-2) - 8 f(-1) + 8 f(1) - f(2)) / 12dx along x, of the level set
    # after enforceBoundaryLevelSet (φ >= -cellDist)
    phi0 = np.maximum(sc.phi, -o.download(capi.FIELD_CELL_DIST).reshape(sc.phi.shape))
    dx = sc.grid.spacing
    gx = (phi0[:, :, 0:-4] - 8 * phi0[:, :, 1:-3] + 8 * phi0[:, :, 3:-1] - phi0[:, :, 4:]) / 12 / dx
    assert np.max(np.abs(lg[:, 0].reshape(phi0.shape)[:, :, 2:-2] - gx)) < 1e-9
    plain = oracle_mod.OracleSim(sc.grid, host_default_config())
    with pytest.raises(ValueError):
        plain.download(capi.FIELD_LEVEL_SET_GRAD)


def test_newton_restart_is_ill_conditioned_on_a_simulated_scene(oracle_mod):
    """The reference's Newton restart on a simulated level set is sensitive to ulp-level
    input changes (closest-point iterations that stop after 20 capped steps, eikonal traces
    along a vanishing gradient), while on a smooth one it is not.  This is why GPU parity
    in that configuration is measured against the oracle's own perturbation spread."""
    from helpers import STATE_FIELDS, perturbed
    sc = scenes.drop(20, seed=3)
    o = oracle_mod.OracleSim(sc.grid, host_default_config(restart_newton=1))
    load_scene(o, sc)
    o.initialize()
    o.stage("restart")
    for dt in scenes.frame_time_steps(o.max_speed, 3, 25, 1.0, sc.grid.spacing):
        o.advance(dt)
    fields = STATE_FIELDS + [capi.FIELD_LEVEL_SET_GRAD]
    snap = {f: o.download(f) for f in fields}

    def run(size):
        s = oracle_mod.OracleSim(sc.grid, host_default_config(restart_newton=1))
        for f, v in snap.items():
            moved = f in (capi.FIELD_LEVEL_SET, capi.FIELD_ORI_LEVEL_SET, capi.FIELD_LEVEL_SET_GRAD)
            s.upload(f, perturbed(v, size, f) if moved else v)
        s.stage("restart")
        return s.download(capi.FIELD_REF_LEVEL_SET)

    dx = sc.grid.spacing
    assert np.max(np.abs(run(1e-15) - run(0.0))) > 1e-3 * dx


def upwind_fixed_point(seed_val, fixed, spacing, band):
    """Independent numpy restatement of the fast-marching equations: every non-seed cell holds
    min(band, Q(per-axis smaller neighbour)) with Q the upwind quadratic of
    FastMarching.cpp:112-128; solved by Jacobi relaxation from above."""
    u = np.where(fixed, seed_val, band).astype(np.float64)
    dim = u.ndim
    dx = spacing

    def axis_min(v, ax):
        lo = np.full_like(v, np.inf)
        hi = np.full_like(v, np.inf)
        sl = [slice(None)] * dim
        sr = [slice(None)] * dim
        sl[ax], sr[ax] = slice(1, None), slice(None, -1)
        lo[tuple(sl)] = v[tuple(sr)]
        hi[tuple(sr)] = v[tuple(sl)]
        return np.where(hi < lo, hi, lo)

    def q2(p0, p1):
        a, b = np.minimum(p0, p1), np.maximum(p0, p1)
        with np.errstate(invalid="ignore"):
            two = ((a + b) + np.sqrt(2 * dx * dx - (a - b) * (a - b))) * .5
        return np.where(np.isinf(b) | (b - a > dx), a + dx, two)

    def q3(p0, p1, p2):
        s0 = np.where(p0 > p1, p1, p0); s1 = np.where(p0 > p1, p0, p1)
        t1 = np.where(s1 > p2, p2, s1); t2 = np.where(s1 > p2, s1, p2)
        drop = np.isinf(t2) | ((t2 - s0) * (t2 - s0) + (t2 - t1) * (t2 - t1) > dx * dx)
        s = s0 + t1 + t2
        with np.errstate(invalid="ignore"):
            three = (s + np.sqrt(s * s - 3 * (s0 * s0 + t1 * t1 + t2 * t2 - dx * dx))) / 3
        return np.where(drop, q2(s0, t1), three)

    # numpy axis 0 is z (3D) or y (2D): the quadratic is symmetric in its per-axis arguments
    # except for the operation order, so pass them in x, y, z order as the reference does
    for _ in range(10000):
        m = [axis_min(u, dim - 1 - a) for a in range(dim)]
        cand = q2(m[0], m[1]) if dim == 2 else q3(m[0], m[1], m[2])
        new = np.where(fixed | ~(cand < u), u, cand)
        if np.array_equal(new, u):
            return u
        u = new
    raise AssertionError("no convergence")


@pytest.mark.parametrize("dim,n", [(2, 64), (3, 24)])
def test_fast_marching_equals_the_upwind_fixed_point(oracle_mod, dim, n):
    """The heap-ordered fast marching of the reference (restated in the oracle) and the fixed
    point of its upwind equations agree, both from sign-change seeds and from marked seeds.
    This is what lets the GPU solve the same equations by parallel relaxation instead of a
    serial heap."""
    from helpers import newton_sphere_case
    grid, phi, _, _ = newton_sphere_case(n, dim)
    dx = 1.0 / n
    phi = phi + 0.05 * dx * np.sin(np.arange(phi.size) * 0.7).reshape(phi.shape)  # break symmetries
    band = 15 * dx
    out = oracle_mod.fast_marching(phi, dx, 15)
    # seeds as FastMarching.cpp:14-30 computes them
    t = [np.full(phi.shape, np.inf) for _ in range(dim)]
    for a in range(dim):
        ax = dim - 1 - a
        for s in (-1, 1):
            nb = np.roll(phi, -s, axis=ax)
            valid = np.ones(phi.shape, bool)
            idx = [slice(None)] * dim
            idx[ax] = -1 if s == 1 else 0
            valid[tuple(idx)] = False
            with np.errstate(divide="ignore", invalid="ignore"):
                cand = phi / (phi - nb) * dx
            use = valid & (phi * nb <= 0) & (cand < t[a])
            t[a] = np.where(use, cand, t[a])
    fixed = np.zeros(phi.shape, bool)
    for a in range(dim):
        fixed |= np.isfinite(t[a])
    with np.errstate(divide="ignore"):
        seed = 1 / np.sqrt(sum((1 / ta) ** 2 for ta in t))
    ref = upwind_fixed_point(seed, fixed, dx, band)
    expect = np.where(phi <= 0, -1.0, 1.0) * ref
    assert np.max(np.abs(out - expect)) <= 1e-12 * dx
    assert np.max(np.abs(out)) <= band
    # marked seeds keep |φ| there
    mark = (np.abs(phi) < 1.5 * dx).astype(np.uint8)
    out2 = oracle_mod.fast_marching(phi, dx, 20, mark)
    ref2 = upwind_fixed_point(np.abs(phi), mark.astype(bool), dx, 20 * dx)
    assert np.max(np.abs(out2 - np.where(phi <= 0, -1.0, 1.0) * ref2)) <= 1e-12 * dx


def test_fast_marching_plane_is_exact(oracle_mod):
    """An axis-aligned plane: the crossing seeds are exact, so are the marched distances
    (p + dx per cell) up to the band width, which caps the rest."""
    n, dx = 40, 1.0 / 40
    x = (np.arange(n) + 0.5) * dx
    x0 = 0.3137
    phi = np.broadcast_to((x - x0)[None, None, :], (8, 8, n)).copy() * 3.0  # not a distance function
    out = oracle_mod.fast_marching(phi, dx, 15)
    exact = np.broadcast_to((x - x0)[None, None, :], (8, 8, n))
    inband = np.abs(exact) < 14.5 * dx
    assert np.max(np.abs(out - exact)[inband]) < 1e-12
    assert np.all(np.abs(out[~inband]) <= 15 * dx + 1e-15)


def test_fast_marching_configuration_steps(oracle_mod):
    """The fast-marching configuration runs initialize and steps (WENO5 replaced by fast
    marching over 15 cells); the level set is a distance function near the interface."""
    sc = scenes.dam_break(3, 20)
    o = oracle_mod.OracleSim(sc.grid, host_default_config(fast_marching=1))
    load_scene(o, sc)
    assert o.initialize() == capi.OK
    o.stage("restart")
    for dt in scenes.frame_time_steps(o.max_speed, 3, 25, 1.0, sc.grid.spacing):
        assert o.advance(dt)["status"] == capi.OK
    phi = o.download(capi.FIELD_LEVEL_SET).reshape(sc.phi.shape)
    assert np.all(np.isfinite(phi))
    assert np.max(np.abs(phi)) <= 15 * sc.grid.spacing * (1 + 1e-12)
