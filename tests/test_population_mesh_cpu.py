"""The population-mesh oracle pinned on the reference's known answers (FFNOInversion.jl/test/population_mesh.jl):
the fixed mesh's shape, exact interpolation of variables linear in height, exact back-mapping of log-linear
populations, and the VJP / JVP of the whole mesh chain against central differences; plus the package's host logic."""
import math
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import population_mesh_oracle as pmo  # noqa: E402

from ffnoml_gb300 import population_mesh as pmesh  # noqa: E402


def mesh_test_atmosphere(nx=3, ny=2, nz=38):
    """The reference's mesh_test_atmosphere (population_mesh.jl:37-48) as service features (6, nz, nx, ny) and
    heights (nz, nx, ny): T, vx, vy, vz, log10 ne, log10 rho."""
    lt = np.linspace(-6.0, 1.4, nz)
    tau = 10.0 ** lt
    k = np.arange(1, nz + 1)[:, None, None]
    x = np.arange(1, nx + 1)[None, :, None]
    y = np.arange(1, ny + 1)[None, None, :]
    t = tau[:, None, None]
    T = (4300 + 1700 * t ** 0.25) * (1 + 0.02 * x - 0.03 * y)
    rho = 3e-4 * t ** 0.45 * (1 + 0.05 * y) * np.ones_like(T)
    ne = 1e19 * t ** 0.6 * (1 + 0.1 * x) * np.ones_like(T)
    z = -1.2e5 * np.log(t) * (1 + 0.03 * x) + 2e4 * y
    v = lambda s: s * np.sin(0.3 * k + x - y) * np.ones_like(T)
    f = np.stack([T, v(1e3), v(-7e2), v(2e3), np.log10(ne), np.log10(rho)])
    return f, z


def cols(a):
    return pmesh.columns(a)


def atm_cols(f):
    return np.stack([cols(f[c]) for c in range(6)])


# toy inner model with an exact VJP (population_mesh.jl:9-35): ln p_l = sum_c A[l,c] phi_c + B[l] z / 1e6
A = np.array([[0.8, 0.1, -0.2, 0.3, 1.1, 0.9], [-0.5, 0.2, 0.1, -0.4, 0.7, 1.3]])
B = np.array([0.4, -0.6])
SCALE = np.array([1 / 5000, 1e-4, 1e-4, 1e-4, 1 / 20, 1 / 10])


def inner_pm(fm, mesh):
    """fm [ncol][nm][6] -> pm [L][ncol][nm] (phi = the features times SCALE; log10 ne, log10 rho as the reference's
    log10(ne) / 20 and log10(rho) / 10)."""
    phi = fm * SCALE
    return np.exp(np.einsum("lc,ijc->lij", A, phi) + B[:, None, None] * mesh[None, None, :] / 1e6)


def inner_vjp(fm, mesh, pm_bar):
    pm = inner_pm(fm, mesh)
    g = pm_bar * pm
    return np.einsum("lij,lc->ijc", g, A) * SCALE


def inner_jvp(fm, mesh, fm_dot):
    pm = inner_pm(fm, mesh)
    return pm * np.einsum("lc,ijc->lij", A, fm_dot * SCALE)


def chain(f, z, mesh):
    fm, kind = pmo.features(atm_cols(f), cols(z), mesh)
    assert not (kind >= pmo.DEEP).any()
    return pmo.backmap(inner_pm(fm, mesh), mesh, cols(z))


def test_fixed_mesh_shape():
    """population_mesh.jl:40-44."""
    m = pmesh.population_mesh(pmesh.PopulationMeshConfig())
    assert np.all(np.diff(m) < 0) and m[0] == 1.4e7 and m[-1] == -1.0e6
    assert np.all(np.abs(np.diff(m[-201:]) + 2e4) < 1e-6)
    assert np.max(-np.diff(m)) <= 1e5 * 1.5 and 300 < len(m) < 500
    assert np.array_equal(m, pmo.population_mesh())
    with pytest.raises(ValueError):
        pmesh.PopulationMeshConfig(bottom_m=5e6)
    with pytest.raises(ValueError):
        pmesh.PopulationMeshConfig(heights_m=(0.0, 1e6))
    assert np.array_equal(pmesh.population_mesh(pmesh.PopulationMeshConfig(heights_m=(2e6, 1e6, 0.0, -5e5))),
                          [2e6, 1e6, 0.0, -5e5])


def test_interpolation_exact_for_linear_variables():
    """population_mesh.jl:56-70: inside a column, ln T, v, log10 ne, log10 rho linear in z are interpolated exactly."""
    f, z = mesh_test_atmosphere()
    zz = z / 1e6
    lin = f.copy()
    lin[0] = np.exp(8.6 - 0.2 * zz)
    lin[1] = 100 + 50 * zz
    lin[4] = 18 - zz
    lin[5] = -4 - 0.8 * zz
    mesh = pmesh.population_mesh(pmesh.PopulationMeshConfig(bottom_m=-1e6, top_m=3e6, spacing_m=2e4,
                                                              uniform_top_m=2e6, stretch=1.05, max_spacing_m=5e4))
    fm, kind = pmo.features(atm_cols(lin), cols(z), mesh)
    zc = cols(z)
    for c in range(zc.shape[0]):
        inside = (mesh >= zc[c, -1]) & (mesh <= zc[c, 0])
        mm = mesh[inside] / 1e6
        assert np.all(kind[c, inside] == pmo.INSIDE)
        assert np.allclose(np.log(fm[c, inside, 0]), 8.6 - 0.2 * mm, rtol=1e-12)
        assert np.allclose(fm[c, inside, 1], 100 + 50 * mm, rtol=1e-12)
        assert np.allclose(fm[c, inside, 4], 18 - mm, rtol=1e-12)
        assert np.allclose(fm[c, inside, 5], -4 - 0.8 * mm, rtol=1e-12)
        assert np.all(kind[c, mesh < zc[c, -1]] == pmo.DEEP)
        above = mesh > zc[c, 0]
        assert np.all(kind[c, above] == pmo.TOP) and np.all(fm[c, above, 1] == lin[1].transpose(2, 1, 0).reshape(-1,
                                                                                                         38)[c, 0])


def test_backmap_exact_for_log_linear_populations():
    """population_mesh.jl:83-87: populations exp(B z / 1e6) on the mesh come back exactly."""
    f, z = mesh_test_atmosphere()
    mesh = pmesh.population_mesh(pmesh.PopulationMeshConfig(bottom_m=-1e6, top_m=3e6, uniform_top_m=2e6,
                                                              stretch=1.05, max_spacing_m=5e4))
    zc = cols(z)
    pm = np.exp(B[:, None, None] * np.broadcast_to(mesh, (2, zc.shape[0], len(mesh))) / 1e6)
    out = pmo.backmap(pm, mesh, zc)
    assert np.allclose(out, np.exp(B[:, None, None] * zc[None] / 1e6), rtol=1e-12)


def _mesh_inside():
    # between every column's bottom (about -0.4 Mm) and above every top (about 1.9 Mm): held top values, no deep points;
    # offset so that no mesh height equals a column height (the maps have kinks there, where central differences
    # average two one-sided slopes)
    return pmesh.population_mesh(pmesh.PopulationMeshConfig(bottom_m=-2.987654e5, top_m=2.5e6, spacing_m=2e4,
                                                              uniform_top_m=1.5e6, stretch=1.05, max_spacing_m=5e4))


def _grads(f, z, mesh, bar):
    """feature_bar (6, nz, nx, ny) and z_bar (nz, nx, ny) of sum(bar * populations) through the oracle chain."""
    nz, nx, ny = z.shape
    a, zc = atm_cols(f), cols(z)
    fm, _ = pmo.features(a, zc, mesh)
    pm = inner_pm(fm, mesh)
    pm_bar, zb1 = pmo.backmap_vjp(pm, mesh, zc, bar)
    fm_bar = inner_vjp(fm, mesh, pm_bar)
    fbar, zb2 = pmo.features_vjp(a, zc, mesh, fm, fm_bar)
    return pmesh.uncolumns(fbar.transpose(2, 0, 1), nx, ny), pmesh.uncolumns(zb1 + zb2, nx, ny)


def test_vjp_and_jvp_against_central_differences():
    """population_mesh.jl:89-115: the VJP against central differences in T, velocities, ne, rho and heights (inside
    and above the columns; the deep extension needs the EOS table)."""
    f, z = mesh_test_atmosphere()
    mesh = _mesh_inside()
    nz, nx, ny = z.shape
    n = nz * nx * ny
    i = np.arange(1, n + 1)
    bar = np.cos(np.arange(1, 2 * n + 1)).reshape(2, nx * ny, nz)
    fbar, zbar = _grads(f, z, mesh, bar)
    dT = (0.01 * np.sin(i)).reshape(nz, nx, ny)
    dv = np.cos(2.0 * i).reshape(nz, nx, ny)
    dL = (0.02 * np.cos(i)).reshape(nz, nx, ny)
    dR = (0.03 * np.sin(3.0 * i)).reshape(nz, nx, ny)
    dz = (5.0 * np.sin(0.7 * i)).reshape(nz, nx, ny)

    def moved(h):
        g = f.copy()
        g[0] = f[0] * (1 + h * dT)
        g[1] = f[1] + h * 1e2 * dv
        g[3] = f[3] - h * 3e2 * dv
        g[4] = f[4] + h * dL
        g[5] = f[5] + h * dR
        return g, z + h * dz

    obj = lambda fz: float(np.sum(bar * chain(fz[0], fz[1], mesh)))
    h = 1e-4
    fd = (obj(moved(h)) - obj(moved(-h))) / (2 * h)
    pred = (np.sum(fbar[0] * f[0] * dT) + np.sum(fbar[1] * 1e2 * dv) - np.sum(fbar[3] * 3e2 * dv) +
            np.sum(fbar[4] * dL) + np.sum(fbar[5] * dR) + np.sum(zbar * dz))
    assert math.isclose(pred, fd, rel_tol=1e-5)
    assert np.any(zbar != 0) and np.any(fbar[5, 0] != 0)
    # JVP at fixed heights along the same feature direction
    a, zc = atm_cols(f), cols(z)
    fm, _ = pmo.features(a, zc, mesh)
    tang = np.zeros_like(f)
    tang[0], tang[1], tang[3], tang[4], tang[5] = f[0] * dT, 1e2 * dv, -3e2 * dv, dL, dR
    fd_c = np.stack([cols(tang[c]) for c in range(6)]).transpose(1, 2, 0)
    pm = inner_pm(fm, mesh)
    pm_dot = inner_jvp(fm, mesh, pmo.features_jvp(a, zc, mesh, fm, fd_c))
    jv = float(np.sum(bar * pmo.backmap_jvp(pm, mesh, zc, pm_dot)))
    fdj = (obj((f + h * tang, z)) - obj((f - h * tang, z))) / (2 * h)
    assert math.isclose(jv, fdj, rel_tol=1e-5)


def test_layout_round_trip():
    rng = np.random.default_rng(0)
    a = rng.normal(size=(5, 3, 4))
    c = pmesh.columns(a)
    assert c.shape == (12, 5) and c[1 + 3 * 2, 4] == a[4, 1, 2]
    assert np.array_equal(pmesh.uncolumns(c, 3, 4), a)
    b = rng.normal(size=(2, 12, 5))
    assert np.array_equal(pmesh.uncolumns(b, 3, 4)[1, 4, 1, 2], b[1, 1 + 3 * 2, 4])


# ------------------------------------------------------------------------------------------------ inclined views
def test_shear_transpose_is_its_adjoint_and_zero_slant_is_the_identity():
    """The oracle's shear (ViewAngle.jl:132-145) and its scatter transpose (:147-162): <S A, B> = <A, S^T B> for both
    directions of an inclined view, and a vertical view reads every level in place."""
    g = np.random.default_rng(5)
    z = np.linspace(2.2e6, -1.3e6, 6)
    A, B = g.normal(size=(6, 7, 4)), g.normal(size=(6, 7, 4))
    t = pmo.slant(0.55, 35.0)
    for s in (-1, 1):
        plan = pmo.shear_plan(z, 48e3, 30e3, t, s)
        assert (plan[0] < 0).any() or (plan[1] < 0).any() or s == 1
        lhs = np.sum(pmo.shear_levels(A, plan) * B)
        rhs = np.sum(A * pmo.shear_levels_transpose(B, plan))
        assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
    ident = pmo.shear_plan(z, 48e3, 30e3, pmo.slant(1.0, 35.0), 1)
    assert np.array_equal(pmo.shear_levels(A, ident), A)


def _hold_bottom(atm):
    """The stand-in hydrostatic extension: points below a column take its bottom values."""
    def fill(f, kind):
        for col in range(f.shape[0]):
            f[col, kind[col] == pmo.DEEP] = atm[:, col, -1]
    return fill


def test_adaptive_mesh_oracle_properties():
    """adaptive_population_mesh (PopulationMesh.jl:213-262): top first from the highest top to the lowest bottom
    (extend = false), every step within [min_spacing_m, max_spacing_m] (the last one may be shorter), neighbouring
    steps within the growth factor's reach, and finer where the features change faster."""
    f, z = mesh_test_atmosphere(nx=4, ny=3)
    a, zc = atm_cols(f), cols(z)
    kw = dict(min_spacing_m=1e4, max_spacing_m=1e5, growth=1.2, log_ne_step=0.1, log_rho_step=0.1,
              velocity_step_m_s=1e3, extend=False, fill=_hold_bottom(a))
    m = pmo.adaptive_mesh(a, zc, 1.4e7, -1e6, lnT_step=0.05, **kw)
    d = -np.diff(m)
    assert m[0] == zc[:, 0].max() and m[-1] == zc[:, -1].min() and (d > 0).all()
    assert d[:-1].min() >= 1e4 * (1 - 1e-12) and d.max() <= 1e5 * (1 + 1e-12)
    fine = pmo.adaptive_mesh(a, zc, 1.4e7, -1e6, lnT_step=0.01, **kw)
    assert len(fine) > len(m)
