"""The FP64 population-mesh kernels against the oracle restatement of PopulationMesh.jl (to rounding of exp / log), and
the whole MeshPopulationModel chain (features -> inner model -> back-map, its VJP and JVP) against the oracle chain."""
import os
import sys

import numpy as np
import pytest
import torch

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import population_mesh_oracle as pmo  # noqa: E402
from test_population_mesh_cpu import (_grads, _hold_bottom, _mesh_inside, atm_cols, chain, cols, inner_jvp,  # noqa: E402
                                      inner_pm, inner_vjp, mesh_test_atmosphere)

pytestmark = pytest.mark.gpu


def _close(a, b, rtol=1e-12):
    a, b = np.asarray(a), np.asarray(b)
    scale = np.maximum(np.abs(b), 1e-300)
    assert np.all(np.abs(a - b) <= rtol * scale + 1e-14 * np.abs(b).max()), np.max(np.abs(a - b) / scale)


@pytest.mark.parametrize("corona", [False, True])
@pytest.mark.parametrize("meshkind", ["inside", "wide"])
def test_kernels_match_oracle(corona, meshkind):
    from ffnoml_gb300.population_mesh import MeshMaps, PopulationMeshConfig, population_mesh
    f, z = mesh_test_atmosphere(nx=5, ny=4, nz=45)
    mesh = _mesh_inside() if meshkind == "inside" else population_mesh(PopulationMeshConfig(
        bottom_m=-1e6, top_m=3e6, uniform_top_m=2e6, stretch=1.05, max_spacing_m=5e4))
    a, zc = atm_cols(f), cols(z)
    maps = MeshMaps(zc, mesh, corona=corona)
    at = torch.as_tensor(a, device="cuda")
    fm, kind = maps.features(at)
    fm0, kind0 = pmo.features(a, zc, mesh, corona=corona)
    assert np.array_equal(kind.cpu().numpy(), kind0)
    if meshkind == "wide":
        assert (kind0 == pmo.DEEP).any() and ((kind0 == pmo.CORONA).any() == corona)
    _close(fm.cpu().numpy(), fm0)
    rng = np.random.default_rng(1)
    fb = rng.normal(size=fm0.shape)
    fbar, zbar = maps.features_vjp(at, fm, torch.as_tensor(fb, device="cuda"))
    fbar0, zbar0 = pmo.features_vjp(a, zc, mesh, fm0, fb, corona=corona)
    _close(fbar.cpu().numpy(), fbar0, 1e-10)
    _close(zbar.cpu().numpy(), zbar0, 1e-10)
    fd = rng.normal(size=(zc.shape[0], zc.shape[1], 6))
    fmd = maps.features_jvp(at, fm, torch.as_tensor(fd, device="cuda"))
    _close(fmd.cpu().numpy(), pmo.features_jvp(a, zc, mesh, fm0, fd, corona=corona), 1e-10)
    pm = np.exp(rng.normal(size=(3, zc.shape[0], len(mesh))))
    pmt = torch.as_tensor(pm, device="cuda")
    _close(maps.backmap(pmt).cpu().numpy(), pmo.backmap(pm, mesh, zc))
    pb = rng.normal(size=(3, zc.shape[0], zc.shape[1]))
    pm_bar, zb = maps.backmap_vjp(pmt, torch.as_tensor(pb, device="cuda"))
    pm_bar0, zb0 = pmo.backmap_vjp(pm, mesh, zc, pb)
    _close(pm_bar.cpu().numpy(), pm_bar0, 1e-10)
    _close(zb.cpu().numpy(), zb0, 1e-10)
    pmd = rng.normal(size=pm.shape)
    _close(maps.backmap_jvp(pmt, torch.as_tensor(pmd, device="cuda")).cpu().numpy(),
           pmo.backmap_jvp(pm, mesh, zc, pmd), 1e-10)


class _Toy:
    """The toy inner model of the CPU tests in the module's array conventions."""

    def __init__(self, mesh):
        self.mesh = mesh

    def _c(self, fm):
        from ffnoml_gb300.population_mesh import columns
        return np.stack([columns(fm[c]) for c in range(6)]).transpose(1, 2, 0)

    def _u(self, x, nx, ny):
        from ffnoml_gb300.population_mesh import uncolumns
        return np.moveaxis(uncolumns(x, nx, ny), 0, -1)

    def predict(self, fm, zm, dx, dy):
        return self._u(inner_pm(self._c(fm), self.mesh), fm.shape[2], fm.shape[3])

    def vjp(self, fm, zm, dx, dy, pm_bar):
        from ffnoml_gb300.population_mesh import columns, uncolumns
        pb = np.stack([columns(pm_bar[..., l]) for l in range(pm_bar.shape[-1])])
        g = inner_vjp(self._c(fm), self.mesh, pb)
        return uncolumns(g.transpose(2, 0, 1), fm.shape[2], fm.shape[3]), None

    def jvp(self, fm, zm, dx, dy, fm_dot):
        return self._u(inner_jvp(self._c(fm), self.mesh, self._c(fm_dot)), fm.shape[2], fm.shape[3])


class _HoldBottom:
    """A stand-in extension below the columns (bottom values held), exercising the extension hooks."""

    def fill(self, f, kind, atm, z, mesh):
        for col in range(f.shape[0]):
            deep = kind[col] == pmo.DEEP
            f[col, deep] = atm[:, col, -1]

    def vjp(self, fm_bar, kind, atm, z, mesh):
        a_bar = np.zeros((z.shape[0], z.shape[1], 6))
        for col in range(z.shape[0]):
            a_bar[col, -1] = fm_bar[col, kind[col] == pmo.DEEP].sum(0) * np.r_[atm[0, col, -1], np.ones(5)]
        return a_bar, np.zeros_like(z)

    def jvp(self, fd, kind, atm, z, mesh):
        out = np.zeros((z.shape[0], len(mesh), 6))
        for col in range(z.shape[0]):
            out[col, kind[col] == pmo.DEEP] = fd[col, -1]
        return out


def test_mesh_model_chain_matches_oracle():
    from ffnoml_gb300.population_mesh import MeshPopulationModel, PopulationMeshConfig
    f, z = mesh_test_atmosphere()
    mesh = _mesh_inside()
    model = MeshPopulationModel(_Toy(mesh), PopulationMeshConfig(heights_m=tuple(mesh)))
    nz, nx, ny = z.shape
    out = model.predict(f, z, 48e3, 48e3)
    ref = chain(f, z, mesh)
    from ffnoml_gb300.population_mesh import uncolumns
    _close(out, np.moveaxis(uncolumns(ref, nx, ny), 0, -1), 1e-11)
    bar_c = np.cos(np.arange(1, 2 * nz * nx * ny + 1)).reshape(2, nx * ny, nz)
    bar = np.moveaxis(uncolumns(bar_c, nx, ny), 0, -1)
    fbar, zbar = model.vjp(f, z, 48e3, 48e3, bar)
    fbar0, zbar0 = _grads(f, z, mesh, bar_c)
    _close(fbar, fbar0, 1e-9)
    _close(zbar, zbar0, 1e-9)
    tang = np.random.default_rng(2).normal(size=f.shape) * np.r_[1.0, 1e2, 1e2, 1e2, 0.01, 0.01][:, None, None, None]
    pd = model.jvp(f, z, 48e3, 48e3, tang)
    h = 1e-5
    fd = (model.predict(f + h * tang, z, 48e3, 48e3) - model.predict(f - h * tang, z, 48e3, 48e3)) / (2 * h)
    assert np.abs(pd - fd).max() < 1e-6 * np.abs(fd).max()


def test_points_below_columns_need_an_extension():
    from ffnoml_gb300.population_mesh import MeshPopulationModel, PopulationMeshConfig
    f, z = mesh_test_atmosphere()
    cfg = PopulationMeshConfig(bottom_m=-1e6, top_m=3e6, uniform_top_m=2e6, stretch=1.05, max_spacing_m=5e4)
    with pytest.raises(ValueError):
        MeshPopulationModel(_Toy(None), cfg).predict(f, z, 48e3, 48e3)
    from ffnoml_gb300.population_mesh import population_mesh
    mesh = population_mesh(cfg)
    model = MeshPopulationModel(_Toy(mesh), cfg, extension=_HoldBottom())
    nz, nx, ny = z.shape
    bar = np.random.default_rng(3).normal(size=(nz, nx, ny, 2))
    fbar, zbar = model.vjp(f, z, 48e3, 48e3, bar)
    tang = np.random.default_rng(4).normal(size=f.shape) * np.r_[1.0, 1e2, 1e2, 1e2, 0.01, 0.01][:, None, None, None]
    h = 1e-5
    obj = lambda g: np.sum(bar * model.predict(g, z, 48e3, 48e3))
    fd = (obj(f + h * tang) - obj(f - h * tang)) / (2 * h)
    assert abs(np.sum(fbar * tang) - fd) < 1e-6 * abs(fd)
    pd = model.jvp(f, z, 48e3, 48e3, tang)
    assert abs(np.sum(bar * pd) - fd) < 1e-6 * abs(fd)


# ------------------------------------------------------------------------------------------------ inclined views
@pytest.mark.parametrize("shape,s", [((6, 7, 4), -1), ((6, 7, 4), 1), ((5, 1, 9), -1), ((4, 12, 1), 1)])
def test_shear_kernel_matches_oracle(shape, s):
    from ffnoml_gb300.population_mesh import ShearPlan
    g = np.random.default_rng(7)
    nz = shape[0]
    z = np.linspace(2.2e6, -1.3e6, nz)
    t = pmo.slant(0.45, 200.0)
    A = g.normal(size=shape)
    plan = ShearPlan(z, 48e3, 30e3, t, s, "cuda")
    ref = pmo.shear_plan(z, 48e3, 30e3, t, s)
    assert np.array_equal(plan.i0.cpu().numpy(), ref[0]) and np.array_equal(plan.j0.cpu().numpy(), ref[1])
    At = torch.as_tensor(A, device="cuda")
    _close(plan.apply(At).cpu().numpy(), pmo.shear_levels(A, ref), 1e-14)
    _close(plan.apply(At, transpose=True).cpu().numpy(), pmo.shear_levels_transpose(A, ref), 1e-14)


def test_adaptive_mesh_matches_oracle():
    """The GPU adaptive mesh (probe features and the per-interval spacing on the device, the walk on the host) against
    the oracle's restatement of adaptive_population_mesh."""
    from ffnoml_gb300.population_mesh import PopulationMeshConfig, adaptive_population_mesh
    f, z = mesh_test_atmosphere(nx=6, ny=5)
    a, zc = atm_cols(f), cols(z)
    cfg = PopulationMeshConfig(adaptive=True, extend=False, lnT_step=0.02)
    ref = pmo.adaptive_mesh(a, zc, cfg.top_m, cfg.bottom_m, cfg.min_spacing_m, cfg.max_spacing_m, cfg.growth,
                            cfg.lnT_step, cfg.log_ne_step, cfg.log_rho_step, cfg.velocity_step_m_s, extend=False,
                            fill=_hold_bottom(a))

    class Hold:
        def fill(self, fh, kind, atm, zz, mesh):
            _hold_bottom(atm)(fh, kind)

    got = adaptive_population_mesh(cfg, a, zc, extension=Hold(), chunk_bytes=1 << 16)    # several column chunks
    assert got.shape == ref.shape
    # the device's log / exp differ from numpy's in the last bits, and each mesh height is the sum of the spacings
    # above it, so the heights agree to a few hundred ulps, not to one
    _close(got, ref, 1e-8)


def test_inclined_view_chain():
    """MeshPopulationModel on an inclined view: the ray mesh features sheared to Cartesian columns for the inner
    model and its populations sheared back (PopulationMesh.jl:296-334), against the same chain composed from the
    oracle; its VJP and JVP against central differences."""
    from ffnoml_gb300.population_mesh import (MeshPopulationModel, PopulationMeshConfig, ViewGeometry, population_mesh,
                                              uncolumns)
    f, z = mesh_test_atmosphere(nx=6, ny=5)
    # the shallowest column bottom of this 6 x 5 atmosphere is near -2.98e5 m (x = 1, y = 5): a mesh inside all columns
    mesh = population_mesh(PopulationMeshConfig(bottom_m=-2.487654e5, top_m=2.5e6, spacing_m=2e4, uniform_top_m=1.5e6,
                                                stretch=1.05, max_spacing_m=5e4))
    assert mesh.min() > cols(z)[:, -1].max()                               # columns run top to bottom
    view = ViewGeometry(mu=0.5, azimuth_deg=30.0)
    model = MeshPopulationModel(_Toy(mesh), PopulationMeshConfig(heights_m=tuple(mesh)), view=view)
    nz, nx, ny = z.shape
    dx, dy = 48e3, 40e3
    out = model.predict(f, z, dx, dy)
    # the oracle chain: ray features on the mesh -> Cartesian (ln T and the others sheared, s = -1) -> toy inner
    # model -> ray populations (ln n sheared, s = +1) -> back-map
    fm, _ = pmo.features(atm_cols(f), cols(z), mesh)                       # [col][m][6]
    grid = lambda c: uncolumns(c[None], nx, ny)[0]                          # [col][m] -> (m, nx, ny)
    t = pmo.slant(0.5, 30.0)
    sm, sp = pmo.shear_plan(mesh, dx, dy, t, -1), pmo.shear_plan(mesh, dx, dy, t, 1)
    fc = [np.exp(pmo.shear_levels(np.log(grid(fm[:, :, 0])), sm))] + \
         [pmo.shear_levels(grid(fm[:, :, c]), sm) for c in range(1, 6)]
    fc_cols = np.stack([cols(v) for v in fc], axis=-1)                      # [col][m][6]
    pc = inner_pm(fc_cols, mesh)                                            # [L][col][m]
    pr = np.stack([cols(np.exp(pmo.shear_levels(np.log(grid(pc[l])), sp))) for l in range(pc.shape[0])])
    ref = pmo.backmap(pr, mesh, cols(z))
    _close(out, np.moveaxis(uncolumns(ref, nx, ny), 0, -1), 1e-10)
    bar = np.random.default_rng(8).normal(size=out.shape)
    fbar, zbar = model.vjp(f, z, dx, dy, bar)
    tang = np.random.default_rng(9).normal(size=f.shape) * np.r_[1.0, 1e2, 1e2, 1e2, 0.01, 0.01][:, None, None, None]
    h = 1e-5
    obj = lambda g: np.sum(bar * model.predict(g, z, dx, dy))
    fd = (obj(f + h * tang) - obj(f - h * tang)) / (2 * h)
    assert abs(np.sum(fbar * tang) - fd) < 1e-6 * abs(fd)
    pd = model.jvp(f, z, dx, dy, tang)
    assert abs(np.sum(bar * pd) - fd) < 1e-6 * abs(fd)
