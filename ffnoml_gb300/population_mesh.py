"""Population-mesh maps on the GPU (FFNOInversion.jl/src/PopulationMesh.jl): the step before and after the FFNO when
an inversion's atmosphere is on log-tau columns. Each column is interpolated onto one shared height mesh (log T,
log ne, log rho log-linear in height, velocities linear; above its top the top values held), the FFNO predicts the
mesh populations, and those are interpolated back to every column point (log-linear in height). The VJP is the
transpose of both maps and the JVP their tangent map, with the FFNO's own VJP / JVP in between.

The interpolation, back-map and their transposes / tangents run as FP64 kernels (ffno_mesh_*; one thread per
(column, point) pair, or per column for the scatters, in the reference's loop order). Mesh points below a column's
bottom (and above its top when a corona temperature is set) follow hydrostatic extensions on the HSEMHS equation of
state (PopulationMesh.jl:122-180); the kernels mark them (kind 2 / 3) and an `extension` object supplied by the
caller fills their features and adds their share of the VJP / JVP. Inclined views (ViewGeometry: the features of the
footprint rays are sheared to Cartesian mesh columns before the FFNO and its populations back, level by level, a
periodic bilinear shear, PopulationMesh.jl:288-326 and ViewAngle.jl:93-162) run the shear on the GPU
(ffno_shear_levels). The adaptive mesh (PopulationMeshConfig(adaptive=True), :213-285) is rebuilt for every
atmosphere from the columns' features on probe heights (ffno_mesh_features and ffno_mesh_refine on the GPU, the
grading and the walk down the heights on the host).

Array conventions: atmosphere variables are numpy arrays shaped (nz, nx, ny) as in the reference (top first along
nz); features (6, nz, nx, ny) = T [K], vx, vy, vz [m/s], log10 ne, log10 rho; populations (nz, nx, ny, L).
"""
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _native as nat
from .executor import _stream

INSIDE, TOP, DEEP, CORONA = 0, 1, 2, 3


@dataclass(frozen=True)
class PopulationMeshConfig:
    """The reference's PopulationMeshConfig (PopulationMesh.jl:30-88) for a fixed mesh, with its checks."""
    bottom_m: float = -1.0e6
    top_m: float = 1.4e7
    spacing_m: float = 2.0e4
    uniform_top_m: float = 4.5e6
    stretch: float = 1.01
    max_spacing_m: float = 1.0e5
    nabla: float = 0.13
    corona_temperature_k: float = 0.0
    corona_transition_m: float = 2.4e5
    heights_m: tuple = field(default_factory=tuple)
    adaptive: bool = False
    min_spacing_m: float = 1.0e4
    growth: float = 1.2
    lnT_step: float = 0.05
    log_ne_step: float = 0.1
    log_rho_step: float = 0.1
    velocity_step_m_s: float = 1.0e3
    extend: bool = True

    def __post_init__(self):
        if not self.bottom_m < self.uniform_top_m <= self.top_m:
            raise ValueError("population mesh needs bottom_m < uniform_top_m <= top_m")
        if not 0 < self.spacing_m <= self.max_spacing_m:
            raise ValueError("population mesh needs 0 < spacing_m <= max_spacing_m")
        if self.stretch < 1:
            raise ValueError("population mesh stretch must be >= 1")
        if not 0 < self.nabla < 1:
            raise ValueError("population mesh nabla must lie in (0, 1)")
        if self.corona_temperature_k < 0:
            raise ValueError("population mesh corona_temperature_k must not be negative")
        if self.corona_transition_m <= 0:
            raise ValueError("population mesh corona_transition_m must be positive")
        h = tuple(float(v) for v in self.heights_m)
        if h and (len(h) < 2 or any(a <= b for a, b in zip(h, h[1:]))):
            raise ValueError("population mesh heights_m must hold at least two distinct heights, top first")
        if h and self.adaptive:
            raise ValueError('population mesh: heights_m and refinement = "adaptive" exclude each other')
        if not 0 < self.min_spacing_m <= self.max_spacing_m:
            raise ValueError("population mesh needs 0 < min_spacing_m <= max_spacing_m")
        if not self.growth > 1:
            raise ValueError("population mesh growth must be > 1")
        if not min(self.lnT_step, self.log_ne_step, self.log_rho_step, self.velocity_step_m_s) > 0:
            raise ValueError("population mesh refinement steps must be positive")
        object.__setattr__(self, "heights_m", h)


VIEW_Z_REF_M = 0.0      # the rays' height origin of the shear: x = xi + t_x (z - z_ref) (ViewAngle.jl:9)


@dataclass(frozen=True)
class ViewGeometry:
    """The line of sight of an inversion (FFNOInversion.jl/src/Types.jl:40-66): mu = cos(theta) and the azimuth;
    inclined when mu < 1, with the slant t = tan(theta) (cos phi, sin phi)."""
    mu: float = 1.0
    azimuth_deg: float = 0.0

    def __post_init__(self):
        if not 0 < self.mu <= 1:
            raise ValueError("view mu must lie in (0, 1]")

    def slant(self):
        if self.mu >= 1.0:
            return 0.0, 0.0
        s = np.sqrt(1.0 - self.mu * self.mu) / self.mu
        return s * np.cos(np.deg2rad(self.azimuth_deg)), s * np.sin(np.deg2rad(self.azimuth_deg))

    @property
    def slanted(self):
        return self.mu < 1.0


class ShearPlan:
    """The per-level offsets of the periodic shear s (ViewAngle.jl:100-130) at mesh heights z, on the device: level k
    is read at (s t_x (z_k - z_ref) / dx, s t_y (z_k - z_ref) / dy) cells; s = +1 Cartesian -> rays, -1 back."""

    def __init__(self, z, dx, dy, t, s, device):
        z = np.asarray(z, dtype=np.float64)
        fx = s * t[0] * (z - VIEW_Z_REF_M) / (float(dx) if t[0] != 0 else 1.0)
        fy = s * t[1] * (z - VIEW_Z_REF_M) / (float(dy) if t[1] != 0 else 1.0)
        i0, j0 = np.floor(fx), np.floor(fy)
        if max(np.abs(i0).max(), np.abs(j0).max()) >= 2 ** 31:
            raise ValueError("inclined view: the shear offsets exceed the grid index range")
        self.i0 = torch.as_tensor(i0.astype(np.int32), device=device)
        self.j0 = torch.as_tensor(j0.astype(np.int32), device=device)
        self.wx = torch.as_tensor(fx - i0, device=device)
        self.wy = torch.as_tensor(fy - j0, device=device)
        self.nz = len(z)

    def apply(self, A, transpose=False):
        """The shear (or its transpose) of A [nz][nx][ny] (FP64, on the device)."""
        A = A.contiguous()
        nz, nx, ny = A.shape
        if nz != self.nz:
            raise ValueError(f"shear plan has {self.nz} levels; the array has {nz}")
        out = torch.empty_like(A)
        nat.call("ffno_shear_levels", A.data_ptr(), nz, nx, ny, self.i0.data_ptr(), self.j0.data_ptr(),
                 self.wx.data_ptr(), self.wy.data_ptr(), int(bool(transpose)), out.data_ptr(), _stream())
        return out


def population_mesh(c=PopulationMeshConfig()):
    """Mesh heights [m], top first: heights_m when given, else spacing_m up to uniform_top_m, then growing by stretch
    per point up to max_spacing_m (PopulationMesh.jl:90-99)."""
    if c.heights_m:
        return np.array(c.heights_m, dtype=np.float64)
    z = [float(c.bottom_m)]
    dz = float(c.spacing_m)
    while z[-1] < c.top_m:
        if z[-1] >= c.uniform_top_m:
            dz = min(dz * c.stretch, c.max_spacing_m)
        z.append(float(c.top_m) if c.top_m - z[-1] < 1.5 * dz else z[-1] + dz)
    return np.array(z[::-1])


# ------------------------------------------------------------------------------------------------ layouts
def columns(a):
    """(nz, nx, ny) -> [ncol][nz] with col = x + nx y (the reference's column-major order)."""
    a = np.asarray(a, dtype=np.float64)
    nz, nx, ny = a.shape
    return np.ascontiguousarray(a.transpose(2, 1, 0).reshape(nx * ny, nz))


def uncolumns(c, nx, ny):
    """[..., ncol, n] -> (..., n, nx, ny)."""
    c = np.asarray(c)
    lead = c.shape[:-2]
    n = c.shape[-1]
    return np.moveaxis(c.reshape(*lead, ny, nx, n), (-3, -2, -1), (-1, -2, -3)).copy()


def _dev(a, device):
    if torch.is_tensor(a):
        return a.to(device=device, dtype=torch.float64).contiguous()
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device=device)


def adaptive_population_mesh(config, atm, z, device="cuda", corona=False, extension=None, chunk_bytes=1 << 29):
    """adaptive_population_mesh (PopulationMesh.jl:213-262): one mesh for every column, as fine as the columns'
    features need. atm [6][ncol][nz] (T, vx, vy, vz, log10 ne, log10 rho) and z [ncol][nz] (top first), on the
    device or host. The columns' features on n probe heights min_spacing_m / 2 apart (ffno_mesh_features), for each
    probe interval the spacing needed to keep the changes of ln T, log10 ne, log10 rho and each velocity within their
    steps, the smallest over all columns (ffno_mesh_refine), clamped to [min_spacing_m, max_spacing_m] and graded so
    that one step is at most `growth` times the next; the mesh walks down from the top with those spacings. Probe
    heights below a column (and above it, with a corona temperature) need the hydrostatic extension."""
    c = config
    atm = _dev(atm, device)
    z = _dev(z, device)
    if c.extend:
        top, bottom = float(c.top_m), float(c.bottom_m)
    else:
        top, bottom = float(z[:, 0].max()), float(z[:, -1].min())
    n = max(2, int(np.ceil(2 * (top - bottom) / c.min_spacing_m)) + 1)
    probe = np.linspace(top, bottom, n)
    dz = float(probe[0] - probe[1])
    need = torch.full((n - 1,), float(c.max_spacing_m), dtype=torch.float64, device=device)
    ncol = z.shape[0]
    per = max(1, int(chunk_bytes // (n * 6 * 8)))
    for c0 in range(0, ncol, per):
        c1 = min(ncol, c0 + per)
        maps = MeshMaps(z[c0:c1], probe, device, corona=corona)
        f, kind = maps.features(atm[:, c0:c1].contiguous())
        if bool((kind >= DEEP).any()):
            if extension is None:
                raise ValueError("adaptive mesh: probe heights lie outside the columns: the hydrostatic extension "
                                 "(an EOS) is needed")
            fh = f.cpu().numpy()
            extension.fill(fh, kind.cpu().numpy(), atm[:, c0:c1].cpu().numpy(), maps.z.cpu().numpy(), probe)
            f = _dev(fh, device)
        nat.call("ffno_mesh_refine", f.data_ptr(), c1 - c0, n, dz, float(c.lnT_step), float(c.log_ne_step),
                 float(c.log_rho_step), float(c.velocity_step_m_s), need.data_ptr(), _stream())
    least = need.cpu().numpy()
    h = np.clip(np.concatenate([[least[0]], np.minimum(least[:-1], least[1:]), [least[-1]]]), c.min_spacing_m,
                c.max_spacing_m)
    a = (c.growth - 1) * dz
    for i in range(1, n):
        h[i] = min(h[i], h[i - 1] + a)
    for i in range(n - 2, -1, -1):
        h[i] = min(h[i], h[i + 1] + a)

    def spacing(zz):
        u = min(max((top - zz) / dz, 0.0), n - 1)
        i = min(int(np.floor(u)), n - 2)
        return h[i] + (u - i) * (h[i + 1] - h[i])

    def lowest(zz, s):
        lo = min(max(int(np.floor((top - zz) / dz)) + 2, 1), n)
        hi = min(max(int(np.ceil((top - zz + s) / dz)), 1), n)
        window = h[lo - 1:hi]
        return min(spacing(zz), spacing(zz - s), window.min() if window.size else np.inf)

    mesh = [top]
    while True:
        zz = mesh[-1]
        step = spacing(zz)
        for _ in range(3):                    # the smallest spacing over the step itself
            step = lowest(zz, step)
        if zz - step <= bottom + step / 2:
            mesh.append(bottom)
            break
        mesh.append(zz - step)
    return np.array(mesh)


class MeshMaps:
    """The device maps of one atmosphere geometry (column heights z [ncol][nz], mesh [nm]) on FP64 tensors."""

    def __init__(self, z_cols, mesh, device="cuda", corona=False):
        self.device = torch.device(device)
        self.z = _dev(z_cols, self.device)
        self.mesh = _dev(mesh, self.device)
        self.ncol, self.nz = self.z.shape
        self.nm = self.mesh.numel()
        if self.nz < 2 or self.nm < 1:
            raise ValueError("a column needs at least two heights and the mesh one")
        if bool((self.z[:, 1:] >= self.z[:, :-1]).any()) or bool((self.mesh[1:] >= self.mesh[:-1]).any()):
            raise ValueError("column heights and the mesh must decrease (top first)")
        self.corona = int(bool(corona))

    def features(self, atm):
        """atm [6][ncol][nz] (T, vx, vy, vz, log10 ne, log10 rho) -> mesh features f [ncol][nm][6] and kind
        [ncol][nm]."""
        f = torch.empty(self.ncol, self.nm, 6, dtype=torch.float64, device=self.device)
        kind = torch.empty(self.ncol, self.nm, dtype=torch.int8, device=self.device)
        nat.call("ffno_mesh_features", atm.data_ptr(), self.z.data_ptr(), self.ncol, self.nz, self.mesh.data_ptr(),
                 self.nm, self.corona, f.data_ptr(), kind.data_ptr(), _stream())
        return f, kind

    def features_vjp(self, atm, f, fm_bar):
        fbar = torch.empty(self.ncol, self.nz, 6, dtype=torch.float64, device=self.device)
        zbar = torch.empty(self.ncol, self.nz, dtype=torch.float64, device=self.device)
        nat.call("ffno_mesh_features_vjp", atm.data_ptr(), self.z.data_ptr(), self.ncol, self.nz,
                 self.mesh.data_ptr(), self.nm, self.corona, f.data_ptr(), fm_bar.data_ptr(), fbar.data_ptr(),
                 zbar.data_ptr(), _stream())
        return fbar, zbar

    def features_jvp(self, atm, f, fd):
        out = torch.empty(self.ncol, self.nm, 6, dtype=torch.float64, device=self.device)
        nat.call("ffno_mesh_features_jvp", atm.data_ptr(), self.z.data_ptr(), self.ncol, self.nz, self.mesh.data_ptr(),
                 self.nm, self.corona, f.data_ptr(), fd.data_ptr(), out.data_ptr(), _stream())
        return out

    def backmap(self, pm):
        """pm [L][ncol][nm] -> column populations [L][ncol][nz]."""
        L = pm.shape[0]
        out = torch.empty(L, self.ncol, self.nz, dtype=torch.float64, device=self.device)
        nat.call("ffno_mesh_backmap", pm.data_ptr(), self.mesh.data_ptr(), self.nm, self.z.data_ptr(), self.ncol,
                 self.nz, L, out.data_ptr(), _stream())
        return out

    def backmap_vjp(self, pm, pop_bar):
        L = pm.shape[0]
        pm_bar = torch.empty_like(pm)
        zbar = torch.empty(self.ncol, self.nz, dtype=torch.float64, device=self.device)
        nat.call("ffno_mesh_backmap_vjp", pm.data_ptr(), self.mesh.data_ptr(), self.nm, self.z.data_ptr(), self.ncol,
                 self.nz, L, pop_bar.data_ptr(), pm_bar.data_ptr(), zbar.data_ptr(), _stream())
        return pm_bar, zbar

    def backmap_jvp(self, pm, pm_dot):
        L = pm.shape[0]
        out = torch.empty(L, self.ncol, self.nz, dtype=torch.float64, device=self.device)
        nat.call("ffno_mesh_backmap_jvp", pm.data_ptr(), pm_dot.data_ptr(), self.mesh.data_ptr(), self.nm,
                 self.z.data_ptr(), self.ncol, self.nz, L, out.data_ptr(), _stream())
        return out


class MeshPopulationModel:
    """The reference's MeshPopulationModel (PopulationMesh.jl:101-118, 343-470) around an inner population model:
    `inner` has predict(features, z, dx, dy) -> (nz, nx, ny, L), vjp(features, z, dx, dy, population_bar) ->
    (feature_bar, z_bar) and jvp(features, z, dx, dy, feature_dot) -> (nz, nx, ny, L), in the array conventions of this
    module (GB300Backend through BackendInner, or any other). `extension`, needed only when some mesh point lies below
    a column (or above it with a corona temperature), has fill(f, kind, atm, z, mesh), vjp(fm_bar, kind, atm, z, mesh)
    -> (a_bar [ncol][nz][6], z_bar [ncol][nz]) and jvp(fd, kind, atm, z, mesh) -> fm_dot on host arrays in the [ncol]
    layouts. `view` (ViewGeometry) inclined: the columns are the footprint rays of that view, and the mesh features
    are sheared to Cartesian columns for the inner model and its populations back (PopulationMesh.jl:296-334,
    377-401, 445-462). config.adaptive: the mesh is rebuilt from each atmosphere (adaptive_population_mesh)."""

    def __init__(self, inner, config=PopulationMeshConfig(), extension=None, device="cuda", view=None):
        self.inner = inner
        self.config = config
        self.mesh = population_mesh(config)
        self.extension = extension
        self.device = torch.device(device)
        self.view = view or ViewGeometry()

    # -------------------------------------------------------------------------------------------- pieces
    def _setup(self, features, z):
        features = np.asarray(features, dtype=np.float64)
        z = np.asarray(z, dtype=np.float64)
        if features.ndim != 4 or features.shape[0] != 6 or features.shape[1:] != z.shape:
            raise ValueError(f"expected features (6,nz,nx,ny) and z (nz,nx,ny), got {features.shape}, {z.shape}")
        nz, nx, ny = z.shape
        atm = _dev(np.stack([columns(features[c]) for c in range(6)]), self.device)
        zc = columns(z)
        corona = self.config.corona_temperature_k > 0
        if self.config.adaptive:
            self.mesh = adaptive_population_mesh(self.config, atm, zc, self.device, corona, self.extension)
        maps = MeshMaps(zc, self.mesh, self.device, corona=corona)
        return maps, atm, (nz, nx, ny)

    def _mesh_features(self, maps, atm, shape):
        f, kind = maps.features(atm)
        if bool((kind >= DEEP).any()):
            if self.extension is None:
                raise ValueError("mesh points lie outside the columns: the hydrostatic extension (an EOS) is needed")
            fh, kh = f.cpu().numpy(), kind.cpu().numpy()
            self.extension.fill(fh, kh, atm.cpu().numpy(), maps.z.cpu().numpy(), self.mesh)
            f = _dev(fh, self.device)
        return f, kind

    def _inner_inputs(self, f, shape):
        nz, nx, ny = shape
        fm = uncolumns(f.permute(2, 0, 1).cpu().numpy(), nx, ny)          # (6, nm, nx, ny)
        zm = np.broadcast_to(self.mesh[:, None, None], (len(self.mesh), nx, ny)).copy()
        return fm, zm

    def _pm(self, pm_cols):
        return _dev(pm_cols, self.device)

    # -------------------------------------------------------------------------------------------- inclined view
    def _plans(self, dx, dy):
        """Shear plans of the mesh levels: rays -> Cartesian (s = -1) and Cartesian -> rays (s = +1)."""
        t = self.view.slant()
        return (ShearPlan(self.mesh, dx, dy, t, -1, self.device), ShearPlan(self.mesh, dx, dy, t, 1, self.device))

    def _to_cartesian(self, fm, plan):
        """Cartesian mesh features from the rays' (6, nm, nx, ny): ln T and the others sheared, T exponentiated back
        (PopulationMesh.jl:296-307)."""
        a = _dev(fm, self.device)
        out = torch.empty_like(a)
        out[0] = torch.exp(plan.apply(torch.log(a[0])))
        for c in range(1, 6):
            out[c] = plan.apply(a[c])
        return out.cpu().numpy()

    def _to_rays(self, pc, plan):
        """Ray mesh populations from the Cartesian ones (nm, nx, ny, L): ln n sheared (PopulationMesh.jl:309-317)."""
        p = _dev(pc, self.device)
        out = torch.empty_like(p)
        for l in range(p.shape[-1]):
            out[..., l] = torch.exp(plan.apply(torch.log(p[..., l])))
        return out.cpu().numpy()

    def _predict_mesh(self, fm, zm, dx, dy):
        """Mesh populations (nm, nx, ny, L) of the ray mesh features, and (plans, Cartesian features and
        populations) for an inclined view."""
        if not self.view.slanted:
            return np.asarray(self.inner.predict(fm, zm, dx, dy), dtype=np.float64), None
        plans = self._plans(dx, dy)
        fc = self._to_cartesian(fm, plans[0])
        pc = np.asarray(self.inner.predict(fc, zm, dx, dy), dtype=np.float64)
        return self._to_rays(pc, plans[1]), (plans, fc, pc)

    # -------------------------------------------------------------------------------------------- API
    def predict(self, features, z, dx, dy):
        """Column populations (nz, nx, ny, L) (PopulationMesh.jl:343-360)."""
        maps, atm, shape = self._setup(features, z)
        f, _ = self._mesh_features(maps, atm, shape)
        fm, zm = self._inner_inputs(f, shape)
        pm, _ = self._predict_mesh(fm, zm, dx, dy)                                # (nm, nx, ny, L)
        pm_c = np.stack([columns(pm[..., l]) for l in range(pm.shape[-1])])
        out = maps.backmap(self._pm(pm_c)).cpu().numpy()
        return np.moveaxis(uncolumns(out, shape[1], shape[2]), 0, -1)

    def vjp(self, features, z, dx, dy, population_bar):
        """(feature_bar (6, nz, nx, ny), z_bar (nz, nx, ny)) (PopulationMesh.jl:362-408)."""
        maps, atm, shape = self._setup(features, z)
        nz, nx, ny = shape
        f, kind = self._mesh_features(maps, atm, shape)
        fm, zm = self._inner_inputs(f, shape)
        pm, cart = self._predict_mesh(fm, zm, dx, dy)
        L = pm.shape[-1]
        pm_c = self._pm(np.stack([columns(pm[..., l]) for l in range(L)]))
        pb = np.asarray(population_bar, dtype=np.float64)
        pb_c = _dev(np.stack([columns(pb[..., l]) for l in range(L)]), self.device)
        pm_bar, zbar_back = maps.backmap_vjp(pm_c, pb_c)
        pm_bar_h = np.moveaxis(uncolumns(pm_bar.cpu().numpy(), nx, ny), 0, -1)        # (nm, nx, ny, L)
        if cart is None:
            fm_bar, _ = self.inner.vjp(fm, zm, dx, dy, pm_bar_h)                       # mesh heights fixed
            fm_bar = np.asarray(fm_bar, dtype=np.float64)
        else:
            # the transposes of the two shears around the inner model (exp / log chain rules outside them):
            # pc_bar = S+^T(pm_bar pm) / pc, then T_bar = S-^T(Tc_bar Tc) / T and the others S-^T(.)
            (sm, sp), fc, pc = cart
            g = _dev(pm_bar_h * pm, self.device)
            pcd = _dev(pc, self.device)
            pc_bar = torch.empty_like(g)
            for l in range(L):
                pc_bar[..., l] = sp.apply(g[..., l], transpose=True) / pcd[..., l]
            fmc_bar, _ = self.inner.vjp(fc, zm, dx, dy, pc_bar.cpu().numpy())
            fmc_bar = _dev(fmc_bar, self.device)
            fcd, fmd = _dev(fc, self.device), _dev(fm, self.device)
            out = torch.empty_like(fmc_bar)
            out[0] = sm.apply(fmc_bar[0] * fcd[0], transpose=True) / fmd[0]
            for c in range(1, 6):
                out[c] = sm.apply(fmc_bar[c], transpose=True)
            fm_bar = out.cpu().numpy()
        fm_bar_c = _dev(np.stack([columns(fm_bar[c]) for c in range(6)]).transpose(1, 2, 0), self.device)
        fbar, zbar = maps.features_vjp(atm, f, fm_bar_c)
        fbar_h, zbar_h = fbar.cpu().numpy(), zbar.cpu().numpy() + zbar_back.cpu().numpy()
        if bool((kind >= DEEP).any()):
            a_bar, z_ext = self.extension.vjp(fm_bar_c.cpu().numpy(), kind.cpu().numpy(), atm.cpu().numpy(),
                                              maps.z.cpu().numpy(), self.mesh)
            T = atm[0].cpu().numpy()
            fbar_h[..., 0] += a_bar[..., 0] / T
            fbar_h[..., 1:] += a_bar[..., 1:]
            zbar_h += z_ext
        feature_bar = uncolumns(fbar_h.transpose(2, 0, 1), nx, ny)
        return feature_bar, uncolumns(zbar_h, nx, ny)

    def jvp(self, features, z, dx, dy, feature_dot):
        """Population tangents (nz, nx, ny, L) at fixed heights (PopulationMesh.jl:427-470)."""
        maps, atm, shape = self._setup(features, z)
        nz, nx, ny = shape
        f, kind = self._mesh_features(maps, atm, shape)
        fm, zm = self._inner_inputs(f, shape)
        pm, cart = self._predict_mesh(fm, zm, dx, dy)
        L = pm.shape[-1]
        fd = np.asarray(feature_dot, dtype=np.float64)
        fd_c = _dev(np.stack([columns(fd[c]) for c in range(6)]).transpose(1, 2, 0), self.device)
        fm_dot = maps.features_jvp(atm, f, fd_c)
        if bool((kind >= DEEP).any()):
            ext = self.extension.jvp(fd_c.cpu().numpy(), kind.cpu().numpy(), atm.cpu().numpy(), maps.z.cpu().numpy(),
                                     self.mesh)
            fm_dot = fm_dot + _dev(ext, self.device)
        fmd = uncolumns(fm_dot.permute(2, 0, 1).cpu().numpy(), nx, ny)
        if cart is None:
            pm_dot = np.asarray(self.inner.jvp(fm, zm, dx, dy, fmd), dtype=np.float64)
        else:
            # the tangents of the two shears: Tc_dot = Tc S-(T_dot / T), the others S-(.); pm_dot = pm S+(pc_dot / pc)
            (sm, sp), fc, pc = cart
            a, fcd, fmt = _dev(fmd, self.device), _dev(fc, self.device), _dev(fm, self.device)
            fmc_dot = torch.empty_like(a)
            fmc_dot[0] = sm.apply(a[0] / fmt[0]) * fcd[0]
            for c in range(1, 6):
                fmc_dot[c] = sm.apply(a[c])
            pc_dot = _dev(self.inner.jvp(fc, zm, dx, dy, fmc_dot.cpu().numpy()), self.device)
            pcd, pmd = _dev(pc, self.device), _dev(pm, self.device)
            out = torch.empty_like(pc_dot)
            for l in range(L):
                out[..., l] = sp.apply(pc_dot[..., l] / pcd[..., l]) * pmd[..., l]
            pm_dot = out.cpu().numpy()
        pm_c = self._pm(np.stack([columns(pm[..., l]) for l in range(L)]))
        pmd_c = self._pm(np.stack([columns(pm_dot[..., l]) for l in range(L)]))
        out = maps.backmap_jvp(pm_c, pmd_c).cpu().numpy()
        return np.moveaxis(uncolumns(out, nx, ny), 0, -1)


class BackendInner:
    """GB300Backend (predict_local / vjp_local / jvp_local) as the inner model of MeshPopulationModel."""

    def __init__(self, backend):
        self.backend = backend

    def predict(self, features, z, dx, dy):
        return self.backend.predict_local(features.astype(np.float32), z.astype(np.float32), dx, dy)

    def vjp(self, features, z, dx, dy, population_bar):
        g = self.backend.vjp_local(features.astype(np.float32), z.astype(np.float32), dx, dy,
                                   population_bar.astype(np.float32))
        return g["features"], g["z_scale"]

    def jvp(self, features, z, dx, dy, feature_dot):
        return self.backend.jvp_local(features.astype(np.float32), z.astype(np.float32), dx, dy,
                                      feature_dot.astype(np.float32))
