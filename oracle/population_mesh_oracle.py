"""CPU restatement of the reference's population-mesh maps (FFNOInversion.jl/src/PopulationMesh.jl), float64 numpy.

TEST INFRASTRUCTURE: only tests/ import this module, as the checker of the CUDA kernels in ffnoml_gb300/csrc/mesh_f64.cu;
the product never calls it.

Layouts follow the reference's column-major Julia arrays read as row-major C arrays: a column (x, y) is col = x + nx y,
and an atmosphere variable [nz, nx, ny] is atm[col][k]; mesh features f[6, nm, nx, ny] are f[col][m][c]; mesh
populations pm[nm, nx, ny, L] are pm[l][col][m]; column populations [nz, nx, ny, L] are out[l][col][k].

Parity is pinned by the reference's own known-answer tests (FFNOInversion.jl/test/population_mesh.jl:56-101): exact
interpolation of variables linear in height inside a column, exact back-mapping of populations log-linear in height,
the fixed mesh's shape (:40-44), and the VJP against central differences. The hydrostatic corona and deep extensions
(:141-180, :122-139) need the HSEMHS EOS table and stay with the caller: points above the column top (with a corona
temperature) and below its bottom are reported by kind and left unfilled here, as in the kernels.
"""
import numpy as np

LN10 = np.log(10.0)
INSIDE, TOP, DEEP, CORONA = 0, 1, 2, 3


def population_mesh(bottom_m=-1.0e6, top_m=1.4e7, spacing_m=2.0e4, uniform_top_m=4.5e6, stretch=1.01,
                    max_spacing_m=1.0e5, heights_m=()):
    """Mesh heights, top first (PopulationMesh.jl:90-99)."""
    if len(heights_m):
        return np.array(heights_m, dtype=np.float64)
    z = [float(bottom_m)]
    dz = float(spacing_m)
    while z[-1] < top_m:
        if z[-1] >= uniform_top_m:
            dz = min(dz * stretch, max_spacing_m)
        z.append(float(top_m) if top_m - z[-1] < 1.5 * dz else z[-1] + dz)
    return np.array(z[::-1])


def column_variables(atm):
    """(ln T, vx, vy, vz, log10 ne, log10 rho) [6][ncol][nz] from atm = (T, vx, vy, vz, log10 ne, log10 rho), the
    service's feature channels (PopulationMesh.jl:182-190 takes the logarithms of ne and rho)."""
    a = np.array(atm, dtype=np.float64)
    a[0] = np.log(a[0])
    return a


def locate(zc, zeta, k):
    """(:top | :inside | :deep, k, w) of height zeta in a column zc (top first), 0-based k, the search resumed from k
    (PopulationMesh.jl:192-198)."""
    if zeta >= zc[0]:
        return TOP, 0, 0.0
    if zeta < zc[-1]:
        return DEEP, len(zc) - 1, 0.0
    while zc[k + 1] > zeta:
        k += 1
    return INSIDE, k, (zc[k] - zeta) / (zc[k] - zc[k + 1])


def features(atm, z, mesh, corona=False):
    """Mesh features f[col][m][6] (T, vx, vy, vz, log10 ne, log10 rho) and kind[col][m] (PopulationMesh.jl:200-227,
    inside and held-top points; deep and corona points are marked and left zero)."""
    a = column_variables(atm)
    ncol, nz = z.shape
    nm = len(mesh)
    f = np.zeros((ncol, nm, 6))
    kind = np.zeros((ncol, nm), np.int8)
    for col in range(ncol):
        zc = z[col]
        k = 0
        for m in range(nm):
            kd, k, w = locate(zc, mesh[m], k)
            if kd == DEEP:
                kind[col, m] = DEEP
                continue
            if kd == TOP and corona and mesh[m] > zc[0]:
                kind[col, m] = CORONA
                continue
            kind[col, m] = kd
            for c in range(6):
                f[col, m, c] = a[c, col, 0] if kd == TOP else (1 - w) * a[c, col, k] + w * a[c, col, k + 1]
            f[col, m, 0] = np.exp(f[col, m, 0])
    return f, kind


def bracket(mesh, zeta):
    """(j0, j1, u) with mesh[j0] >= zeta >= mesh[j1], clamped to the ends (PopulationMesh.jl:335-341), 0-based."""
    nm = len(mesh)
    if zeta >= mesh[0]:
        return 0, 0, 0.0
    if zeta <= mesh[-1]:
        return nm - 1, nm - 1, 0.0
    j = int(np.sum(mesh >= zeta)) - 1        # the last index with mesh[j] >= zeta (mesh decreasing)
    return j, j + 1, (mesh[j] - zeta) / (mesh[j] - mesh[j + 1])


def backmap(pm, mesh, z):
    """Column populations out[l][col][k] = exp((1-u) ln pm[j0] + u ln pm[j1]) (PopulationMesh.jl:343-360)."""
    L, ncol, _ = pm.shape
    nz = z.shape[1]
    out = np.empty((L, ncol, nz))
    for col in range(ncol):
        for k in range(nz):
            j0, j1, u = bracket(mesh, z[col, k])
            out[:, col, k] = np.exp((1 - u) * np.log(pm[:, col, j0]) + u * np.log(pm[:, col, j1]))
    return out


def backmap_vjp(pm, mesh, z, pop_bar):
    """pm_bar[l][col][m] and z_bar[col][k] of the back-map (PopulationMesh.jl:371-381), the reference's loop order."""
    L, ncol, nm = pm.shape
    nz = z.shape[1]
    pm_bar = np.zeros_like(pm)
    z_bar = np.zeros((ncol, nz))
    for col in range(ncol):
        for k in range(nz):
            j0, j1, u = bracket(mesh, z[col, k])
            for l in range(L):
                p = np.exp((1 - u) * np.log(pm[l, col, j0]) + u * np.log(pm[l, col, j1]))
                g = pop_bar[l, col, k] * p
                pm_bar[l, col, j0] += g * (1 - u) / pm[l, col, j0]
                pm_bar[l, col, j1] += g * u / pm[l, col, j1]
                if j0 != j1:
                    z_bar[col, k] -= g * (np.log(pm[l, col, j1]) - np.log(pm[l, col, j0])) / (mesh[j0] - mesh[j1])
    return pm_bar, z_bar


def backmap_jvp(pm, mesh, z, pm_dot):
    """Tangent of the back-map at fixed heights (PopulationMesh.jl:458-468)."""
    L, ncol, _ = pm.shape
    nz = z.shape[1]
    out = np.empty((L, ncol, nz))
    for col in range(ncol):
        for k in range(nz):
            j0, j1, u = bracket(mesh, z[col, k])
            p = np.exp((1 - u) * np.log(pm[:, col, j0]) + u * np.log(pm[:, col, j1]))
            out[:, col, k] = p * ((1 - u) * pm_dot[:, col, j0] / pm[:, col, j0] + u * pm_dot[:, col, j1] / pm[:, col, j1])
    return out


def features_vjp(atm, z, mesh, f, fb, corona=False):
    """Transpose of `features` for inside and held-top points: fb[col][m][6] -> feature_bar[col][k][6] (w.r.t. T, vx,
    vy, vz, log10 ne, log10 rho) and z_bar[col][k] (PopulationMesh.jl:522-573 without the deep and corona terms)."""
    a = column_variables(atm)
    T = atm[0]
    ncol, nz = z.shape
    fbar = np.zeros((ncol, nz, 6))
    z_bar = np.zeros((ncol, nz))
    for col in range(ncol):
        zc = z[col]
        a_bar = np.zeros((6, nz))
        k = 0
        for m in range(len(mesh)):
            kd, k, w = locate(zc, mesh[m], k)
            if kd == DEEP or (kd == TOP and corona and mesh[m] > zc[0]):
                continue
            G = [fb[col, m, c] * (f[col, m, 0] if c == 0 else 1.0) for c in range(6)]
            if kd == TOP:
                for c in range(6):
                    a_bar[c, 0] += G[c]
            else:
                w_bar = 0.0
                for c in range(6):
                    a_bar[c, k] += G[c] * (1 - w)
                    a_bar[c, k + 1] += G[c] * w
                    w_bar += G[c] * (a[c, col, k + 1] - a[c, col, k])
                d = zc[k] - zc[k + 1]
                z_bar[col, k] += w_bar * (1 - w) / d
                z_bar[col, k + 1] += w_bar * w / d
        fbar[col, :, 0] = a_bar[0] / T[col]
        fbar[col, :, 1:] = a_bar[1:].T
    return fbar, z_bar


def features_jvp(atm, z, mesh, f, fd, corona=False):
    """Tangent of `features` at fixed heights: fd[col][k][6] (w.r.t. T, vx, vy, vz, log10 ne, log10 rho) ->
    fm_dot[col][m][6] (PopulationMesh.jl:475-518 without the deep and corona terms)."""
    T = atm[0]
    ncol, nz = z.shape
    out = np.zeros((ncol, len(mesh), 6))
    for col in range(ncol):
        zc = z[col]
        ad = fd[col].T.copy()
        ad[0] = fd[col, :, 0] / T[col]
        k = 0
        for m in range(len(mesh)):
            kd, k, w = locate(zc, mesh[m], k)
            if kd == DEEP or (kd == TOP and corona and mesh[m] > zc[0]):
                continue
            for c in range(6):
                out[col, m, c] = ad[c, 0] if kd == TOP else (1 - w) * ad[c, k] + w * ad[c, k + 1]
            out[col, m, 0] *= f[col, m, 0]
    return out


# ------------------------------------------------------------------------------------------------ inclined views
VIEW_Z_REF_M = 0.0      # the ray origin of the shear (FFNOInversion.jl/src/ViewAngle.jl:9)


def slant(mu, azimuth_deg):
    """t = tan(theta) (cos phi, sin phi) of an inclined view, mu = cos(theta) (FFNOInversion.jl/src/Types.jl:64-66);
    (0, 0) for mu = 1."""
    if mu >= 1.0:
        return 0.0, 0.0
    s = np.sqrt(1.0 - mu * mu) / mu
    return s * np.cos(np.deg2rad(azimuth_deg)), s * np.sin(np.deg2rad(azimuth_deg))


def shear_plan(z, dx, dy, t, s):
    """Per level k: the integer cell offsets (i0, j0) and the fractions (wx, wy) of the shear s (t_x (z_k - z_ref)/dx,
    t_y (z_k - z_ref)/dy) (ViewAngle.jl:107-115)."""
    z = np.asarray(z, dtype=np.float64)
    fx = s * t[0] * (z - VIEW_Z_REF_M) / dx
    fy = s * t[1] * (z - VIEW_Z_REF_M) / dy
    i0, j0 = np.floor(fx).astype(np.int64), np.floor(fy).astype(np.int64)
    return i0, j0, fx - i0, fy - j0


def shear_levels(A, plan):
    """out[k, i, j] = the periodic bilinear read of level k of A (nz, nx, ny) at the level's offset (ViewAngle.jl:
    132-145), by loops as the reference writes it."""
    i0, j0, wx, wy = plan
    nz, nx, ny = A.shape
    out = np.empty_like(A, dtype=np.float64)
    for k in range(nz):
        for i in range(nx):
            ia = (i + i0[k]) % nx
            ib = (ia + 1) % nx
            for j in range(ny):
                ja = (j + j0[k]) % ny
                jb = (ja + 1) % ny
                out[k, i, j] = (1 - wy[k]) * ((1 - wx[k]) * A[k, ia, ja] + wx[k] * A[k, ib, ja]) + \
                    wy[k] * ((1 - wx[k]) * A[k, ia, jb] + wx[k] * A[k, ib, jb])
    return out


def shear_levels_transpose(out_bar, plan):
    """The transpose of shear_levels as the reference's scatter (ViewAngle.jl:147-162), into a zero array."""
    i0, j0, wx, wy = plan
    nz, nx, ny = out_bar.shape
    A_bar = np.zeros_like(out_bar, dtype=np.float64)
    for k in range(nz):
        for i in range(nx):
            ia = (i + i0[k]) % nx
            ib = (ia + 1) % nx
            for j in range(ny):
                ja = (j + j0[k]) % ny
                jb = (ja + 1) % ny
                g = out_bar[k, i, j]
                A_bar[k, ia, ja] += (1 - wy[k]) * (1 - wx[k]) * g
                A_bar[k, ib, ja] += (1 - wy[k]) * wx[k] * g
                A_bar[k, ia, jb] += wy[k] * (1 - wx[k]) * g
                A_bar[k, ib, jb] += wy[k] * wx[k] * g
    return A_bar


# ------------------------------------------------------------------------------------------------ adaptive mesh
def adaptive_mesh(atm, z, mesh_top, mesh_bottom, min_spacing_m, max_spacing_m, growth, lnT_step, log_ne_step,
                  log_rho_step, velocity_step_m_s, extend=True, fill=None):
    """adaptive_population_mesh (PopulationMesh.jl:213-262): atm [6][ncol][nz], z [ncol][nz] top first. Probe
    heights below a column are filled by fill(f, kind) (a stand-in for the hydrostatic extension), else refused."""
    top, bottom = (float(mesh_top), float(mesh_bottom)) if extend else (float(z[:, 0].max()), float(z[:, -1].min()))
    n = max(2, int(np.ceil(2 * (top - bottom) / min_spacing_m)) + 1)
    probe = np.linspace(top, bottom, n)
    dz = probe[0] - probe[1]
    f, kind = features(atm, z, probe)
    if (kind >= DEEP).any():
        if fill is None:
            raise ValueError("probe heights below a column need the hydrostatic extension")
        fill(f, kind)
    need = np.full(n - 1, float(max_spacing_m))
    for col in range(f.shape[0]):
        g = f[col]
        r = np.maximum.reduce([np.abs(np.log(g[:-1, 0] / g[1:, 0])) / lnT_step,
                               np.abs(g[:-1, 4] - g[1:, 4]) / log_ne_step,
                               np.abs(g[:-1, 5] - g[1:, 5]) / log_rho_step] +
                              [np.abs(g[:-1, v] - g[1:, v]) / velocity_step_m_s for v in (1, 2, 3)])
        pos = r > 0
        need[pos] = np.minimum(need[pos], dz / r[pos])
    h = np.clip(np.concatenate([[need[0]], np.minimum(need[:-1], need[1:]), [need[-1]]]), min_spacing_m,
                max_spacing_m)
    a = (growth - 1) * dz
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
        for _ in range(3):
            step = lowest(zz, step)
        if zz - step <= bottom + step / 2:
            mesh.append(bottom)
            break
        mesh.append(zz - step)
    return np.array(mesh)
