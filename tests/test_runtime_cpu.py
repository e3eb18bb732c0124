"""GB300Backend's request validation (ffno_fsdp_runtime.py:245-258, 306-320, 350-365: the same ValueErrors) runs on
the host before any device work: the device steps are replaced by a stub that fails the test if reached."""
import types

import numpy as np
import pytest

from ffnoml_gb300.runtime import GB300Backend


def _backend(levels=12):
    be = GB300Backend.__new__(GB300Backend)                  # no device: the host checks alone
    be.model = types.SimpleNamespace(out_channels=levels)

    def no_device(*args, **kw):
        raise AssertionError("device work before the request was validated")
    be._prepare = be._upload = be._stage = no_device
    return be


def _request(shape=(8, 5, 4)):
    g = np.random.default_rng(1)
    f = g.normal(size=(6,) + shape).astype(np.float32)
    f[0] = 5000.0
    return f, np.linspace(1e6, 0.0, shape[0])[:, None, None] * np.ones(shape, np.float32)


@pytest.mark.parametrize("op", ["predict", "vjp", "jvp"])
def test_feature_and_height_shapes_are_checked(op):
    be, (f, z) = _backend(), _request()
    call = {"predict": lambda ff, zz: be.predict_local(ff, zz, 48e3, 48e3),
            "vjp": lambda ff, zz: be.vjp_local(ff, zz, 48e3, 48e3, np.zeros(zz.shape + (12,), np.float32)),
            "jvp": lambda ff, zz: be.jvp_local(ff, zz, 48e3, 48e3, np.zeros_like(ff))}[op]
    with pytest.raises(ValueError, match=r"features must have shape"):
        call(f[:5], z)
    with pytest.raises(ValueError, match=r"z_scale must have shape"):
        call(f, z[:-1])


def test_cotangent_shape_is_checked():
    be, (f, z) = _backend(), _request()
    with pytest.raises(ValueError, match=r"population_cotangent has shape .*expected \(8, 5, 4, 12\)"):
        be.vjp_local(f, z, 48e3, 48e3, np.zeros((8, 5, 4, 6), np.float32))


def test_tangent_shape_and_values_are_checked():
    be, (f, z) = _backend(), _request()
    with pytest.raises(ValueError, match=r"feature_tangent has shape"):
        be.jvp_local(f, z, 48e3, 48e3, np.zeros((6, 8, 5, 3), np.float32))
    t = np.zeros_like(f)
    t[3, 2, 1, 0] = np.inf
    with pytest.raises(ValueError, match=r"NaN or Inf"):
        be.jvp_local(f, z, 48e3, 48e3, t)


def test_host_geometry_decides_the_shared_grid_like_the_column_kernel():
    """Executor.geometry_host (the service backend's per-request analysis, no device read-back): every column equal
    to column 0 after subtracting its own minimum, in float32, gives the shared path; one column apart, or two
    samples whose columns differ, gives the per-column path with every column's heights."""
    import numpy as np
    from ffnoml_gb300 import create_ffno3d
    from ffnoml_gb300.executor import Executor
    ex = Executor(create_ffno3d(6, 6, atoms=["H"], width=16, n_layers=1, hidden_spectral=16, hidden_vertical=16,
                                z_min_wavelength=0.5))
    D, H, W = 12, 5, 4
    col = np.linspace(14.0, -1.0, D, dtype=np.float32)
    z = np.broadcast_to(col[:, None, None], (D, H, W)).copy()[None]
    g = ex.geometry_host(z)
    assert g.shared and g.columns is None and abs(g.span - 15.0) < 1e-6
    assert np.allclose(g.column_raw, col)
    bent = z.copy()
    bent[0, 3, 2, 1] += np.float32(0.25)
    g = ex.geometry_host(bent)
    assert not g.shared and g.columns.shape == (1, H * W, D)
    assert g.columns[0, 2 * W + 1, 3] == np.float32(col[3] + np.float32(0.25))
    two = np.concatenate([z, z * np.float32(0.5)])
    g = ex.geometry_host(two)
    assert not g.shared and g.columns.shape == (2, H * W, D)


def _geo_fields(g):
    return (g.shared, g.span, np.asarray(g.column).tobytes(), np.asarray(g.column_raw).tobytes(), g.length,
            g.k.numpy().tobytes(), None if g.columns is None else np.asarray(g.columns).tobytes())


@pytest.mark.parametrize("kind", ["shared", "per_column", "shifted", "rounding", "nonfinite"])
def test_heights_scan_gives_the_exact_geometry(kind):
    """The request's height analysis (_heights_scan on the heights in metres, column (0, 0) alone divided when every
    column equals it) gives the geometry of the analysis of all heights divided by 1e6, in the backend's layout and in
    the wire layout (columns first); non-finite heights are reported as such."""
    import torch
    from ffnoml_gb300 import create_ffno3d
    from ffnoml_gb300.runtime import _heights_scan
    ex = create_ffno3d(6, 12, atoms=["H", "CA"], width=32, n_layers=2).executor()
    D, H, W = 40, 6, 5
    z = (np.linspace(14.0, -1.0, D, dtype=np.float32)[:, None, None] * np.ones((D, H, W), np.float32)) * 1e6
    if kind == "per_column":
        z = z * (1.0 + 0.01 * np.arange(H * W, dtype=np.float32).reshape(1, H, W))
    elif kind == "shifted":         # every column the same grid shifted: shared after the shift, not equal in metres
        z = z + 1e4 * np.arange(H * W, dtype=np.float32).reshape(1, H, W)
    elif kind == "rounding":        # columns differing in metres by one ULP, which the division may merge
        z[:, 2, 3] = np.nextafter(z[:, 2, 3], np.float32(np.inf))
    elif kind == "nonfinite":
        z[7, 1, 1] = np.inf
    z = z.astype(np.float32)
    finite, same = _heights_scan(z)
    zw = np.ascontiguousarray(z.transpose(2, 1, 0)).reshape(W * H, D)
    assert (finite, same) == _heights_scan(zw, columns_first=True)
    assert finite == (kind != "nonfinite")
    assert same == (kind == "shared")
    if not finite:
        return
    exact = ex.geometry_host((z / np.float32(1e6))[None])
    fast = ex.geometry_host((z[:, :1, :1] / np.float32(1e6))[None]) if same else exact
    assert _geo_fields(fast)[:6] == _geo_fields(exact)[:6]
    assert fast.columns is None or np.array_equal(fast.columns, exact.columns)
