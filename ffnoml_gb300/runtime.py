"""Single-GPU persistent backend: the drop-in for DistributedFSDPBackend's predict_local / vjp_local
(ffno_fsdp_runtime.py:81-348) with the same argument meaning, units, layouts and errors, on one GB300.

Arrays cross the host boundary as numpy float32 in the service's layouts: features (6, nz, nx, ny) in SI (T [K],
vx, vy, vz [m/s], log10 ne [m^-3], log10 rho [kg m^-3]), z (nz, nx, ny) in metres, populations (nz, nx, ny, L) in
m^-3. The model sees D = nz, H = nx, W = ny. Weights and tables stay resident; host<->device copies go through
pinned staging buffers that are reused per shape.
"""
import hashlib
import os
import threading
import warnings
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

import numpy as np
import torch

from . import _native as nat
from .executor import _stream

INPUT_CHANNELS = ("temperature", "vx", "vy", "vz", "log10_ne", "log10_rho")


def _numpy_globals():
    """numpy's array/dtype/scalar reconstruction functions and classes, for the weights-only unpickler (checkpoints
    whose normalisation statistics or metadata hold numpy values)."""
    found = []
    for mod_name, names in (("numpy._core.multiarray", ("_reconstruct", "scalar")),
                            ("numpy.core.multiarray", ("_reconstruct", "scalar")),
                            ("numpy", ("ndarray", "dtype"))):
        try:
            mod = __import__(mod_name, fromlist=list(names))
        except ImportError:
            continue
        found += [getattr(mod, n) for n in names if hasattr(mod, n)]
    found += [getattr(np.dtypes, n) for n in dir(getattr(np, "dtypes", object)) if n.endswith("DType")]
    return [g for g in found if g is not None]


def load_checkpoint(path, map_location="cpu"):
    """The training checkpoint dict (model_state, normalization_stats, io_metadata), as the reference's
    train_utils.load_checkpoint (train_utils.py:20-92) loads it: weights-only, then weights-only with numpy's
    reconstruction types allowed, and only then a full unpickle, with a warning (load only trusted checkpoints)."""
    try:
        return torch.load(path, map_location=map_location, weights_only=True)
    except Exception:
        pass
    safe = getattr(torch.serialization, "safe_globals", None)
    if safe is not None:
        try:
            with safe(_numpy_globals()):
                return torch.load(path, map_location=map_location, weights_only=True)
        except Exception:
            pass
    warnings.warn(f"checkpoint {path} cannot be loaded weights-only; falling back to torch.load(weights_only=False), "
                  "which runs the file's pickled code: load only trusted checkpoints", RuntimeWarning, stacklevel=2)
    return torch.load(path, map_location=map_location, weights_only=False)


_POOL = None
_POOL_LOCK = threading.Lock()


def _host_copy(dst, src):
    """dst[...] = src for large host arrays, in chunks on a few threads (numpy releases the GIL while copying)."""
    if not dst.flags.c_contiguous or dst.dtype != np.float32 or dst.size != np.size(src):
        raise ValueError("host copy needs a C-contiguous float32 destination of the source's size")
    d, v = dst.reshape(-1), np.ascontiguousarray(src, dtype=np.float32).reshape(-1)
    n = d.size
    parts = min(_THREADS, os.cpu_count() or 1, max(1, n >> 20))      # pieces of at least 4 MB
    if parts <= 1:
        np.copyto(d, v)
        return
    step = -(-n // parts)
    futures = [_pool().submit(np.copyto, d[i:i + step], v[i:i + step]) for i in range(0, n, step)]
    for f in futures:
        f.result()


_THREADS = 16      # host threads for copies and scans of request arrays (one GB300 node's Grace has 72 cores)


def _pool():
    global _POOL
    with _POOL_LOCK:
        if _POOL is None:
            _POOL = ThreadPoolExecutor(max_workers=_THREADS, thread_name_prefix="ffno-host-copy")
    return _POOL


def _heights_scan(z, columns_first=False):
    """(every height finite, every column equal to column (0, 0)) of float32 heights: z (D, H, W), or with
    columns_first z (N, D), one column a row (the wire layout). In chunks on a few threads (numpy releases the GIL
    inside the comparisons)."""
    if columns_first:
        zr = z.reshape(z.shape[0], -1)         # [N][D]: chunks of columns against the first
        ref = lambda a, b: zr[:1]
    else:
        zr = z.reshape(z.shape[0], -1)         # [D][HW]: chunks of depths against column 0 at those depths
        ref = lambda a, b: zr[a:b, :1]

    def scan(a, b):
        part = zr[a:b]
        return bool(np.isfinite(part).all()), bool((part == ref(a, b)).all())

    n = zr.shape[0]
    parts = min(_THREADS, os.cpu_count() or 1, max(1, zr.size >> 20), n)
    if parts <= 1:
        return scan(0, n)
    step = -(-n // parts)
    res = [f.result() for f in [_pool().submit(scan, a, min(n, a + step)) for a in range(0, n, step)]]
    return all(r[0] for r in res), all(r[1] for r in res)


def _check(flags, what):
    f = int(flags)
    if f & 1:
        raise ValueError(f"{what} contains NaN or Inf")
    if f & 2:
        raise ValueError(f"{what} temperature must be positive")
    if f & 4:
        raise RuntimeError("FFNO returned non-positive or non-finite populations")
    if f & 8:
        raise RuntimeError("FFNO VJP returned NaN or Inf")


class GB300Backend:
    """One resident FFNO3D on one GPU.

    GB300Backend(model, level_names, normalization=None): model is an ffnoml_gb300.FFNO3D (moved to the device here);
    normalization (mean_X, std_X, mean_Y, std_Y) defaults to the model's buffers. from_checkpoint builds it from a
    training checkpoint the way DistributedFSDPBackend does (ffno_fsdp_runtime.py:116-165)."""

    def __init__(self, model, level_names, normalization=None, device="cuda", name="model"):
        if not torch.cuda.is_available():
            raise RuntimeError("the GB300 backend requires CUDA")
        self.device = torch.device(device)
        self.model = model.to(self.device).eval()
        self.level_names = tuple(str(v) for v in level_names)
        if len(self.level_names) != model.out_channels:
            raise RuntimeError("checkpoint Cout differs from configured level_names")
        norm = normalization or {k: getattr(model, k).detach().cpu().numpy() for k in
                                 ("mean_X", "std_X", "mean_Y", "std_Y")}
        f = lambda k: torch.as_tensor(np.asarray(norm[k], dtype=np.float32), device=self.device).contiguous()
        self.mean_x, self.std_x, self.mean_y, self.std_y = f("mean_X"), f("std_X"), f("mean_Y"), f("std_Y")
        if torch.any(self.std_x <= 0) or torch.any(self.std_y <= 0):
            raise RuntimeError("checkpoint normalization standard deviations must be positive")
        self.name = name
        self.call_count = 0
        self._local = threading.local()       # staging buffers and flags per calling thread (service slots)

    @property
    def _flags(self):
        """This thread's status words on the device: [0] the request's inputs, [1] the results."""
        loc = self._local
        if not hasattr(loc, "flags"):
            loc.flags = torch.zeros(2, dtype=torch.int32, device=self.device)
        return loc.flags

    def _out_flags(self):
        return self._flags.data_ptr() + 4

    def _guarded(self, fn):
        """Run the model part of a call; if it fails on a request whose inputs are invalid, report the inputs."""
        try:
            return fn()
        except Exception:
            torch.cuda.current_stream().synchronize()
            _check(self._flags.tolist()[0], "FFNO request")
            raise

    def _finish(self):
        """Wait for the call's work; raise on invalid inputs; return the results' status word."""
        torch.cuda.current_stream().synchronize()
        req, out = self._flags.tolist()
        _check(req, "FFNO request")
        return out

    @property
    def _staging(self):
        loc = self._local
        if not hasattr(loc, "staging"):
            loc.staging = {}
        return loc.staging

    @classmethod
    def from_checkpoint(cls, checkpoint_path, factory, level_names, factory_kwargs=None, device="cuda"):
        ck = load_checkpoint(checkpoint_path)
        norm, io = ck.get("normalization_stats"), ck.get("io_metadata")
        if norm is None or io is None:
            raise RuntimeError("checkpoint must contain normalization_stats and io_metadata")
        if int(io["Cin"]) != len(INPUT_CHANNELS):
            raise RuntimeError(f"checkpoint Cin={io['Cin']} does not match {INPUT_CHANNELS}")
        model = factory(Cin=int(io["Cin"]), Cout=int(io["Cout"]), device="cpu", **dict(factory_kwargs or {}))
        model.load_state_dict(ck["model_state"], strict=True)
        backend = cls(model, level_names, normalization=norm, device=device)
        backend.checkpoint_hash = hashlib.sha256(Path(checkpoint_path).read_bytes()).hexdigest()
        return backend

    def describe(self):
        return {"backend": "gb300_single_gpu", "input_channels": INPUT_CHANNELS, "level_names": self.level_names,
                "device": str(self.device), "world_size": 1,
                "full_parameter_count": sum(p.numel() for p in self.model.parameters()),
                "output_representation": "linear_population_m3", "precision": self.model.precision}

    # ------------------------------------------------------------------------------------------------ staging
    def _stage(self, key, shape):
        """(pinned host buffer, device buffer) of this shape, reused across calls."""
        k = (key, tuple(shape))
        if k not in self._staging:
            host = torch.empty(shape, dtype=torch.float32, pin_memory=True)
            dev = torch.empty(shape, dtype=torch.float32, device=self.device)
            self._staging[k] = (host, dev)
        return self._staging[k]

    def _dev_buffer(self, key, n):
        """A device float32 buffer of n values for this thread, grown as needed and reused across calls."""
        t = self._staging.get(("dev", key))
        if t is None or t.numel() < n:
            t = torch.empty(max(n, 5 * (0 if t is None else t.numel()) // 4), dtype=torch.float32, device=self.device)
            self._staging[("dev", key)] = t
        return t[:n]

    def _upload(self, key, array):
        """A device copy of a host array: the array is copied into this thread's pinned buffer on several host
        threads, then to the device by the copy engine. (A copy straight from the caller's pageable memory measured
        slower per call on a GB300 node: 15 against 3 ms for a request's 117 MB of inputs.)"""
        host, dev = self._stage(key, array.shape)
        _host_copy(host.numpy(), array)
        dev.copy_(host, non_blocking=True)
        return dev

    def _download(self, key, tensor):
        """Queue the copy of a result into this thread's pinned buffer for it (reused across calls)."""
        host, _ = self._stage(key + "_out", tensor.shape)
        host.copy_(tensor, non_blocking=True)
        return host

    @staticmethod
    def _result(host):
        """A fresh numpy copy of a pinned result buffer (the buffer is reused by the next call). The fresh array's
        pages are first written here, on several host threads; a device copy straight into it would fault them in
        one at a time inside the copy."""
        out = np.empty(tuple(host.shape), dtype=np.float32)
        _host_copy(out, host.numpy())
        return out

    def _validate(self, features, z_scale):
        features = np.asarray(features, dtype=np.float32)
        z_scale = np.asarray(z_scale, dtype=np.float32)
        if features.ndim != 4 or features.shape[0] != len(INPUT_CHANNELS):
            raise ValueError("local features must have shape (6,nz,nx_local,ny)")
        if tuple(features.shape[1:]) != tuple(z_scale.shape):
            raise ValueError("local z_scale must have shape (nz,nx_local,ny)")
        return features, z_scale

    def _prepare(self, features, z_scale):
        nz, nx, ny = z_scale.shape
        V = nz * nx * ny
        # the heights' analysis from the host copy, in the device's float32 values (z / 1e6 with IEEE division, as
        # ffno_si_inputs computes it), so that the model's stream is not synchronised to read it back. Columns equal
        # in metres are equal in Mm, so when every column equals column (0, 0) only that column is divided; otherwise
        # the analysis runs on the divided heights. (Heights that are not finite are left to the device path, which
        # reports them through the request's flags.)
        found = []
        scan = threading.Thread(target=lambda: found.append(self._scan_heights(z_scale)), daemon=True)
        scan.start()                     # beside the uploads' host copies
        try:
            f_dev = self._upload("features", features)
            z_dev = self._upload("z", z_scale)
        finally:
            scan.join()
        if not found:
            raise RuntimeError("the heights' analysis failed")
        self._local.geo = found[0]
        x = torch.empty(1, 6, nz, nx, ny, dtype=torch.float32, device=self.device)
        zmm = torch.empty(1, nz, nx, ny, dtype=torch.float32, device=self.device)
        self._flags.zero_()
        # the request's status word is read once with the results (_finish): no synchronisation before the model
        nat.call("ffno_si_inputs", f_dev.data_ptr(), z_dev.data_ptr(), V, self.mean_x.data_ptr(),
                 self.std_x.data_ptr(), x.data_ptr(), zmm.data_ptr(), self._flags.data_ptr(), _stream())
        return f_dev, x, zmm, V

    def _scan_heights(self, z_scale):
        """The geometry of heights z_scale (D, H, W) in metres (None if any is not finite)."""
        finite, same = _heights_scan(z_scale)
        ex = self.model.executor()
        if not finite:
            geo = None
        elif same:
            geo = ex.geometry_host((z_scale[:, :1, :1] / np.float32(1e6))[None])
        else:
            geo = ex.geometry_host((z_scale / np.float32(1e6))[None])
        return geo

    # ------------------------------------------------------------------------------------------------ wire layout
    # The service's arrays are little-endian float32 in Fortran order (ffno_fsdp_service.py:219-322). The *_wire
    # methods take a request's arrays as they arrived, back to back in one host buffer (pinned, for the copy engine),
    # and write the reply's arrays in that order into `out`: no host-side transpose or copy; the layouts change on the
    # device (ffno_reverse_axes4: Fortran order is the C order of the reversed shape). They validate like their
    # *_local twins and raise the same errors.
    def _wire_in(self, buf, shape, n_extra):
        """Device arrays of a request buffer [6V features | V z | n_extra V]: the model's SI features [6][V], z [V]
        (C order) and the extra array [V][n_extra] (a cotangent (nz, nx, ny, L)) or [n_extra][V] (a feature
        tangent), with the host geometry of the heights."""
        nz, nx, ny = shape
        V = nz * nx * ny
        n = V * (7 + n_extra)
        if buf.numel() < n:
            raise ValueError("request buffer shorter than its arrays")
        raw = self._dev_buffer("wire_in", n)
        raw.copy_(buf[:n], non_blocking=True)
        s = _stream()
        f = torch.empty(6, V, dtype=torch.float32, device=self.device)
        z = torch.empty(V, dtype=torch.float32, device=self.device)
        nat.call("ffno_reverse_axes4", raw.data_ptr(), ny, nx, nz, 6, f.data_ptr(), s)
        nat.call("ffno_reverse_axes4", raw.data_ptr() + 24 * V, 1, ny, nx, nz, z.data_ptr(), s)
        extra = None
        if n_extra:
            extra = torch.empty(n_extra * V, dtype=torch.float32, device=self.device)
            src = raw.data_ptr() + 28 * V
            if n_extra == 6:    # a feature tangent (6, nz, nx, ny)
                nat.call("ffno_reverse_axes4", src, ny, nx, nz, 6, extra.data_ptr(), s)
            else:               # a population cotangent (nz, nx, ny, L)
                nat.call("ffno_reverse_axes4", src, n_extra, ny, nx, nz, extra.data_ptr(), s)
        # the heights' analysis on the host, in the device's float32 values: the wire z is [ny][nx][nz], columns
        # contiguous, column (0, 0) first
        zraw = buf[6 * V:7 * V].numpy().reshape(ny * nx, nz)
        finite, same = _heights_scan(zraw, columns_first=True)
        ex = self.model.executor()
        if not finite:
            geo = None
        elif same:      # every column equals column (0, 0) in metres, so in Mm too: only that column is divided
            geo = ex.geometry_columns((zraw[:1] / np.float32(1e6))[None], None)
        else:
            zw = zraw.reshape(ny, nx, nz) / np.float32(1e6)
            geo = ex.geometry_columns(zw.reshape(1, ny * nx, nz),
                                      lambda: zw.transpose(1, 0, 2).reshape(1, nx * ny, nz).astype(np.float64))
        return f, z, extra, geo, V

    def _wire_model_inputs(self, f, z, V, shape):
        nz, nx, ny = shape
        x = torch.empty(1, 6, nz, nx, ny, dtype=torch.float32, device=self.device)
        zmm = torch.empty(1, nz, nx, ny, dtype=torch.float32, device=self.device)
        self._flags.zero_()
        nat.call("ffno_si_inputs", f.data_ptr(), z.data_ptr(), V, self.mean_x.data_ptr(), self.std_x.data_ptr(),
                 x.data_ptr(), zmm.data_ptr(), self._flags.data_ptr(), _stream())
        return x, zmm

    def _wire_out(self, arrays, out):
        """Device arrays (each with its C-order shape, reversed into Fortran order on the device) -> out (host),
        back to back."""
        total = sum(a.numel() for a, _ in arrays)
        if out.numel() < total:
            raise ValueError("reply buffer shorter than the reply's arrays")
        dev = self._dev_buffer("wire_out", total)
        off = 0
        for a, shape in arrays:
            s0, s1, s2, s3 = shape
            nat.call("ffno_reverse_axes4", a.data_ptr(), s0, s1, s2, s3, dev.data_ptr() + 4 * off, _stream())
            off += a.numel()
        out[:total].copy_(dev, non_blocking=True)

    def predict_wire(self, buf, shape, dx, dy, out):
        """PREDICT on a request buffer [features | z] in wire layout: populations (nz, nx, ny, L) in wire layout into
        out. Returns the number of floats written."""
        f, z, _, geo, V = self._wire_in(buf, shape, 0)
        x, zmm = self._wire_model_inputs(f, z, V, shape)
        L = self.model.out_channels
        ex, errs = self.model.executor(), []
        with torch.no_grad():
            y = self._guarded(lambda: ex.forward(x, zmm, float(dx), float(dy), geo=geo, errs=errs)[0])
        pop = torch.empty(V, L, dtype=torch.float32, device=self.device)
        nat.call("ffno_si_populations", y.data_ptr(), V, L, self.mean_y.data_ptr(), self.std_y.data_ptr(),
                 pop.data_ptr(), self._out_flags(), _stream())
        self._wire_out([(pop, (shape[0], shape[1], shape[2], L))], out)
        _check(self._finish(), "FFNO output")
        ex.check_flags(errs)
        self.call_count += 1
        return V * L

    def vjp_wire(self, buf, shape, dx, dy, out):
        """VJP on a request buffer [features | z | population cotangent] in wire layout: features_bar (6, nz, nx, ny)
        then z_bar (nz, nx, ny) in wire layout into out. Returns the number of floats written."""
        L = self.model.out_channels
        f, z, cot, geo, V = self._wire_in(buf, shape, L)
        x, zmm = self._wire_model_inputs(f, z, V, shape)
        ex = self.model.executor()
        y, state = self._guarded(lambda: ex.forward(x, zmm, float(dx), float(dy), keep=True, geo=geo))
        ybar = torch.empty_like(y)
        nat.call("ffno_si_population_cotangent", y.data_ptr(), cot.data_ptr(), V, L, self.mean_y.data_ptr(),
                 self.std_y.data_ptr(), ybar.data_ptr(), self._out_flags(), _stream())
        errs = []
        xbar, zbar = self._guarded(lambda: ex.backward(state, ybar, errs=errs))
        fbar = torch.empty(6, V, dtype=torch.float32, device=self.device)
        zbar_m = torch.empty(V, dtype=torch.float32, device=self.device)
        nat.call("ffno_si_input_grads", f.data_ptr(), xbar.data_ptr(), zbar.data_ptr(), V, self.std_x.data_ptr(),
                 fbar.data_ptr(), zbar_m.data_ptr(), self._out_flags(), _stream())
        nz, nx, ny = shape
        self._wire_out([(fbar, (6, nz, nx, ny)), (zbar_m, (1, nz, nx, ny))], out)
        flags = self._finish()
        if flags & 1:
            raise ValueError("FFNO VJP cotangent contains NaN or Inf")
        _check(flags, "FFNO VJP")
        ex.check_flags(errs)
        self.call_count += 1
        return 7 * V

    def jvp_wire(self, buf, shape, dx, dy, out):
        """JVP on a request buffer [features | z | feature tangent] in wire layout: the population tangent
        (nz, nx, ny, L) in wire layout into out. Returns the number of floats written."""
        f, z, tangent, _, V = self._wire_in(buf, shape, 6)
        x, zmm = self._wire_model_inputs(f, z, V, shape)
        x_dot = torch.empty_like(x)
        nat.call("ffno_si_input_tangent", f.data_ptr(), tangent.data_ptr(), V, self.std_x.data_ptr(),
                 x_dot.data_ptr(), self._out_flags(), _stream())
        y, y_dot = self._guarded(lambda: self.model.executor().jvp(x, zmm, float(dx), float(dy), x_dot))
        L = self.model.out_channels
        pop_dot = torch.empty(V, L, dtype=torch.float32, device=self.device)
        nat.call("ffno_si_population_tangent", y.data_ptr(), y_dot.data_ptr(), V, L, self.mean_y.data_ptr(),
                 self.std_y.data_ptr(), pop_dot.data_ptr(), self._out_flags(), _stream())
        self._wire_out([(pop_dot, (shape[0], shape[1], shape[2], L))], out)
        flags = self._finish()
        if flags & 1:
            raise ValueError("FFNO JVP tangent contains NaN or Inf")
        if flags & 8:
            raise RuntimeError("FFNO JVP returned NaN or Inf")
        _check(flags, "FFNO JVP")
        self.call_count += 1
        return V * L

    # ------------------------------------------------------------------------------------------------ API
    def predict_local(self, features, z_scale, dx, dy):
        """(6,nz,nx,ny) SI features, (nz,nx,ny) heights [m] -> (nz,nx,ny,L) populations [m^-3]
        (ffno_fsdp_runtime.py:294-304)."""
        features, z_scale = self._validate(features, z_scale)
        _, x, zmm, V = self._prepare(features, z_scale)
        L = self.model.out_channels
        ex, errs = self.model.executor(), []
        with torch.no_grad():
            y = self._guarded(lambda: ex.forward(x, zmm, float(dx), float(dy), geo=self._local.geo, errs=errs)[0])
        pop = torch.empty(*z_scale.shape, L, dtype=torch.float32, device=self.device)
        nat.call("ffno_si_populations", y.data_ptr(), V, L, self.mean_y.data_ptr(), self.std_y.data_ptr(),
                 pop.data_ptr(), self._out_flags(), _stream())
        host = self._download("pop", pop)
        _check(self._finish(), "FFNO output")
        ex.check_flags(errs)
        self.call_count += 1
        return self._result(host)

    def jvp_local(self, features, z_scale, dx, dy, feature_tangent):
        """Forward-mode derivative of the populations along feature_tangent (6,nz,nx,ny) in the SI units of features
        (the heights stay fixed): (nz,nx,ny,L) in m^-3 (ffno_fsdp_runtime.py:350-372). FP32 whatever the model's
        precision."""
        features, z_scale = self._validate(features, z_scale)
        tangent = np.asarray(feature_tangent, dtype=np.float32)
        if tangent.shape != features.shape:
            raise ValueError(f"local feature_tangent has shape {tangent.shape}; expected {features.shape}")
        if not np.isfinite(tangent).all():
            raise ValueError("FFNO JVP tangent contains NaN or Inf")
        f_dev, x, zmm, V = self._prepare(features, z_scale)
        t_dev = self._upload("tangent", tangent)
        x_dot = torch.empty_like(x)
        nat.call("ffno_si_input_tangent", f_dev.data_ptr(), t_dev.data_ptr(), V, self.std_x.data_ptr(),
                 x_dot.data_ptr(), self._out_flags(), _stream())
        y, y_dot = self._guarded(lambda: self.model.executor().jvp(x, zmm, float(dx), float(dy), x_dot))
        L = self.model.out_channels
        pop_dot = torch.empty(*z_scale.shape, L, dtype=torch.float32, device=self.device)
        nat.call("ffno_si_population_tangent", y.data_ptr(), y_dot.data_ptr(), V, L, self.mean_y.data_ptr(),
                 self.std_y.data_ptr(), pop_dot.data_ptr(), self._out_flags(), _stream())
        host = self._download("pop_dot", pop_dot)
        flags = self._finish()
        if flags & 1:
            raise ValueError("FFNO JVP tangent contains NaN or Inf")
        if flags & 8:
            raise RuntimeError("FFNO JVP returned NaN or Inf")
        _check(flags, "FFNO JVP")
        self.call_count += 1
        return self._result(host)

    def vjp_local(self, features, z_scale, dx, dy, population_cotangent):
        """Input VJP along the population cotangent (nz,nx,ny,L): {"features": (6,nz,nx,ny), "z_scale": (nz,nx,ny)}
        per SI unit (ffno_fsdp_runtime.py:306-348)."""
        features, z_scale = self._validate(features, z_scale)
        cot = np.asarray(population_cotangent, dtype=np.float32)
        L = self.model.out_channels
        expected = tuple(z_scale.shape) + (L,)
        if tuple(cot.shape) != expected:
            raise ValueError(f"local population_cotangent has shape {cot.shape}; expected {expected}")
        f_dev, x, zmm, V = self._prepare(features, z_scale)
        # the cotangent is not needed before the forward: its host copy into pinned staging runs on another thread
        # while the forward does
        cot_host, cot_dev = self._stage("cot", cot.shape)
        copier = threading.Thread(target=_host_copy, args=(cot_host.numpy(), cot), daemon=True)
        copier.start()
        ex = self.model.executor()
        try:
            y, state = self._guarded(lambda: ex.forward(x, zmm, float(dx), float(dy), keep=True,
                                                        geo=self._local.geo))
        finally:
            copier.join()
        cot_dev.copy_(cot_host, non_blocking=True)
        ybar = torch.empty_like(y)
        nat.call("ffno_si_population_cotangent", y.data_ptr(), cot_dev.data_ptr(), V, L, self.mean_y.data_ptr(),
                 self.std_y.data_ptr(), ybar.data_ptr(), self._out_flags(), _stream())
        errs = []
        xbar, zbar = self._guarded(lambda: ex.backward(state, ybar, errs=errs))
        fbar = torch.empty(6, *z_scale.shape, dtype=torch.float32, device=self.device)
        zbar_m = torch.empty(*z_scale.shape, dtype=torch.float32, device=self.device)
        nat.call("ffno_si_input_grads", f_dev.data_ptr(), xbar.data_ptr(), zbar.data_ptr(), V,
                 self.std_x.data_ptr(), fbar.data_ptr(), zbar_m.data_ptr(), self._out_flags(), _stream())
        hf, hz = self._download("fbar", fbar), self._download("zbar", zbar_m)
        flags = self._finish()
        if flags & 1:
            raise ValueError("FFNO VJP cotangent contains NaN or Inf")
        _check(flags, "FFNO VJP")
        ex.check_flags(errs)
        self.call_count += 1
        return {"features": self._result(hf), "z_scale": self._result(hz)}
