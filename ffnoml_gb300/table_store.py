"""On-disk store of the shape-constant tables of the FFNO3D path, so that a restarted process skips rebuilding them.

The tables (ffnoml_gb300.tables) depend only on the cube's plane shape and spacing, on the height column, and on the
frequency-MLP weights: the plane DFT tables (rfft / complex DFT / c2r along W and H), the Filon height transform and
its inverse, and every block's frequency-MLP outputs g(k), U(k), V(k) (models/ffno_model.py:346-392 for the
horizontal operator, :231-309 for the height operator). The reference recomputes them on every call of a layer;
here they are built once per process (Executor caches) and, with a TableStore, once per machine.

Entries are uncompressed .npz files named by the SHA-256 of the inputs that determine them (array bytes, shapes,
floats, the store version), written to a temporary file and renamed into place, so concurrent writers and an
interrupted write never leave a partial entry under its final name. An entry that fails to load is rebuilt and
rewritten. Per-column height tables (every column its own grid) are request data, not shape constants, and are not
stored.
"""
import hashlib
import os
import tempfile
import zipfile

import numpy as np
import torch

from . import tables as tb

VERSION = 1


def _digest_update(h, part):
    if isinstance(part, torch.Tensor):
        part = part.detach().cpu().numpy()
    if isinstance(part, np.ndarray):
        a = np.ascontiguousarray(part)
        h.update(f"nd{a.dtype.str}{a.shape}".encode())
        h.update(a.tobytes())
    elif isinstance(part, (tuple, list)):
        h.update(f"seq{len(part)}".encode())
        for p in part:
            _digest_update(h, p)
    elif isinstance(part, dict):
        h.update(f"map{len(part)}".encode())
        for k in sorted(part):
            h.update(str(k).encode())
            _digest_update(h, part[k])
    elif isinstance(part, float):
        h.update(b"f" + np.float64(part).tobytes())
    else:
        h.update(f"{type(part).__name__}:{part!r}".encode())


def digest(*parts):
    """SHA-256 hex digest of the parts (arrays and tensors by dtype, shape and bytes; floats bit-exactly)."""
    h = hashlib.sha256(f"ffnoml_gb300 tables v{VERSION}".encode())
    _digest_update(h, list(parts))
    return h.hexdigest()


class TableStore:
    """A directory of table entries: root/<kind>/<digest>.npz."""

    def __init__(self, root):
        self.root = os.path.abspath(os.fspath(root))
        os.makedirs(self.root, exist_ok=True)
        self.hits = 0
        self.builds = 0

    def path(self, kind, key):
        return os.path.join(self.root, kind, key + ".npz")

    def load(self, kind, key):
        try:
            with np.load(self.path(kind, key), allow_pickle=False) as z:
                return {k: z[k] for k in z.files}
        except (OSError, ValueError, EOFError, KeyError, zipfile.BadZipFile):
            return None

    def save(self, kind, key, arrays):
        d = os.path.join(self.root, kind)
        os.makedirs(d, exist_ok=True)
        fd, tmp = tempfile.mkstemp(prefix=key[:16] + ".", suffix=".tmp", dir=d)
        try:
            with os.fdopen(fd, "wb") as fh:
                np.savez(fh, **arrays)
            os.replace(tmp, self.path(kind, key))
        except BaseException:
            if os.path.exists(tmp):
                os.unlink(tmp)
            raise

    def fetch(self, kind, parts, build):
        """The entry for these parts: loaded if present and readable, else build() (a dict of arrays) saved."""
        key = digest(kind, *parts)
        arrays = self.load(kind, key)
        if arrays is not None:
            self.hits += 1
            return arrays
        arrays = {k: np.asarray(v) for k, v in build().items()}
        self.builds += 1
        self.save(kind, key, arrays)
        return arrays


class NoStore:
    """Build every time (no persistence)."""

    hits = 0
    builds = 0

    def fetch(self, kind, parts, build):
        self.builds += 1
        return {k: np.asarray(v) for k, v in build().items()}


def default_store():
    """A TableStore at $FFNO_GB300_TABLE_CACHE if that is set, else NoStore."""
    root = os.environ.get("FFNO_GB300_TABLE_CACHE")
    return TableStore(root) if root else NoStore()


def freq_key(freq_params):
    """Digest of the frequency-MLP parameters (name -> tensor) that determine g, U, V."""
    return digest({k: v for k, v in freq_params.items()})


# ------------------------------------------------------------------------------------------------ entries
def plane_arrays(store, H, W):
    """twf, thf, thi, twi of an H x W plane."""
    def build():
        twf, thf, thi, twi = tb.plane_dft(H, W)
        return dict(twf=twf, thf=thf, thi=thi, twi=twi)
    return store.fetch("plane", (int(H), int(W)), build)


def _freq_build(freq_params, op, features, rank, n_layers):
    out = {}
    for i in range(n_layers):
        g, u, v = tb.freq_tables(freq_params, f"blocks.{i}.{op}", features, rank)
        out[f"g{i}"] = g.numpy()
        if u is not None:
            out[f"u{i}"] = u.numpy()
            out[f"v{i}"] = v.numpy()
    return out


def plane_freq_arrays(store, freq_params, fkey, n_layers, rank, H, W, dx, dy):
    """Every block's horizontal g, U, V (g{i}, u{i}, v{i}) for an H x W plane with spacings dx, dy."""
    def build():
        return _freq_build(freq_params, "spec", tb.plane_features(H, W, dx, dy), rank, n_layers)
    return store.fetch("plane_freq", (fkey, int(n_layers), int(rank), int(H), int(W), float(dx), float(dy)), build)


def height_arrays(store, freq_params, fkey, n_layers, rank, column, length, k, feature_wavelength):
    """The shared-grid height transform (live, tzf, tzi) and every block's vertical g, U, V."""
    column = np.ascontiguousarray(column, dtype=np.float64)
    kk = k.detach().cpu().double().numpy() if isinstance(k, torch.Tensor) else np.asarray(k, np.float64)

    def build():
        live, tzf, tzi = tb.height_tables(column, length, k)
        feats = tb.height_features(k[:live], feature_wavelength)
        out = _freq_build(freq_params, "vertical", feats, rank, n_layers)
        out.update(live=np.asarray(live, np.int64), tzf=tzf, tzi=tzi)
        return out
    return store.fetch("height", (fkey, int(n_layers), int(rank), column, float(length), kk, float(feature_wavelength)),
                       build)


def freq_list(arrays, n_layers):
    """[(g, u, v)] per block as float64 tensors (u, v None without the low-rank term)."""
    t = lambda n: torch.from_numpy(arrays[n]) if n in arrays else None
    return [(t(f"g{i}"), t(f"u{i}"), t(f"v{i}")) for i in range(n_layers)]
