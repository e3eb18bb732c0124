"""The on-disk store of shape-constant tables: entries reload bit-exactly, a second process (a fresh store on the
same directory) builds nothing, keys follow every input that determines a table, and unreadable entries are rebuilt."""
import multiprocessing as mp
import os

import numpy as np
import torch

from ffnoml_gb300 import table_store as ts
from ffnoml_gb300 import tables as tb


def _model():
    from ffnoml_gb300 import create_ffno3d
    torch.manual_seed(0)
    m = create_ffno3d(6, 12, atoms=["H", "CA"], width=16, n_layers=2, hidden_spectral=16, hidden_vertical=16)
    with torch.no_grad():
        for n, p in m.named_parameters():
            if "freq_u" in n:
                p.normal_(0, 0.1)
    return m


def _params(m):
    return {k: v.detach().cpu() for k, v in m.state_dict().items() if ".freq_" in k}


def test_plane_freq_round_trip_and_restart(tmp_path):
    m = _model()
    fp = _params(m)
    fk = ts.freq_key(fp)
    a = ts.TableStore(tmp_path)
    t1 = ts.plane_freq_arrays(a, fp, fk, m.n_layers, m.freq_mix_rank, 24, 20, 48e3, 40e3)
    assert a.builds == 1 and a.hits == 0
    # a fresh store on the same directory (a restarted process) loads the entry and builds nothing
    b = ts.TableStore(tmp_path)
    t2 = ts.plane_freq_arrays(b, fp, fk, m.n_layers, m.freq_mix_rank, 24, 20, 48e3, 40e3)
    assert b.builds == 0 and b.hits == 1
    assert sorted(t1) == sorted(t2)
    for k in t1:
        assert t1[k].dtype == t2[k].dtype and np.array_equal(t1[k], t2[k])
    # and the entry equals the tables built directly
    feats = tb.plane_features(24, 20, 48e3, 40e3)
    for i, (g, u, v) in enumerate(ts.freq_list(t2, m.n_layers)):
        g0, u0, v0 = tb.freq_tables(fp, f"blocks.{i}.spec", feats, m.freq_mix_rank)
        assert torch.equal(g, g0) and torch.equal(u, u0) and torch.equal(v, v0)


def test_keys_follow_every_input(tmp_path):
    m = _model()
    fp = _params(m)
    fk = ts.freq_key(fp)
    s = ts.TableStore(tmp_path)
    args = (m.n_layers, m.freq_mix_rank, 16, 16, 48e3, 48e3)
    ts.plane_freq_arrays(s, fp, fk, *args)
    ts.plane_freq_arrays(s, fp, fk, *args)
    assert (s.builds, s.hits) == (1, 1)
    ts.plane_freq_arrays(s, fp, fk, m.n_layers, m.freq_mix_rank, 16, 16, 48e3, 48e3 * (1 + 2 ** -40))  # spacing
    ts.plane_freq_arrays(s, fp, fk, m.n_layers, m.freq_mix_rank, 16, 18, 48e3, 48e3)                   # shape
    fp2 = {k: (v + 1e-7 if "freq_mlp.0.bias" in k else v) for k, v in fp.items()}
    ts.plane_freq_arrays(s, fp2, ts.freq_key(fp2), *args)                                            # weights
    assert s.builds == 4


def test_height_entry_and_plane_entry(tmp_path):
    m = _model()
    fp = _params(m)
    fk = ts.freq_key(fp)
    s = ts.TableStore(tmp_path)
    z = np.linspace(14.0, -1.0, 40)
    col = z - z.min()
    length, k = tb.height_box(15.0, m.z_reference_length, m.z_min_wavelength, 9)
    h1 = ts.height_arrays(s, fp, fk, m.n_layers, m.freq_mix_rank, col, length, k, m.z_feature_wavelength)
    h2 = ts.height_arrays(ts.TableStore(tmp_path), fp, fk, m.n_layers, m.freq_mix_rank, col, length, k,
                          m.z_feature_wavelength)
    live, tzf, tzi = tb.height_tables(col, length, k)
    assert int(h2["live"]) == live and np.array_equal(h2["tzf"], tzf) and np.array_equal(h2["tzi"], tzi)
    assert all(np.array_equal(h1[n], h2[n]) for n in h1)
    p = ts.plane_arrays(s, 12, 10)
    for n, ref in zip(("twf", "thf", "thi", "twi"), tb.plane_dft(12, 10)):
        assert np.array_equal(p[n], ref)


def test_unreadable_entry_is_rebuilt(tmp_path):
    s = ts.TableStore(tmp_path)
    ts.plane_arrays(s, 8, 8)
    key = ts.digest("plane", 8, 8)
    path = s.path("plane", key)
    with open(path, "wb") as fh:
        fh.write(b"not a zip")
    s2 = ts.TableStore(tmp_path)
    p = ts.plane_arrays(s2, 8, 8)
    assert s2.builds == 1 and np.array_equal(p["twf"], tb.plane_dft(8, 8)[0])
    assert ts.TableStore(tmp_path).load("plane", key) is not None     # rewritten whole


def _writer(root, n):
    s = ts.TableStore(root)
    for _ in range(n):
        ts.plane_arrays(s, 10, 6)


def test_concurrent_writers_leave_whole_entries(tmp_path):
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_writer, args=(str(tmp_path), 3)) for _ in range(3)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    d = os.path.join(str(tmp_path), "plane")
    assert [f for f in os.listdir(d) if f.endswith(".tmp")] == []
    got = ts.TableStore(tmp_path).load("plane", ts.digest("plane", 10, 6))
    assert got is not None and np.array_equal(got["thi"], tb.plane_dft(10, 6)[2])


def test_no_store_builds_every_time():
    s = ts.NoStore()
    ts.plane_arrays(s, 8, 8)
    ts.plane_arrays(s, 8, 8)
    assert s.builds == 2
