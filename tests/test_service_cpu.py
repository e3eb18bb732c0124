"""The protocol-v2 service on the CPU with a fake backend: handshake, PREDICT / VJP / MEMORY / SHUTDOWN framing in
Fortran order, ERROR replies that keep the connection usable, request pipelining and in-order replies, and
concurrent admission from two connections (replies in order per connection)."""
import threading
import time

import numpy as np
import pytest

from ffnoml_gb300.service import Client, Server


class FakeModel:
    width = 16


class FakeBackend:
    """predict: populations[z, x, y, l] = sum of the features at the voxel + l; vjp: features_bar = cotangent sum."""

    def __init__(self, levels=6, delay=0.0):
        self.level_names = tuple(f"l{i}" for i in range(levels))
        self.model = FakeModel()
        self.delay = delay
        self.calls = []

    def _check(self, features, z):
        if not np.isfinite(features).all():
            raise ValueError("FFNO request contains NaN or Inf")

    def predict_local(self, features, z, dx, dy):
        self._check(features, z)
        self.calls.append(("PREDICT", time.perf_counter()))
        time.sleep(self.delay)
        base = features.sum(axis=0) + z + dx * 0 + dy * 0
        return np.stack([base + l for l in range(len(self.level_names))], axis=-1).astype(np.float32)

    def vjp_local(self, features, z, dx, dy, cot):
        self._check(features, z)
        time.sleep(self.delay)
        s = cot.sum(axis=-1)
        return {"features": np.broadcast_to(s, features.shape).astype(np.float32) * 2, "z_scale": s.astype(np.float32)}

    def jvp_local(self, features, z, dx, dy, tangent):
        self._check(features, z)
        base = tangent.sum(axis=0)
        return np.stack([base * (l + 1) for l in range(len(self.level_names))], axis=-1).astype(np.float32)


def _server(backend, slots=2):
    srv = Server({"H": backend}, "tok", port=0, slots=slots, budget_bytes=1 << 40, device="cpu")
    srv.start()
    return srv


def _inputs(shape, seed):
    g = np.random.default_rng(seed)
    return g.normal(size=(6,) + shape).astype(np.float32), g.normal(size=shape).astype(np.float32)


def test_handshake_predict_vjp_memory_shutdown():
    srv = _server(FakeBackend())
    c = Client(srv.port, "tok")
    assert c.ready[:2] == ["READY", "2"] and int(c.ready[2]) >= 2 and c.ready[4] == "FULL_SHARD_H_SLAB"
    f, z = _inputs((3, 4, 5), 0)
    pop = c.request("PREDICT", "H", f, z, 48e3, 48e3, 6)
    assert pop.shape == (3, 4, 5, 6)
    assert np.allclose(pop[..., 2], f.sum(0) + z + 2, atol=1e-5)
    cot = np.ones((3, 4, 5, 6), np.float32)
    out = c.request("VJP", "H", f, z, 48e3, 48e3, 6, cot)
    assert np.allclose(out["z_scale"], 6.0) and np.allclose(out["features"], 12.0)
    assert len(c.memory()) == 1
    assert c.shutdown().strip() == "BYE"


def test_errors_keep_the_connection_usable():
    srv = _server(FakeBackend())
    c = Client(srv.port, "tok")
    f, z = _inputs((2, 2, 2), 1)
    bad = f.copy()
    bad[0, 0, 0, 0] = np.nan
    c.send("PREDICT", "H", bad, z, 1.0, 1.0, 6)
    with pytest.raises(RuntimeError, match="NaN"):
        c.receive("PREDICT", z.shape, 6)
    c.send("PREDICT", "nope", f, z, 1.0, 1.0, 6)
    with pytest.raises(RuntimeError, match="unknown model"):
        c.receive("PREDICT", z.shape, 6)
    c.send("PREDICT", "H", f, z, 1.0, 1.0, 12)
    with pytest.raises(RuntimeError, match="level count"):
        c.receive("PREDICT", z.shape, 12)
    c.sock.sendall(b"FROB\n")
    assert "invalid command" in c.sock.recv(100).decode()
    assert c.request("PREDICT", "H", f, z, 1.0, 1.0, 6).shape == (2, 2, 2, 6)
    c.shutdown()


def test_handshake_token_is_checked():
    srv = _server(FakeBackend())
    with pytest.raises(RuntimeError):
        Client(srv.port, "wrong")
    srv.shutdown()


def test_pipelined_requests_reply_in_order():
    srv = _server(FakeBackend(delay=0.05), slots=3)
    c = Client(srv.port, "tok")
    shapes = [(2, 3, 4), (5, 2, 2), (1, 1, 7), (4, 4, 1)]
    inputs = [_inputs(s, i) for i, s in enumerate(shapes)]
    for f, z in inputs:
        c.send("PREDICT", "H", f, z, 1.0, 1.0, 6)
    for (f, z), s in zip(inputs, shapes):
        pop = c.receive("PREDICT", s, 6)
        assert pop.shape == s + (6,) and np.allclose(pop[..., 0], f.sum(0) + z, atol=1e-5)
    c.shutdown()


def test_two_connections_run_concurrently():
    backend = FakeBackend(delay=0.3)
    srv = _server(backend, slots=2)
    results = {}

    def run(key, seed):
        c = Client(srv.port, "tok")
        f, z = _inputs((2, 2, 2), seed)
        results[key] = (c.request("PREDICT", "H", f, z, 1.0, 1.0, 6), f, z)
        c.close()

    t0 = time.perf_counter()
    ts = [threading.Thread(target=run, args=(k, k)) for k in range(2)]
    [t.start() for t in ts]
    [t.join() for t in ts]
    elapsed = time.perf_counter() - t0
    assert elapsed < 0.55                               # the two 0.3 s requests overlapped
    for pop, f, z in results.values():
        assert np.allclose(pop[..., 1], f.sum(0) + z + 1, atol=1e-5)
    srv.shutdown()


def test_jvp_request_round_trip():
    srv = _server(FakeBackend())
    c = Client(srv.port, "tok")
    f, z = _inputs((3, 4, 5), 4)
    t = np.random.default_rng(5).normal(size=f.shape).astype(np.float32)
    got = c.request("JVP", "H", f, z, 48e3, 48e3, 6, t)
    assert got.shape == (3, 4, 5, 6)
    np.testing.assert_allclose(got[..., 2], 3 * t.sum(axis=0), rtol=1e-6)
    c.close()
    srv.shutdown()


def _raw(port):
    import socket
    s = socket.create_connection(("127.0.0.1", port), timeout=30)
    return s, s.makefile("rb")


def test_oversized_request_is_refused_before_its_arrays():
    srv = Server({"H": FakeBackend()}, "tok", port=0, slots=2, budget_bytes=1 << 40, device="cpu",
                 max_request_bytes=1 << 20)
    srv.start()
    s, rd = _raw(srv.port)
    s.sendall(b"HELLO tok\n")
    assert rd.readline().startswith(b"READY 2")
    s.sendall(b"PREDICT H 1000 1000 1000 6 1.0 1.0\n")   # 28 GB of arrays announced: refused, connection closed
    line = rd.readline()
    assert line.startswith(b"ERROR") and b"exceed the limit" in line
    assert rd.readline() == b""
    s.close()
    c = Client(srv.port, "tok")                          # the server keeps serving other connections
    f, z = _inputs((4, 3, 2), 5)
    assert c.request("PREDICT", "H", f, z, 1.0, 1.0, 6).shape == (4, 3, 2, 6)
    c.close()
    srv.shutdown()


def test_endless_command_line_closes_the_connection():
    srv = _server(FakeBackend())
    s, rd = _raw(srv.port)
    s.sendall(b"HELLO tok\n")
    assert rd.readline().startswith(b"READY 2")
    try:
        s.sendall(b"A" * (1 << 17))
    except OSError:
        pass                                             # the server may close while the line is still arriving
    try:
        assert rd.readline() == b""                      # closed (or reset: the rest of the line was never read)
    except ConnectionResetError:
        pass
    s.close()
    srv.shutdown()


def test_handshake_with_undecodable_bytes_is_refused():
    srv = _server(FakeBackend())
    s, rd = _raw(srv.port)
    s.sendall(b"HELLO \xff\xfe\n")
    assert rd.readline().startswith(b"ERROR invalid handshake")
    s.close()
    srv.shutdown()
