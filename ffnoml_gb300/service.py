"""Protocol-v2 FFNO service on one GB300 with continuous batching.

Wire protocol (ffno_fsdp_service.py:22, 156-343; FFNOInversion.jl/src/FSDPService.jl), unchanged:
  HELLO <token>\\n                          -> READY 2 <slots> <nmodels> FULL_SHARD_H_SLAB\\n
  PREDICT|VJP|JVP <name> nz nx ny L dx dy\\n + little-endian float32 arrays in Fortran order:
      features (6, nz, nx, ny) SI, z (nz, nx, ny) metres; VJP adds the population cotangent (nz, nx, ny, L),
      JVP the feature tangent (6, nz, nx, ny)
  -> OK <OP> nz nx ny L\\n + arrays: PREDICT populations (nz, nx, ny, L); VJP features_bar (6, nz, nx, ny) and
      z_bar (nz, nx, ny); JVP population tangent (nz, nx, ny, L)
  MEMORY\\n -> OK MEMORY <n>\\n + one line per GPU: host, local rank, peak allocated, reserved, total (bytes)
  SHUTDOWN\\n -> BYE\\n
A request that fails validation is answered with ERROR <message>\\n once its arrays have been read (as
ffno_batched_service.py:74-77 does), and the connection stays usable. A header whose sizes do not parse, or whose
arrays would exceed `max_request_bytes` (default: the host's physical memory), is answered with ERROR and the
connection is closed (its arrays are not read); so is a command line longer than 64 KiB.

Continuous batching: each connection has a reader that parses requests as they arrive and hands them to the scheduler
without waiting for earlier replies, and a writer that sends replies in request order. The scheduler admits requests
first-come first-served into `slots` GPU workers, each with its own CUDA stream, as long as the HBM their workspaces
need fits in the budget (free device memory at start x memory_fraction): requests of uneven sizes run concurrently and
their kernels overlap on the device. Weights and the shape-constant tables stay resident in the shared backends.
`slots` is reported as the world size in READY (at least 2, so the Julia client accepts the service).
"""
import collections
import hmac
import os
import queue
import socket
import threading
import time

import numpy as np
import torch

PROTOCOL_VERSION = 2
OPERATIONS = ("PREDICT", "VJP", "JVP")
MAX_LINE = 1 << 16


# ---------------------------------------------------------------------------------------------------- wire helpers
def read_exact(stream, count):
    buf = bytearray(count)
    view = memoryview(buf)
    off = 0
    while off < count:
        n = stream.recv_into(view[off:])
        if n == 0:
            raise EOFError("client disconnected during array transfer")
        off += n
    return bytes(buf)


def read_into(stream, view):
    """Fill a writable byte memoryview from the socket."""
    off, count = 0, len(view)
    while off < count:
        n = stream.recv_into(view[off:])
        if n == 0:
            raise EOFError("client disconnected during array transfer")
        off += n


def read_array(stream, shape):
    count = int(np.prod(shape))
    raw = read_exact(stream, count * 4)
    return np.frombuffer(raw, dtype="<f4").reshape(shape, order="F").copy()


def array_bytes(value):
    return np.asfortranarray(value, dtype="<f4").tobytes(order="F")


def readline(stream, limit=MAX_LINE):
    """One \\n-terminated line from a socket (bytes, without the terminator); b'' at end of stream. A line longer
    than `limit` bytes raises ConnectionError (no command of the protocol comes near it)."""
    out = bytearray()
    while True:
        ch = stream.recv(1)
        if not ch:
            return bytes(out) if out else b""
        if ch == b"\n":
            return bytes(out)
        if len(out) >= limit:
            raise ConnectionError("command line too long")
        out += ch


def request_bytes(op, nz, nx, ny, levels):
    """Bytes of the arrays that follow a request header."""
    per_voxel = 7 + {"PREDICT": 0, "VJP": levels, "JVP": 6}[op]
    return 4 * nz * nx * ny * per_voxel


def host_memory_bytes():
    try:
        return os.sysconf("SC_PAGE_SIZE") * os.sysconf("SC_PHYS_PAGES")
    except (ValueError, OSError, AttributeError):
        return 1 << 62


# ---------------------------------------------------------------------------------------------------- host buffers
class HostBuffers:
    """A pool of host float32 buffers for request and reply arrays: pinned (page-locked) when CUDA is available, so
    that the copy engine moves them without staging. A request's arrays are received straight into one buffer and
    a reply's arrays are sent straight from one, in the protocol's own layout; buffers are kept by size class (powers
    of two) for reuse, at most `keep` free ones a class."""

    def __init__(self, keep=4):
        self.keep = keep
        self.free = collections.defaultdict(list)
        self.lock = threading.Lock()
        self.pinned = torch.cuda.is_available()

    def acquire(self, n):
        size = 1 << max(20, (int(n) - 1).bit_length())
        with self.lock:
            if self.free[size]:
                return self.free[size].pop()
        return torch.empty(size, dtype=torch.float32, pin_memory=self.pinned)

    def release(self, buf):
        if buf is None:
            return
        with self.lock:
            if len(self.free[buf.numel()]) < self.keep:
                self.free[buf.numel()].append(buf)


def _bytes_view(buf, n):
    """The first n floats of a host buffer as a writable byte memoryview."""
    return memoryview(buf.numpy()[:n]).cast("B")


# ---------------------------------------------------------------------------------------------------- scheduling
class Request:
    """One request: its header fields and its arrays as received, back to back in a host buffer (wire layout:
    features (6, nz, nx, ny), z (nz, nx, ny), then the cotangent or tangent, each little-endian float32 in Fortran
    order)."""

    def __init__(self, op, name, shape, levels, dx, dy, buf, pool=None):
        self.op, self.name, self.shape, self.levels, self.dx, self.dy = op, name, shape, levels, dx, dy
        self.buf, self.pool = buf, pool
        self.done = threading.Event()
        self.reply = None            # bytes to send, or (header bytes, host buffer, float count)
        self.t_arrive = time.perf_counter()
        self.t_start = self.t_done = None

    @property
    def voxels(self):
        nz, nx, ny = self.shape
        return nz * nx * ny

    @property
    def arrays(self):
        """The request's arrays as numpy views (Fortran order) over its buffer."""
        nz, nx, ny = self.shape
        V = nz * nx * ny
        a = self.buf.numpy()
        out = [a[:6 * V].reshape((6, nz, nx, ny), order="F"), a[6 * V:7 * V].reshape((nz, nx, ny), order="F")]
        if self.op == "VJP":
            out.append(a[7 * V:(7 + self.levels) * V].reshape((nz, nx, ny, self.levels), order="F"))
        elif self.op == "JVP":
            out.append(a[7 * V:13 * V].reshape((6, nz, nx, ny), order="F"))
        return out

    def release(self):
        if self.pool is not None:
            self.pool.release(self.buf)
        self.buf = None

    def finish(self, reply):
        self.reply = reply
        self.t_done = time.perf_counter()
        self.done.set()


def workspace_bytes(op, voxels, width, levels):
    """Upper estimate of the device memory one request needs (activations, spectral buffers, VJP state), bytes."""
    per_voxel = 4 * width * {"PREDICT": 22, "VJP": 48, "JVP": 42}[op] + 4 * (20 + 3 * levels)
    return int(voxels * per_voxel * 1.25) + (64 << 20)


class Scheduler:
    """FIFO admission into `slots` GPU workers under an HBM budget."""

    def __init__(self, backends, slots=4, memory_fraction=0.8, budget_bytes=None, device=None, pool=None):
        self.backends = backends
        self.pool = pool
        self.slots = max(1, int(slots))
        # a VJP recomputes each block in its backward: its workspace stays within the admission estimate while
        # other requests run beside it
        for b in backends.values():
            model = getattr(b, "model", None)
            if model is not None and hasattr(model, "executor"):
                model.executor().cache_states = False
        self.device = torch.device(device or "cuda")
        if self.device.type == "cuda" and self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        self.failed = None               # a worker's setup error, reported to every request from then on
        if budget_bytes is None:
            free, _ = torch.cuda.mem_get_info(self.device)
            budget_bytes = int(free * memory_fraction)
        self.cuda = self.device.type == "cuda"
        self.budget = int(budget_bytes)
        self.in_flight = 0
        self.cv = threading.Condition()
        self.pending = collections.deque()
        self.stop = False
        self.completed = []
        self.workers = [threading.Thread(target=self._worker, args=(i,), daemon=True) for i in range(self.slots)]
        for w in self.workers:
            w.start()

    def submit(self, req):
        with self.cv:
            self.pending.append(req)
            self.cv.notify_all()

    def _cost(self, req):
        b = self.backends.get(req.name)
        width = b.model.width if b is not None else 64
        return min(workspace_bytes(req.op, req.voxels, width, req.levels), self.budget)

    def _take(self):
        with self.cv:
            while True:
                if self.stop and not self.pending:
                    return None, 0
                if self.pending:
                    req = self.pending[0]
                    cost = self._cost(req)
                    if self.in_flight + cost <= self.budget or self.in_flight == 0:
                        self.pending.popleft()
                        self.in_flight += cost
                        return req, cost
                self.cv.wait(0.05)

    def _release(self, cost):
        with self.cv:
            self.in_flight -= cost
            self.cv.notify_all()

    def _worker(self, index):
        import contextlib
        try:
            if self.cuda:
                torch.cuda.set_device(self.device)
                stream = torch.cuda.Stream(self.device)
            ctx = (lambda: torch.cuda.stream(stream)) if self.cuda else contextlib.nullcontext
        except Exception as exc:
            self.failed = exc
            ctx = None
        while True:
            req, cost = self._take()
            if req is None:
                return
            req.t_start = time.perf_counter()
            try:
                if ctx is None:
                    raise RuntimeError(f"service slot unavailable: {self.failed}")
                with ctx():
                    reply = execute(self.backends, req, self.pool)
            except Exception as exc:  # reported to the client, the service stays up
                reply = f"ERROR {type(exc).__name__}: {exc}".replace("\n", " ").encode() + b"\n"
            finally:
                self._release(cost)
                req.release()
            req.finish(reply)
            with self.cv:
                self.completed.append(req)

    def close(self):
        with self.cv:
            self.stop = True
            self.cv.notify_all()
        for w in self.workers:
            w.join(timeout=30)


def execute(backends, req, pool=None):
    """Run one request on the current stream; returns the reply: bytes, or (header bytes, host buffer, float count)
    when the backend takes the wire layout (GB300Backend.*_wire: the arrays are reordered on the device, so the host
    neither transposes nor copies them)."""
    if req.name not in backends:
        raise KeyError(f"unknown model {req.name!r}")
    backend = backends[req.name]
    if req.levels != len(backend.level_names):
        raise ValueError("request level count differs from the model")
    nz, nx, ny = req.shape
    head = f"OK {req.op} {nz} {nx} {ny} {req.levels}\n".encode()
    wire = getattr(backend, req.op.lower() + "_wire", None)
    if wire is not None and pool is not None:
        V = nz * nx * ny
        out = pool.acquire(7 * V if req.op == "VJP" else req.levels * V)
        try:
            n = wire(req.buf, req.shape, req.dx, req.dy, out)
        except BaseException:
            pool.release(out)
            raise
        return head, out, n
    if req.op == "PREDICT":
        pop = backend.predict_local(req.arrays[0], req.arrays[1], req.dx, req.dy)
        return head + array_bytes(pop)
    if req.op == "VJP":
        out = backend.vjp_local(req.arrays[0], req.arrays[1], req.dx, req.dy, req.arrays[2])
        return head + array_bytes(out["features"]) + array_bytes(out["z_scale"])
    pop_dot = backend.jvp_local(req.arrays[0], req.arrays[1], req.dx, req.dy, req.arrays[2])
    return head + array_bytes(pop_dot)


# ---------------------------------------------------------------------------------------------------- server
class Server:
    """The protocol-v2 server. backends: name -> object with predict_local / vjp_local / level_names / model."""

    def __init__(self, backends, token, host="127.0.0.1", port=0, slots=4, memory_fraction=0.8, budget_bytes=None,
                 device=None, log=None, max_request_bytes=None):
        self.backends = dict(backends)
        self.token = str(token)
        self.max_request_bytes = int(max_request_bytes or host_memory_bytes())
        self.slots = max(2, int(slots))
        self.pool = HostBuffers()
        self.scheduler = Scheduler(self.backends, self.slots, memory_fraction, budget_bytes, device, self.pool)
        self.listener = socket.socket(socket.AF_INET, socket.SOCK_STREAM)
        self.listener.setsockopt(socket.SOL_SOCKET, socket.SO_REUSEADDR, 1)
        self.listener.bind((host, int(port)))
        self.listener.listen(8)
        self.port = self.listener.getsockname()[1]
        self.log = log or (lambda msg: None)
        self.peak = 0
        self._stop = threading.Event()
        self._threads = []

    def serve_forever(self):
        self.log(f"FFNO_GB300_SERVICE_LISTENING port={self.port} slots={self.slots} models={','.join(self.backends)}")
        self.listener.settimeout(0.2)
        while not self._stop.is_set():
            try:
                conn, addr = self.listener.accept()
            except socket.timeout:
                continue
            except OSError:
                break
            t = threading.Thread(target=self._connection, args=(conn,), daemon=True)
            t.start()
            self._threads.append(t)
        self.scheduler.close()

    def start(self):
        t = threading.Thread(target=self.serve_forever, daemon=True)
        t.start()
        return t

    def shutdown(self):
        self._stop.set()
        try:
            self.listener.close()
        except OSError:
            pass

    def _memory_reply(self):
        dev = self.scheduler.device
        if dev.type != "cuda":
            return f"OK MEMORY 1\n{socket.gethostname()} 0 0 0 0\n".encode()
        free, total = torch.cuda.mem_get_info(dev)
        peak = max(self.peak, torch.cuda.max_memory_allocated(dev))
        line = f"{socket.gethostname()} {dev.index or 0} {peak} {torch.cuda.memory_reserved(dev)} {total}\n"
        self.peak = 0
        torch.cuda.reset_peak_memory_stats(dev)
        return f"OK MEMORY 1\n{line}".encode()

    def _connection(self, conn):
        conn.setsockopt(socket.IPPROTO_TCP, socket.TCP_NODELAY, 1)
        replies = queue.Queue()

        def writer():
            while True:
                item = replies.get()
                if item is None:
                    return
                if isinstance(item, Request):
                    item.done.wait()
                    data = item.reply
                else:
                    data = item
                try:
                    if isinstance(data, tuple):          # header, then the arrays straight from the host buffer
                        head, buf, n = data
                        try:
                            conn.sendall(head)
                            conn.sendall(_bytes_view(buf, n))
                        finally:
                            self.pool.release(buf)
                    else:
                        conn.sendall(data)
                except OSError:
                    return

        wt = threading.Thread(target=writer, daemon=True)
        wt.start()
        try:
            hello = readline(conn).decode(errors="replace").split()
            if len(hello) != 2 or hello[0] != "HELLO" or not hmac.compare_digest(hello[1].encode(),
                                                                                   self.token.encode()):
                conn.sendall(b"ERROR invalid handshake\n")
                return
            conn.sendall(f"READY {PROTOCOL_VERSION} {self.slots} {len(self.backends)} FULL_SHARD_H_SLAB\n".encode())
            while True:
                line = readline(conn)
                if not line:
                    break
                fields = line.decode(errors="replace").strip().split()
                if not fields:
                    continue
                op = fields[0]
                if op == "SHUTDOWN":
                    replies.put(b"BYE\n")
                    self.shutdown()
                    break
                if op == "MEMORY":
                    replies.put(self._memory_reply())
                    continue
                if op not in OPERATIONS or len(fields) != 8:
                    replies.put(f"ERROR invalid command: {' '.join(fields)}\n".encode())
                    continue
                _, name, nz, nx, ny, levels, dx, dy = fields
                try:
                    nz, nx, ny, levels = int(nz), int(nx), int(ny), int(levels)
                    dx, dy = float(dx), float(dy)
                    if min(nz, nx, ny, levels) < 1:
                        raise ValueError("sizes must be positive")
                    nbytes = request_bytes(op, nz, nx, ny, levels)
                    if nbytes > self.max_request_bytes:
                        raise ValueError(f"request arrays of {nbytes} bytes exceed the limit of "
                                         f"{self.max_request_bytes}")
                except ValueError as exc:
                    replies.put(f"ERROR invalid command: {exc}\n".encode())
                    break                                   # the arrays' length is unknown: the stream is lost
                n = nbytes // 4
                buf = self.pool.acquire(n)
                try:
                    read_into(conn, _bytes_view(buf, n))
                except BaseException:
                    self.pool.release(buf)
                    raise
                req = Request(op, name, (nz, nx, ny), levels, dx, dy, buf, self.pool)
                replies.put(req)
                self.scheduler.submit(req)
        except (EOFError, ConnectionError, OSError):
            pass
        finally:
            replies.put(None)
            wt.join(timeout=600)
            try:
                conn.close()
            except OSError:
                pass


# ---------------------------------------------------------------------------------------------------- client
class Client:
    """A minimal protocol-v2 client (what FFNOInversion.jl's FSDPService.jl speaks), for tests and the benchmark."""

    def __init__(self, port, token, host="127.0.0.1", timeout=120):
        self.sock = socket.create_connection((host, port), timeout=timeout)
        self.sock.setsockopt(socket.IPPROTO_TCP, socket.TCP_NODELAY, 1)
        self.sock.sendall(f"HELLO {token}\n".encode())
        self.ready = readline(self.sock).decode().split()
        if not self.ready or self.ready[0] != "READY":
            raise RuntimeError(f"handshake failed: {self.ready}")

    def send(self, op, name, features, z, dx, dy, levels, extra=None):
        nz, nx, ny = z.shape
        msg = f"{op} {name} {nz} {nx} {ny} {levels} {dx} {dy}\n".encode()
        msg += array_bytes(features) + array_bytes(z)
        if extra is not None:
            msg += array_bytes(extra)
        self.sock.sendall(msg)

    def receive(self, op, shape, levels):
        head = readline(self.sock).decode().split()
        if not head or head[0] != "OK":
            raise RuntimeError(" ".join(head))
        nz, nx, ny = shape
        if op == "PREDICT":
            return read_array(self.sock, (nz, nx, ny, levels))
        if op == "VJP":
            return {"features": read_array(self.sock, (6, nz, nx, ny)), "z_scale": read_array(self.sock, (nz, nx, ny))}
        return read_array(self.sock, (nz, nx, ny, levels))

    def request(self, op, name, features, z, dx, dy, levels, extra=None):
        self.send(op, name, features, z, dx, dy, levels, extra)
        return self.receive(op, z.shape, levels)

    @staticmethod
    def encode(op, name, features, z, dx, dy, levels, extra=None):
        """A request's bytes (header and arrays), for a client that sends the same request many times."""
        nz, nx, ny = z.shape
        msg = f"{op} {name} {nz} {nx} {ny} {levels} {dx} {dy}\n".encode() + array_bytes(features) + array_bytes(z)
        return msg + (array_bytes(extra) if extra is not None else b"")

    def request_raw(self, msg, reply_bytes, into=None):
        """Send encoded request bytes; return the reply's header fields, its arrays' bytes read into `into` (a
        writable buffer of at least reply_bytes, reused by the caller)."""
        self.sock.sendall(msg)
        head = readline(self.sock).decode().split()
        if not head or head[0] != "OK":
            raise RuntimeError(" ".join(head))
        view = memoryview(into if into is not None else bytearray(reply_bytes))[:reply_bytes]
        read_into(self.sock, view)
        return head

    def memory(self):
        self.sock.sendall(b"MEMORY\n")
        head = readline(self.sock).decode().split()
        return [readline(self.sock).decode().split() for _ in range(int(head[2]))]

    def shutdown(self):
        self.sock.sendall(b"SHUTDOWN\n")
        reply = readline(self.sock).decode()
        self.sock.close()
        return reply

    def close(self):
        self.sock.close()


def main():
    """python -m ffnoml_gb300.service manifest.toml — the manifest of ffno_fsdp_service.py ([service] port, token,
    bind_host; [[models]] name, checkpoint_path, level_names, factory_kwargs), plus optional [service] slots,
    table_cache (a directory where the shape-constant tables persist across restarts) and max_request_bytes."""
    import argparse
    import tomllib

    from .factory import create_ffno3d
    from .runtime import GB300Backend
    from .table_store import TableStore

    ap = argparse.ArgumentParser()
    ap.add_argument("manifest")
    ap.add_argument("--precision", default=os.environ.get("FFNO_GB300_PRECISION", "bf16"), choices=["fp32", "bf16"])
    args = ap.parse_args()
    with open(args.manifest, "rb") as fh:
        cfg = tomllib.load(fh)
    svc = cfg["service"]
    store = TableStore(svc["table_cache"]) if svc.get("table_cache") else None
    backends = {}
    for m in sorted(cfg["models"], key=lambda item: item["name"]):
        b = GB300Backend.from_checkpoint(m["checkpoint_path"], create_ffno3d, m["level_names"],
                                         m.get("factory_kwargs", {}))
        b.model.set_precision(args.precision)
        if store is not None:
            b.model.executor().tables = store
        backends[str(m["name"])] = b
    server = Server(backends, svc["token"], svc.get("bind_host", "0.0.0.0"), int(svc["port"]),
                    slots=int(svc.get("slots", 4)), log=lambda s: print(s, flush=True),
                    max_request_bytes=svc.get("max_request_bytes"))
    server.serve_forever()


if __name__ == "__main__":
    main()
