"""Host-RAM streaming forward of FFNO3D, for cubes whose activations do not fit in HBM (the reference's
BatchedFFNOBackend, ffno_batched_backend.py:116-308).

Every operation of the model is local, acts on depth planes, or acts on columns, so it can run over slabs of the cube
without changing the operator (ffno_batched_backend.py:1-13): the lift, gates, branch post-MLPs, fusion, pw / mlp and
the head over depth slabs; the horizontal spectral convolution over depth slabs (each plane's rfft2 / mixing / irfft2
is its own); the height operator over row slabs [D][h0:h1][W] (each column alone). The hidden states live in pinned
host memory, channels last like the device layout; slabs move with strided copies (ffno_copy2d) on two copy streams,
pipelined over two device buffer sets so that one slab's copies overlap another's kernels. A depth-weighted
GroupNorm gathers every slab's partial statistics (the kernels' per-CTA Chan partials, FP64) into one buffer and
finalizes once, so the statistics are those of the whole cube; its application is folded into the next stage's
kernels as in the resident executor, so each GroupNorm costs no extra pass over the cube.

The kernels are the resident path's (split-BF16 tensor cores or FP32, as the model's precision says). Host buffers:
four hidden states (x, and three rotating buffers for the branch / fusion / pw / mlp intermediates). Shared height
grids only (per-column grids raise NotImplementedError). Forward only, as in the reference.
"""
import copy

import numpy as np
import torch

from . import _native as nat
from .executor import EPS, Workspace, _descs, _stream
from .runtime import INPUT_CHANNELS, _check, _host_copy


def _pinned(n):
    return torch.empty(n, dtype=torch.float32, pin_memory=True)


def _record(stream):
    e = torch.cuda.Event()
    e.record(stream)
    return e


class StreamingForward:
    """FFNO3D forward of one cube held in host memory, `chunk_depth` depth planes and `chunk_rows` rows of columns at
    a time on the device (ffno_batched_backend.py:117-145 takes the same two chunk sizes)."""

    def __init__(self, model, chunk_depth=16, chunk_rows=16, normalization=None):
        if chunk_depth < 1 or chunk_rows < 1:
            raise ValueError("chunk sizes must be positive")
        self.model = model
        # mean_X, std_X, mean_Y, std_Y (a checkpoint's normalization_stats; default: the model's buffers)
        self.normalization = normalization
        self.ex = model.executor()
        self.chunk_depth = int(chunk_depth)
        self.chunk_rows = int(chunk_rows)
        self.slabs = 0          # device slabs processed by the last call

    # ------------------------------------------------------------------------------------------------ helpers
    def _view(self, ws, V):
        """ws's buffers for a smaller cube of V voxels (prefixes of the same buffers)."""
        if V == ws.V:
            return ws
        w = copy.copy(ws)
        w.V = V
        w.nparts = nat.lib().ffno_stats_parts(V)
        w.nparts_tc = nat.lib().ffno_tc_parts(V)
        w.coefs = dict(ws.coefs)
        return w

    def _h2d(self, dst, src, offset, n):
        """n floats of pinned host tensor src from element offset into device tensor dst."""
        dst.view(-1)[:n].copy_(src[offset:offset + n], non_blocking=True)

    def _d2h(self, dst, offset, src, n):
        dst[offset:offset + n].copy_(src.reshape(-1)[:n], non_blocking=True)

    def _rows(self, dst, dpitch, src, spitch, width, rows):
        nat.call("ffno_copy2d", dst, dpitch, src, spitch, width, rows, _stream())

    def _stats(self, ws, tc):
        """Append this slab's GroupNorm partials to the cube's list."""
        P = ws.nparts_tc if tc else ws.nparts
        n = P * self.G * 3
        self.parts[self.npart * self.G * 3:(self.npart + P) * self.G * 3].copy_(ws.partials[:n])
        self.npart += P

    def _finalize(self, name, gamma, beta):
        nat.call("ffno_gn_finalize", self.parts.data_ptr(), self.npart, self.C, self.G, gamma.data_ptr(),
                 beta.data_ptr(), EPS, self.coefs[name].data_ptr(), self.gstats[name].data_ptr(), _stream())
        self.npart = 0

    def _depth_slabs(self):
        for d0 in range(0, self.D, self.chunk_depth):
            yield d0, min(self.D, d0 + self.chunk_depth)

    def _row_slabs(self):
        for h0 in range(0, self.H, self.chunk_rows):
            yield h0, min(self.H, h0 + self.chunk_rows)

    def _load(self, ws, names, d0, d1, hosts):
        """Depth slab d0:d1 of host hidden states into the named workspace buffers."""
        n = (d1 - d0) * self.HW * self.C
        for name, h in zip(names, hosts):
            self._h2d(getattr(ws, name), h, d0 * self.HW * self.C, n)

    def _store(self, ws, names, d0, d1, hosts):
        n = (d1 - d0) * self.HW * self.C
        for name, h in zip(names, hosts):
            self._d2h(h, d0 * self.HW * self.C, getattr(ws, name), n)

    def _run(self, items, make, load, compute, store):
        """One stage over its slabs, pipelined over two device buffer sets: the host -> device copies of slab k (on
        the h2d stream) overlap the kernels of slab k-1 (the current stream) and the device -> host copies of slab
        k-2 (the d2h stream); events order every reuse of a buffer set, and the stage ends with the current stream
        waiting for its last copy back, so the next stage (and a GroupNorm finalize) sees whole host buffers."""
        comp = torch.cuda.current_stream()
        self.h2d.wait_event(_record(comp))
        free = [None, None]
        for k, item in enumerate(items):
            b = k & 1
            ws = make(b, item)
            self.slabs += 1
            with torch.cuda.stream(self.h2d):
                if free[b] is not None:
                    self.h2d.wait_event(free[b])
                if load is not None:
                    load(ws, item)
                loaded = _record(self.h2d)
            comp.wait_event(loaded)
            compute(ws, item)
            done = _record(comp)
            with torch.cuda.stream(self.d2h):
                self.d2h.wait_event(done)
                if store is not None:
                    store(ws, item)
                free[b] = _record(self.d2h)
        comp.wait_event(_record(self.d2h))

    def _buffers(self, dev, D, H, W, C, L, cd):
        """Pinned host hidden states and device inputs, kept while the cube shape repeats (pinning GBs of host
        memory costs more than a forward)."""
        key = (str(dev), D, H, W, C, L, cd)
        if getattr(self, "_bufs_key", None) != key:
            self._bufs = None
            V = D * H * W
            self._bufs = dict(X=_pinned(V * C), A=_pinned(V * C), B=_pinned(V * C), F=_pinned(V * C),
                              pop=_pinned(V * L), f_in=_pinned(6 * V), z_in=_pinned(V),
                              xn=torch.empty(6, V, dtype=torch.float32, device=dev),
                              zmm=torch.empty(1, D, H, W, dtype=torch.float32, device=dev),
                              xs=torch.empty(6, cd * H * W, dtype=torch.float32, device=dev))
            self._bufs_key = key
        return self._bufs

    # ------------------------------------------------------------------------------------------------ forward
    def __call__(self, features, z_m, dx, dy, log10=False):
        """SI features (6, D, H, W) and heights z_m (D, H, W) in metres (host arrays) -> populations (D, H, W, L)
        in m^-3 (numpy), as BatchedFFNOBackend.predict_si (ffno_batched_backend.py:285-308); with log10, the
        de-normalised log10 populations (L, D, H, W) as its predict_log10 (:251-283)."""
        m, ex = self.model, self.ex
        features = np.ascontiguousarray(features, dtype=np.float32)
        z_m = np.ascontiguousarray(z_m, dtype=np.float32)
        if features.ndim != 4 or features.shape[0] != len(INPUT_CHANNELS) or features.shape[1:] != z_m.shape:
            raise ValueError(f"expected features (6,D,H,W) and z (D,H,W), got {features.shape}, {z_m.shape}")
        dev = next(m.parameters()).device
        D, H, W = z_m.shape
        C, L = m.width, m.out_channels
        self.D, self.H, self.W, self.HW, self.C = D, H, W, H * W, C
        V = D * H * W
        s = _stream()
        pk = ex.packed(dev)
        self.G = pk.groups
        src = self.normalization or {k: getattr(m, k).detach().cpu().numpy() for k in
                                     ("mean_X", "std_X", "mean_Y", "std_Y")}
        norm = {k: torch.as_tensor(np.asarray(src[k], dtype=np.float32), device=dev).contiguous() for k in
                ("mean_X", "std_X", "mean_Y", "std_Y")}
        flags = torch.zeros(1, dtype=torch.int32, device=dev)
        # normalised inputs [6][V] and heights [V] (Mm) stay on the device (7 floats a voxel against C of a hidden
        # state); converted slab by slab from the pinned host arrays by the resident path's kernel
        cd, cr = min(self.chunk_depth, D), min(self.chunk_rows, H)
        bufs = self._buffers(dev, D, H, W, C, L, cd)
        # the request into pinned buffers kept with the hidden states (pinning on every call costs more than copying)
        f_host, zm_host = bufs["f_in"], bufs["z_in"]
        _host_copy(f_host.numpy(), features)
        _host_copy(zm_host.numpy(), z_m)
        xn, zmm, xs = bufs["xn"], bufs["zmm"], bufs["xs"]
        fs = torch.empty(6, cd * H * W, dtype=torch.float32, device=dev)
        zin = torch.empty(cd * H * W, dtype=torch.float32, device=dev)
        for d0, d1 in self._depth_slabs():
            Vs, o = (d1 - d0) * self.HW, d0 * self.HW
            self._rows(fs.data_ptr(), Vs * 4, f_host.data_ptr() + o * 4, V * 4, Vs * 4, 6)
            self._h2d(zin, zm_host, o, Vs)
            nat.call("ffno_si_inputs", fs.data_ptr(), zin.data_ptr(), Vs, norm["mean_X"].data_ptr(),
                     norm["std_X"].data_ptr(), xs.data_ptr(), zmm.view(-1)[o:].data_ptr(), flags.data_ptr(), s)
            self._rows(xn.data_ptr() + o * 4, V * 4, xs.data_ptr(), Vs * 4, Vs * 4, 6)
        torch.cuda.current_stream().synchronize()
        _check(flags.item(), "FFNO streaming request")
        del fs, zin
        geo = ex.geometry(zmm)
        if not geo.shared:
            raise NotImplementedError("the streaming forward runs shared height grids")
        hgt = ex.height(pk, geo, dev)
        pln, pfr = ex.plane(H, W, dev), ex.plane_freq(pk, H, W, float(dx), float(dy), dev)
        live = hgt["live"]
        dw = torch.empty(V, dtype=torch.float32, device=dev)
        nat.call("ffno_depth_weights", zmm.data_ptr(), D, H * W, dw.data_ptr(), s)
        # host hidden states, two device buffer sets per slab kind (the copies of one slab overlap the kernels of
        # the other), the copy streams
        X, A, B, F, pop_host = bufs["X"], bufs["A"], bufs["B"], bufs["F"], bufs["pop"]
        key = (cd, cr, live)
        if bufs.get("ws_key") != key:
            bufs["wsd"] = bufs["wsr"] = None
            bufs["wsd"] = [Workspace(cd, H, W, C, live, self.G, dev) for _ in range(2)]
            bufs["wsr"] = [Workspace(D, cr, W, C, live, self.G, dev) for _ in range(2)]
            bufs["ws_key"] = key
        wsd, wsr = bufs["wsd"], bufs["wsr"]
        for w in wsd + wsr:
            w.err.zero_()
        if getattr(self, "h2d", None) is None or self.h2d.device != dev:
            self.h2d, self.d2h = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
        nslab = max(-(-D // cd), -(-H // cr))
        maxp = max(wsd[0].partials.numel(), wsr[0].partials.numel()) // (self.G * 3)
        self.parts = torch.empty(nslab * maxp * self.G * 3, dtype=torch.float64, device=dev)
        self.npart = 0
        self.coefs = {n: torch.empty(3 * C, dtype=torch.float32, device=dev) for n in ("lift",) + _NORMS}
        self.gstats = {n: torch.empty(self.G * 3, dtype=torch.float64, device=dev) for n in ("lift",) + _NORMS}
        self.slabs = 0
        depth = list(self._depth_slabs())

        def slab_inputs(d0, d1):
            """Normalised model inputs of depth slab d0:d1, contiguous [6][Vs] (in xs; the current stream)."""
            Vs = (d1 - d0) * self.HW
            self._rows(xs.data_ptr(), Vs * 4, xn.data_ptr() + d0 * self.HW * 4, V * 4, Vs * 4, 6)
            return xs

        def depth_ws(b, it):
            ws = self._view(wsd[b], (it[1] - it[0]) * self.HW)
            ws.buf = b
            ws.dw = dw[it[0] * self.HW:it[1] * self.HW]
            for n in self.coefs:
                ws.coefs[n] = self.coefs[n]
            return ws

        def row_ws(b, it):
            rows = it[1] - it[0]
            ws = self._view(wsr[b], D * rows * W)
            ws.dw = dw.view(D, H, W)[:, it[0]:it[1]].contiguous().view(-1)
            ws.zr = zmm.view(D, H, W)[:, it[0]:it[1]].contiguous()
            for n in self.coefs:
                ws.coefs[n] = self.coefs[n]
            return ws

        # lift: pre-activation and statistics, then GELU(GN(.)) into X
        def lift(ws, it):
            x = slab_inputs(*it)
            nat.call("ffno_lift_fwd", x.data_ptr(), m.in_channels, ws.V, C, pk.lift_w.data_ptr(), ws.dw.data_ptr(),
                     ws.pre.data_ptr(), ws.partials.data_ptr(), ws.nparts, self.G, _stream())
            self._stats(ws, False)

        self._run(depth, depth_ws, None, lift, lambda ws, it: self._store(ws, ["pre"], it[0], it[1], [A]))
        self._finalize("lift", pk.lift_g, pk.lift_b)

        def act(ws, it):
            nat.call("ffno_gn_act", ws.pre.data_ptr(), self.coefs["lift"].data_ptr(), ws.V, C, 1, ws.x.data_ptr(),
                     _stream())

        self._run(depth, depth_ws, lambda ws, it: self._load(ws, ["pre"], it[0], it[1], [A]), act,
                  lambda ws, it: self._store(ws, ["x"], it[0], it[1], [X]))
        for i in range(m.n_layers):
            self._block(pk, i, depth_ws, row_ws, hgt, pln, pfr[i], X, A, B, F)

        # head, and the SI populations (or log10 n) of each slab, one output buffer per buffer set
        outs = [torch.empty(L, cd * H * W, dtype=torch.float32, device=dev) for _ in range(2)]
        pops = [torch.empty(cd * H * W, L, dtype=torch.float32, device=dev) for _ in range(2)]

        def head(ws, it):
            b = ws.buf
            x = slab_inputs(*it)
            y = outs[b].view(-1)[:L * ws.V].view(L, ws.V)      # the head writes [L][Vs] contiguously
            ex._head(pk, ws.x, x, y, ws.err, ws.V)
            if log10:   # y std_Y + mean_Y
                torch.addcmul(norm["mean_Y"][:, None], y, norm["std_Y"][:, None],
                              out=pops[b].view(-1)[:L * ws.V].view(L, ws.V))
            else:
                nat.call("ffno_si_populations", y.data_ptr(), ws.V, L, norm["mean_Y"].data_ptr(),
                         norm["std_Y"].data_ptr(), pops[b].data_ptr(), flags.data_ptr(), _stream())

        def head_out(ws, it):
            b = ws.buf
            if log10:   # rows of [L][V]
                self._rows(pop_host.data_ptr() + it[0] * self.HW * 4, V * 4, pops[b].data_ptr(), ws.V * 4, ws.V * 4,
                           L)
            else:
                self._d2h(pop_host, it[0] * self.HW * L, pops[b], ws.V * L)

        self._run(depth, depth_ws, lambda ws, it: self._load(ws, ["x"], it[0], it[1], [X]), head, head_out)
        torch.cuda.current_stream().synchronize()
        _check(flags.item(), "FFNO streaming output")
        if any(int(w.err.item()) for w in wsd + wsr):
            raise RuntimeError("tensor-core kernel timed out")
        out = np.empty((L, D, H, W) if log10 else (D, H, W, L), dtype=np.float32)
        _host_copy(out, pop_host.numpy()[:V * L])
        return out

    # ------------------------------------------------------------------------------------------------ one block
    def _block(self, pk, i, depth_ws, row_ws, hgt, pln, fq, X, A, B, F):
        ex = self.ex
        C, D, H, W, HW, Wf = self.C, self.D, self.H, self.W, self.HW, self.W // 2 + 1
        bp = pk.blocks[i]
        live = hgt["live"]
        tc = ex._tc()
        r_f, r_pw, r_mlp = bp["res"]
        depth = list(self._depth_slabs())
        ld = lambda names, hosts: (lambda ws, it: self._load(ws, names, it[0], it[1], hosts))
        st = lambda names, hosts: (lambda ws, it: self._store(ws, names, it[0], it[1], hosts))

        # horizontal spectral branch over depth slabs -> spec_pre (A)
        def spectral(ws, it):
            s, Ds = _stream(), it[1] - it[0]
            if tc:
                nat.call("ffno_gate_fwd_tc", ws.x.data_ptr(), ws.V, C, bp["tc_s_gate"].data_ptr(), None, None,
                         ws.xs.data_ptr(), ws.err.data_ptr(), s)
            else:
                nat.call("ffno_gate_fwd", ws.x.data_ptr(), ws.V, C, bp["s_g1"].data_ptr(), bp["s_g2"].data_ptr(), None,
                         None, ws.xs.data_ptr(), s)
            d = _descs(Ds, H, W, C, live)
            ex._xf(pln, "twf", ws.xs, ws.sa, d["wf"], ws)
            ex._xf(pln, "thf", ws.sa, ws.sb, d["hf"], ws)
            ex._mix(ws, "s", bp, fq, ws.sb, ws.sa, H * Wf, Ds, C, 2 * H * Wf * C, H * Wf * C, False)
            ex._xf(pln, "thi", ws.sa, ws.sb, d["hf"], ws)
            ex._xf(pln, "twi", ws.sb, ws.ys, d["wi"], ws)
            self._stats(ws, ex._mlp2(ws, 0, ws.ys, None, None, 0.0, None, bp["s_p1"], bp["s_p2"], bp.get("tc_s_post"),
                                     ws.spec_pre))

        self._run(depth, depth_ws, ld(["x"], [X]), spectral, st(["spec_pre"], [A]))
        self._finalize("spec", bp["spec_g"], bp["spec_b"])

        # height branch over row slabs [D][h0:h1][W] -> vert_pre (B): strided copies of D rows each
        hq = hgt["freq"][i]
        rowb = HW * C * 4

        def rows_in(ws, it):
            width = (it[1] - it[0]) * W * C * 4
            self._rows(ws.x.data_ptr(), width, X.data_ptr() + it[0] * W * C * 4, rowb, width, D)

        def rows_out(ws, it):
            width = (it[1] - it[0]) * W * C * 4
            self._rows(B.data_ptr() + it[0] * W * C * 4, rowb, ws.vert_pre.data_ptr(), width, width, D)

        def vertical(ws, it):
            s, rows = _stream(), it[1] - it[0]
            if tc:
                nat.call("ffno_gate_fwd_tc", ws.x.data_ptr(), ws.V, C, bp["tc_v_gate"].data_ptr(), bp["v_zp"].data_ptr(),
                         ws.zr.data_ptr(), ws.xv.data_ptr(), ws.err.data_ptr(), s)
            else:
                nat.call("ffno_gate_fwd", ws.x.data_ptr(), ws.V, C, bp["v_g1"].data_ptr(), bp["v_g2"].data_ptr(),
                         bp["v_zp"].data_ptr(), ws.zr.data_ptr(), ws.xv.data_ptr(), s)
            d = _descs(D, rows, W, C, live)
            RW = rows * W
            ex._xf(hgt, "tzf", ws.xv, ws.va, d["zf"], ws)
            ex._mix(ws, "v", bp, hq, ws.va, ws.vb, live, RW, RW * C, C, live * RW * C, False)
            ex._xf(hgt, "tzi", ws.vb, ws.yv, d["zi"], ws)
            self._stats(ws, ex._mlp2(ws, 0, ws.yv, None, None, 0.0, None, bp["v_p1"], bp["v_p2"], bp.get("tc_v_post"),
                                     ws.vert_pre))

        self._run(list(self._row_slabs()), row_ws, rows_in, vertical, rows_out)
        self._finalize("vert", bp["vert_g"], bp["vert_b"])

        # fusion -> fused_pre (F)
        def fusion(ws, it):
            s = _stream()
            if tc:
                ex._fuse1_tc(ws, bp, ws.x, None)
                nat.call("ffno_fuse2_tc", ws.spec_pre.data_ptr(), self.coefs["spec"].data_ptr(),
                         ws.vert_pre.data_ptr(), self.coefs["vert"].data_ptr(), ws.gates.data_ptr(), ws.V, C,
                         bp["tc_fuse2"].data_ptr(), ws.dw.data_ptr(), ws.fused_pre.data_ptr(),
                         ws.partials.data_ptr(), ws.nparts_tc, self.G, ws.err.data_ptr(), s)
            else:
                nat.call("ffno_fuse_fwd", ws.x.data_ptr(), ws.spec_pre.data_ptr(), self.coefs["spec"].data_ptr(),
                         ws.vert_pre.data_ptr(), self.coefs["vert"].data_ptr(), ws.V, C, bp["bg1"].data_ptr(),
                         bp["bg2"].data_ptr(), bp["bgb"].data_ptr(), bp["f1"].data_ptr(), bp["f2"].data_ptr(),
                         ws.dw.data_ptr(), ws.fused_pre.data_ptr(), ws.partials.data_ptr(), ws.nparts, self.G, s)
            self._stats(ws, tc)

        self._run(depth, depth_ws, ld(["x", "spec_pre", "vert_pre"], [X, A, B]), fusion, st(["fused_pre"], [F]))
        self._finalize("fuse", bp["fuse_g"], bp["fuse_b"])

        # x1 = x + r_f gelu(GN(fused_pre)) (A), pw_pre (B)
        def pw(ws, it):
            self._stats(ws, ex._mlp2(ws, 1, ws.x, ws.fused_pre, self.coefs["fuse"], r_f, ws.x1, bp["pw1"], bp["pw2"],
                                     bp.get("tc_pw"), ws.pw_pre))

        self._run(depth, depth_ws, ld(["x", "fused_pre"], [X, F]), pw, st(["x1", "pw_pre"], [A, B]))
        self._finalize("pw", bp["pw_g"], bp["pw_b"])

        # x2 = x1 + r_pw GN(pw_pre) (F), mlp_pre (A, over x1 slab by slab)
        def mlp(ws, it):
            self._stats(ws, ex._mlp2(ws, 2, ws.x1, ws.pw_pre, self.coefs["pw"], r_pw, ws.x2, bp["m1"], bp["m2"],
                                     bp.get("tc_mlp"), ws.mlp_pre))

        self._run(depth, depth_ws, ld(["x1", "pw_pre"], [A, B]), mlp, st(["x2", "mlp_pre"], [F, A]))
        self._finalize("mlp", bp["mlp_g"], bp["mlp_b"])

        # block output x = x2 + r_mlp GN(mlp_pre) (X)
        def out(ws, it):
            nat.call("ffno_resid_out", ws.x2.data_ptr(), ws.mlp_pre.data_ptr(), self.coefs["mlp"].data_ptr(), r_mlp,
                     ws.V, C, ws.x.data_ptr(), _stream())

        self._run(depth, depth_ws, ld(["x2", "mlp_pre"], [F, A]), out, st(["x"], [X]))


_NORMS = ("spec", "vert", "fuse", "pw", "mlp")
# the service's float32 populations are 10^clamp(log10 n, +-37) (the device kernel clamps); a value within 1e-6 dex
# of a bound was limited
LOG10_POPULATION_LIMIT = 37.0
_LIMITED_HI, _LIMITED_LO = 10.0 ** (LOG10_POPULATION_LIMIT - 1e-6), 10.0 ** (1e-6 - LOG10_POPULATION_LIMIT)


class StreamingBackend:
    """The reference's BatchedFFNOBackend interface (ffno_batched_backend.py:116-308) on one GB300: a checkpoint's
    FFNO3D predicting a whole cube of any size that fits in host RAM. predict_log10 takes model units, predict_si the
    service's SI units; chunk_depth / chunk_rows are the device slab sizes."""

    def __init__(self, model, level_names, normalization=None, device="cuda", chunk_depth=16, chunk_rows=16,
                 log=print):
        if not torch.cuda.is_available():
            raise RuntimeError("the GB300 streaming backend requires CUDA")
        self.device = torch.device(device)
        self.model = model.to(self.device).eval()
        self.levels = int(model.out_channels)
        self.level_names = tuple(str(v) for v in level_names)
        if len(self.level_names) != self.levels:
            raise RuntimeError("checkpoint Cout differs from configured level_names")
        self.normalization = normalization or {k: getattr(model, k).detach().cpu().numpy() for k in
                                               ("mean_X", "std_X", "mean_Y", "std_Y")}
        self.forward = StreamingForward(self.model, chunk_depth, chunk_rows, self.normalization)
        self.log = log

    @classmethod
    def from_checkpoint(cls, checkpoint_path, factory, level_names, factory_kwargs=None, device="cuda", **kw):
        from .runtime import load_checkpoint
        ck = load_checkpoint(checkpoint_path)
        norm, io = ck.get("normalization_stats"), ck.get("io_metadata")
        if norm is None or io is None:
            raise RuntimeError("checkpoint must contain normalization_stats and io_metadata")
        model = factory(Cin=int(io["Cin"]), Cout=int(io["Cout"]), device="cpu", **dict(factory_kwargs or {}))
        model.load_state_dict(ck["model_state"], strict=True)
        return cls(model, level_names, normalization=norm, device=device, **kw)

    def predict_si(self, features, z_m, dx, dy):
        """Linear populations [m^-3], (D, H, W, levels), from SI features (T [K], vx, vy, vz [m/s], log10 ne,
        log10 rho) and heights z_m [m] (ffno_batched_backend.py:285-308)."""
        features = np.asarray(features, dtype=np.float32)
        if features.ndim != 4 or features.shape[0] != len(INPUT_CHANNELS):
            raise ValueError(f"expected features (6,D,H,W), got {features.shape}")
        if not (np.isfinite(features).all() and np.isfinite(np.asarray(z_m)).all()):
            raise ValueError("FFNO request contains NaN or Inf")
        if not (features[0] > 0).all():
            raise ValueError("FFNO request temperature must be positive")
        pop = self.forward(features, z_m, float(dx), float(dy))
        limited = int(np.count_nonzero((pop >= _LIMITED_HI) | (pop <= _LIMITED_LO)))
        if limited:
            self.log(f"STREAMING {limited} predicted populations beyond 10^+-{LOG10_POPULATION_LIMIT:g} limited to it")
        if not np.isfinite(pop).all() or (pop <= 0).any():
            raise RuntimeError("FFNO returned non-positive or non-finite populations")
        return pop

    def predict_log10(self, features, z_scale, dx, dy):
        """log10 populations (levels, D, H, W) from features in model units (log10 T, velocities in km/s, log10 ne,
        log10 rho) and z in Mm (ffno_batched_backend.py:251-283)."""
        f = np.array(features, dtype=np.float64)
        if f.ndim != 4 or f.shape[0] != len(INPUT_CHANNELS):
            raise ValueError(f"expected features (6,D,H,W), got {f.shape}")
        if not (np.isfinite(f).all() and np.isfinite(np.asarray(z_scale)).all()):
            raise ValueError("FFNO request contains NaN or Inf")
        f[0] = 10.0 ** f[0]
        f[1:4] *= 1e3
        return self.forward(f.astype(np.float32), np.asarray(z_scale, dtype=np.float64) * 1e6, float(dx), float(dy),
                            log10=True)
