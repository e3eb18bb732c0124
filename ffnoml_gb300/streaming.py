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
grids use one pair of height tables; per-column grids (every column its own heights) keep every column's tables on the
device and each row slab uses its own columns' tables.

StreamingVJP adds the input VJP, which the reference's batched backend does not have: every block's input is kept in
pinned host memory during the forward, and the backward recomputes each block slab by slab before running the resident
path's backward kernels over the same slabs (its class docstring has the stages).
"""
import copy

import numpy as np
import torch

from . import _native as nat
from .executor import EPS, Workspace, _descs, _GradBuffers, _stream
from .runtime import INPUT_CHANNELS, _check, _host_copy


class _Call:
    """The state of one streaming call (shapes, device inputs, tables, workspaces)."""

    def __init__(self, **kw):
        self.__dict__.update(kw)


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

    # ------------------------------------------------------------------------------------------------ set-up
    def _setup(self, features, z_m, dx, dy):
        """Validate a request, convert its SI inputs slab by slab into the normalised inputs and heights kept on the
        device, and prepare the tables, workspaces and statistics buffers of the call."""
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
        # shared grids: one table pair; per-column grids: every column's tables on the device ([HW][2M'][D] and
        # [HW][D][2M'], built by ffno_percol_tables), which each row slab addresses from its first column
        hgt = ex.height(pk, geo, dev) if geo.shared else ex.height_percol(pk, geo, 0, dev)
        pln, pfr = ex.plane(H, W, dev), ex.plane_freq(pk, H, W, float(dx), float(dy), dev)
        live = hgt["live"]
        dw = torch.empty(V, dtype=torch.float32, device=dev)
        nat.call("ffno_depth_weights", zmm.data_ptr(), D, H * W, dw.data_ptr(), s)
        # two device buffer sets per slab kind (the copies of one slab overlap the kernels of the other), the copy
        # streams
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
            ws.buf = b
            ws.dw = dw.view(D, H, W)[:, it[0]:it[1]].contiguous().view(-1)
            ws.zr = zmm.view(D, H, W)[:, it[0]:it[1]].contiguous()
            for n in self.coefs:
                ws.coefs[n] = self.coefs[n]
            return ws

        return _Call(dev=dev, D=D, H=H, W=W, V=V, C=C, L=L, cd=cd, cr=cr, pk=pk, hgt=hgt, pln=pln, pfr=pfr,
                     live=live, dw=dw, xn=xn, zmm=zmm, xs=xs, flags=flags, norm=norm, bufs=bufs, wsd=wsd, wsr=wsr,
                     depth_ws=depth_ws, row_ws=row_ws, f_host=f_host, geo=geo, dx=float(dx), dy=float(dy))

    def _slab_inputs(self, cx, d0, d1):
        """Normalised model inputs of depth slab d0:d1, contiguous [6][Vs] (in cx.xs; the current stream)."""
        Vs = (d1 - d0) * self.HW
        self._rows(cx.xs.data_ptr(), Vs * 4, cx.xn.data_ptr() + d0 * self.HW * 4, cx.V * 4, Vs * 4, 6)
        return cx.xs

    def _lift(self, cx, X, A):
        """The lift over depth slabs into host X (A holds the pre-activation in between)."""
        m, pk, C = self.model, cx.pk, cx.C
        depth = list(self._depth_slabs())

        def lift(ws, it):
            x = self._slab_inputs(cx, *it)
            nat.call("ffno_lift_fwd", x.data_ptr(), m.in_channels, ws.V, C, pk.lift_w.data_ptr(), ws.dw.data_ptr(),
                     ws.pre.data_ptr(), ws.partials.data_ptr(), ws.nparts, self.G, _stream())
            self._stats(ws, False)

        self._run(depth, cx.depth_ws, None, lift, lambda ws, it: self._store(ws, ["pre"], it[0], it[1], [A]))
        self._finalize("lift", pk.lift_g, pk.lift_b)

        def act(ws, it):
            nat.call("ffno_gn_act", ws.pre.data_ptr(), self.coefs["lift"].data_ptr(), ws.V, C, 1, ws.x.data_ptr(),
                     _stream())

        self._run(depth, cx.depth_ws, lambda ws, it: self._load(ws, ["pre"], it[0], it[1], [A]), act,
                  lambda ws, it: self._store(ws, ["x"], it[0], it[1], [X]))

    # ------------------------------------------------------------------------------------------------ forward
    def __call__(self, features, z_m, dx, dy, log10=False):
        """SI features (6, D, H, W) and heights z_m (D, H, W) in metres (host arrays) -> populations (D, H, W, L)
        in m^-3 (numpy), as BatchedFFNOBackend.predict_si (ffno_batched_backend.py:285-308); with log10, the
        de-normalised log10 populations (L, D, H, W) as its predict_log10 (:251-283)."""
        cx = self._setup(features, z_m, dx, dy)
        m, ex, pk = self.model, self.ex, cx.pk
        D, H, W, V, L, cd = cx.D, cx.H, cx.W, cx.V, cx.L, cx.cd
        X, A, B, F, pop_host = cx.bufs["X"], cx.bufs["A"], cx.bufs["B"], cx.bufs["F"], cx.bufs["pop"]
        self._lift(cx, X, A)
        rotating = dict(spec_pre=A, vert_pre=B, fused_pre=F, x1=A, pw_pre=B, x2=F, mlp_pre=A)
        for i in range(m.n_layers):
            self._block(cx, i, X, X, rotating)

        # head, and the SI populations (or log10 n) of each slab, one output buffer per buffer set
        outs = [torch.empty(L, cd * H * W, dtype=torch.float32, device=cx.dev) for _ in range(2)]
        pops = [torch.empty(cd * H * W, L, dtype=torch.float32, device=cx.dev) for _ in range(2)]
        norm, flags = cx.norm, cx.flags

        def head(ws, it):
            b = ws.buf
            x = self._slab_inputs(cx, *it)
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

        self._run(list(self._depth_slabs()), cx.depth_ws, lambda ws, it: self._load(ws, ["x"], it[0], it[1], [X]),
                  head, head_out)
        torch.cuda.current_stream().synchronize()
        _check(flags.item(), "FFNO streaming output")
        self._check_err(cx)
        out = np.empty((L, D, H, W) if log10 else (D, H, W, L), dtype=np.float32)
        _host_copy(out, pop_host.numpy()[:V * L])
        return out

    def _vert_forward(self, cx, ws, it, bp, hq):
        """The height operator's transforms and mode mixing on row slab it = (h0, h1): ws.xv -> ws.yv (ws.va: the
        modes, ws.vb: the mixed modes), with the shared tables or the slab's columns' own tables."""
        ex, hgt, live = self.ex, cx.hgt, cx.live
        D, W, C = self.D, self.W, self.C
        rows = it[1] - it[0]
        RW, s = rows * W, _stream()
        d = _descs(D, rows, W, C, live)
        if hgt.get("percol"):
            c0 = it[0] * W
            nat.call("ffno_xform_pt", hgt["tzf"].data_ptr() + 4 * c0 * 2 * live * D, 2 * live * D, ws.xv.data_ptr(),
                     ws.va.data_ptr(), d["pcf"], 0, s)
            ex._mix(ws, "v", bp, hq, ws.va, ws.vb, live, RW, RW * C, C, live * RW * C, False)
            nat.call("ffno_xform_pt", hgt["tzi"].data_ptr() + 4 * c0 * 2 * live * D, 2 * live * D, ws.vb.data_ptr(),
                     ws.yv.data_ptr(), d["pci"], 0, s)
        else:
            ex._xf(hgt, "tzf", ws.xv, ws.va, d["zf"], ws)
            ex._mix(ws, "v", bp, hq, ws.va, ws.vb, live, RW, RW * C, C, live * RW * C, False)
            ex._xf(hgt, "tzi", ws.vb, ws.yv, d["zi"], ws)

    @staticmethod
    def _check_err(cx):
        if any(int(w.err.item()) for w in cx.wsd + cx.wsr):
            raise RuntimeError("tensor-core kernel timed out")

    # ------------------------------------------------------------------------------------------------ one block
    def _block(self, cx, i, Xin, Xout, dst):
        """Block i over slabs: input hidden state in host Xin, output into host Xout (None: not written, a
        recomputation for the VJP), every intermediate into the host buffer dst names (spec_pre, vert_pre, fused_pre,
        x1, pw_pre, x2, mlp_pre; buffers may be shared when their lives do not overlap)."""
        ex = self.ex
        pk, depth_ws, row_ws, hgt, pln, fq = cx.pk, cx.depth_ws, cx.row_ws, cx.hgt, cx.pln, cx.pfr[i]
        X = Xin
        C, D, H, W, HW, Wf = self.C, self.D, self.H, self.W, self.HW, self.W // 2 + 1
        bp = pk.blocks[i]
        live = hgt["live"]
        tc, tcg = ex._tc(), ex._tc_chan()      # every kernel family / the channel MLPs and input gates
        r_f, r_pw, r_mlp = bp["res"]
        depth = list(self._depth_slabs())
        ld = lambda names, hosts: (lambda ws, it: self._load(ws, names, it[0], it[1], hosts))
        st = lambda names, hosts: (lambda ws, it: self._store(ws, names, it[0], it[1], hosts))

        # horizontal spectral branch over depth slabs -> spec_pre (A)
        def spectral(ws, it):
            s, Ds = _stream(), it[1] - it[0]
            if tcg:
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

        self._run(depth, depth_ws, ld(["x"], [X]), spectral, st(["spec_pre"], [dst["spec_pre"]]))
        self._finalize("spec", bp["spec_g"], bp["spec_b"])

        # height branch over row slabs [D][h0:h1][W] -> vert_pre (B): strided copies of D rows each
        hq = hgt["freq"][i]
        rowb = HW * C * 4

        def rows_in(ws, it):
            width = (it[1] - it[0]) * W * C * 4
            self._rows(ws.x.data_ptr(), width, X.data_ptr() + it[0] * W * C * 4, rowb, width, D)

        def rows_out(ws, it):
            width = (it[1] - it[0]) * W * C * 4
            self._rows(dst["vert_pre"].data_ptr() + it[0] * W * C * 4, rowb, ws.vert_pre.data_ptr(), width, width,
                       D)

        def vertical(ws, it):
            s, rows = _stream(), it[1] - it[0]
            if tcg:
                nat.call("ffno_gate_fwd_tc", ws.x.data_ptr(), ws.V, C, bp["tc_v_gate"].data_ptr(), bp["v_zp"].data_ptr(),
                         ws.zr.data_ptr(), ws.xv.data_ptr(), ws.err.data_ptr(), s)
            else:
                nat.call("ffno_gate_fwd", ws.x.data_ptr(), ws.V, C, bp["v_g1"].data_ptr(), bp["v_g2"].data_ptr(),
                         bp["v_zp"].data_ptr(), ws.zr.data_ptr(), ws.xv.data_ptr(), s)
            self._vert_forward(cx, ws, it, bp, hq)
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

        self._run(depth, depth_ws, ld(["x", "spec_pre", "vert_pre"], [X, dst["spec_pre"], dst["vert_pre"]]), fusion,
                  st(["fused_pre"], [dst["fused_pre"]]))
        self._finalize("fuse", bp["fuse_g"], bp["fuse_b"])

        # x1 = x + r_f gelu(GN(fused_pre)) (A), pw_pre (B)
        def pw(ws, it):
            self._stats(ws, ex._mlp2(ws, 1, ws.x, ws.fused_pre, self.coefs["fuse"], r_f, ws.x1, bp["pw1"], bp["pw2"],
                                     bp.get("tc_pw"), ws.pw_pre))

        self._run(depth, depth_ws, ld(["x", "fused_pre"], [X, dst["fused_pre"]]), pw,
                  st(["x1", "pw_pre"], [dst["x1"], dst["pw_pre"]]))
        self._finalize("pw", bp["pw_g"], bp["pw_b"])

        # x2 = x1 + r_pw GN(pw_pre) (F), mlp_pre (A, over x1 slab by slab)
        def mlp(ws, it):
            self._stats(ws, ex._mlp2(ws, 2, ws.x1, ws.pw_pre, self.coefs["pw"], r_pw, ws.x2, bp["m1"], bp["m2"],
                                     bp.get("tc_mlp"), ws.mlp_pre))

        self._run(depth, depth_ws, ld(["x1", "pw_pre"], [dst["x1"], dst["pw_pre"]]), mlp,
                  st(["x2", "mlp_pre"], [dst["x2"], dst["mlp_pre"]]))
        self._finalize("mlp", bp["mlp_g"], bp["mlp_b"])

        # block output x = x2 + r_mlp GN(mlp_pre) (X)
        def out(ws, it):
            nat.call("ffno_resid_out", ws.x2.data_ptr(), ws.mlp_pre.data_ptr(), self.coefs["mlp"].data_ptr(), r_mlp,
                     ws.V, C, ws.x.data_ptr(), _stream())

        if Xout is not None:
            self._run(depth, depth_ws, ld(["x2", "mlp_pre"], [dst["x2"], dst["mlp_pre"]]), out, st(["x"], [Xout]))


class StreamingVJP(StreamingForward):
    """Input VJP of FFNO3D on a cube held in host memory, the cube on the device a slab at a time (the reference's
    BatchedFFNOBackend streams the forward only; ffno_batched_backend.py:206-289 is the forward this differentiates).

    The forward keeps every block's input hidden state in pinned host memory (the reference's per-block activation
    checkpoints, models/ffno_model.py:751-780). The backward runs the blocks in reverse: each block's forward is
    recomputed slab by slab into host buffers (with its GroupNorm statistics of the whole cube), then back-propagated
    stage by stage with the resident path's backward kernels. A GroupNorm backward needs two sums over the whole cube
    (S1 = sum g, S2 = sum g xhat), so each one is a statistics pass over depth slabs (every slab's per-CTA partials
    gathered, reduced once in a fixed order) followed by the pass that applies it. The pointwise and horizontal stages
    run over depth slabs, the height branch over row slabs [D][h0:h1][W]; the height tables' gradients accumulate over
    the row slabs (FP64; per column for per-column grids) and reach the heights as in the resident path. Per voxel the
    device keeps the normalised inputs, heights, depth weights and their gradients (15 floats); every [V][C] state
    stays on the host."""

    _INTER = ("spec_pre", "vert_pre", "fused_pre", "x1", "pw_pre", "x2", "mlp_pre")

    def _vjp_buffers(self, V, C, L, n_layers):
        key = (V, C, L, n_layers)
        if getattr(self, "_vjp_key", None) != key:
            self._vjp = None
            self._vjp = dict(ck=[_pinned(V * C) for _ in range(n_layers + 1)],
                             S={n: _pinned(V * C) for n in self._INTER},
                             G=_pinned(V * C), GA=_pinned(V * C), T1=_pinned(V * C), T2=_pinned(V * C),
                             T3=_pinned(V * C), cot=_pinned(V * L), fbar=_pinned(6 * V), zbar=_pinned(V))
            self._vjp_key = key
        return self._vjp

    def __call__(self, features, z_m, dx, dy, population_cotangent):
        """SI features (6, D, H, W), heights z_m (D, H, W) in metres and the cotangent of the populations (D, H, W, L)
        (host arrays) -> {"features": (6, D, H, W), "z_scale": (D, H, W)}, the VJP per SI unit, as
        GB300Backend.vjp_local returns it (ffno_fsdp_runtime.py:306-348)."""
        m, ex = self.model, self.ex
        cot = np.ascontiguousarray(population_cotangent, dtype=np.float32)
        expected = tuple(np.shape(z_m)) + (m.out_channels,)
        if tuple(cot.shape) != expected:
            raise ValueError(f"population_cotangent has shape {cot.shape}; expected {expected}")
        cx = self._setup(features, z_m, dx, dy)
        pk, dev = cx.pk, cx.dev
        D, H, W, V, C, L, cd, cr = cx.D, cx.H, cx.W, cx.V, cx.C, cx.L, cx.cd, cx.cr
        HW, G, s = H * W, self.G, _stream()
        hb = self._vjp_buffers(V, C, L, m.n_layers)
        ck, S = hb["ck"], hb["S"]
        _host_copy(hb["cot"].numpy(), cot)
        # forward, keeping every block's input
        self._lift(cx, ck[0], S["spec_pre"])
        rotating = dict(spec_pre=S["spec_pre"], vert_pre=S["vert_pre"], fused_pre=S["fused_pre"], x1=S["spec_pre"],
                        pw_pre=S["vert_pre"], x2=S["fused_pre"], mlp_pre=S["spec_pre"])
        for i in range(m.n_layers):
            self._block(cx, i, ck[i], ck[i + 1], rotating)
        # per-voxel gradients on the device: depth weights, heights (z_proj terms in row-slab order), model inputs
        f32 = dict(dtype=torch.float32, device=dev)
        wbar = torch.zeros(V, **f32)
        zbar_rows = torch.zeros(V, **f32)
        xin_bar = torch.zeros(6, V, **f32)
        live = cx.live
        # the height tables' gradients: one pair for a shared grid, one per column for per-column grids
        ncol = 1 if cx.geo.shared else HW
        tzf_bar = torch.zeros(ncol, 2 * live, D, dtype=torch.float64, device=dev)
        tzi_bar = torch.zeros(ncol, D, 2 * live, dtype=torch.float64, device=dev)
        nparts = [w.nparts for w in cx.wsd] + [w.nparts for w in cx.wsr]
        gbd = [_GradBuffers(cd, H, W, C, live, G, max(nparts), dev) for _ in range(2)]
        gbr = [_GradBuffers(D, cr, W, C, live, G, max(nparts), dev) for _ in range(2)]
        nslab = -(-D // cd)
        self.bparts = torch.empty(nslab * max(nparts) * G * 2, dtype=torch.float64, device=dev)
        self.bsums = torch.empty(G * 2, dtype=torch.float64, device=dev)
        self.cx, self.gbd, self.gbr, self.wbar = cx, gbd, gbr, wbar
        self.zbar_rows, self.tzf_bar, self.tzi_bar = zbar_rows, tzf_bar, tzi_bar
        depth = list(self._depth_slabs())
        cot_dev = [torch.empty(cd * HW * L, **f32) for _ in range(2)]
        ys = [torch.empty(L, cd * HW, **f32) for _ in range(2)]
        xib = torch.empty(6, cd * HW, **f32)
        tc = ex._tc()

        # head: the populations' cotangent into the normalised output's (the forward of the slab's head first), the
        # head's backward -> the last block output's gradient (G) and the head's direct input gradient
        def head_in(ws, it):
            self._load(ws, ["x"], it[0], it[1], [ck[-1]])
            Vs = (it[1] - it[0]) * HW
            self._h2d(cot_dev[ws.buf], hb["cot"], it[0] * HW * L, Vs * L)

        def head(ws, it):
            b, Vs = ws.buf, ws.V
            x = self._slab_inputs(cx, *it)
            y = ys[b].view(-1)[:L * Vs].view(L, Vs)
            ex._head(pk, ws.x, x, y, ws.err, Vs)
            ybar = ws.yv.view(-1)[:L * Vs]        # a free [Vs][C] buffer of the slab holds y_bar [L][Vs]
            nat.call("ffno_si_population_cotangent", y.data_ptr(), cot_dev[b].data_ptr(), Vs, L,
                     cx.norm["mean_Y"].data_ptr(), cx.norm["std_Y"].data_ptr(), ybar.data_ptr(), cx.flags.data_ptr(), s)
            gb = gbd[b]
            if tc or ex._tc_fuse96():
                nat.call("ffno_head_bwd_tc", ws.x.data_ptr(), x.data_ptr(), ybar.data_ptr(), Vs, C,
                         pk.tcb_head.data_ptr(), pk.b2.data_ptr(), pk.nhp, pk.head32, gb.xbar.data_ptr(),
                         xib.data_ptr(), ws.err.data_ptr(), s)
            else:
                nat.call("ffno_head_bwd", ws.x.data_ptr(), x.data_ptr(), ybar.data_ptr(), Vs, C, pk.p1.data_ptr(),
                         pk.p2.data_ptr(), pk.b2.data_ptr(), pk.p2t.data_ptr(), pk.p1t.data_ptr(), pk.nhp, pk.head,
                         gb.xbar.data_ptr(), xib.data_ptr(), s)
            self._rows(xin_bar.data_ptr() + it[0] * HW * 4, V * 4, xib.data_ptr(), Vs * 4, Vs * 4, 6)

        self._run(depth, cx.depth_ws, head_in, head, self._st_gb(gbd, "xbar", hb["G"]))
        # the blocks in reverse: G holds the gradient of block i's output, then of its input
        for i in reversed(range(m.n_layers)):
            self._block(cx, i, ck[i], None, S)
            self._block_bwd(i, ck[i], S, hb)
            hb["G"], hb["GA"] = hb["GA"], hb["G"]
        # lift: recompute its pre-activation and statistics (into T1), then its GroupNorm backward and the lift
        # convolution's transpose into the input gradient
        self._lift(cx, hb["T2"], hb["T1"])
        self._gn_bwd_stats("lift", 1, 1.0, hb["G"], hb["T1"], pk.lift_g, pk.lift_b)

        def lift_bwd(ws, it):
            gb, Vs = gbd[ws.buf], ws.V
            self._gn_apply("lift", 1, 1.0, ws, gb.xbar, gb.g2, pk.lift_g, pk.lift_b, gb.pbar, it)
            o = it[0] * HW
            self._rows(xib.data_ptr(), Vs * 4, xin_bar.data_ptr() + o * 4, V * 4, Vs * 4, 6)
            nat.call("ffno_lift_bwd", gb.pbar.data_ptr(), m.in_channels, Vs, C, pk.lift_w.data_ptr(), xib.data_ptr(),
                     s)
            self._rows(xin_bar.data_ptr() + o * 4, V * 4, xib.data_ptr(), Vs * 4, Vs * 4, 6)

        self._run(depth, cx.depth_ws, self._ld_gb(gbd, [("xbar", hb["G"]), ("g2", hb["T1"])]), lift_bwd, None)
        # heights: the z_proj terms (row-slab order) into the cube's order, then the depth weights' and the shared
        # column's height-table terms
        zbar = torch.empty(V, **f32)
        for h0, h1 in self._row_slabs():
            rows = h1 - h0
            width = rows * W * 4
            self._rows(zbar.data_ptr() + h0 * W * 4, HW * 4, zbar_rows.data_ptr() + D * h0 * W * 4, width, width, D)
        nat.call("ffno_depth_weights_bwd", cx.zmm.data_ptr(), wbar.data_ptr(), D, HW, zbar.data_ptr(), s)
        if cx.geo.shared:
            # the shared tables depend on column (0, 0): their gradient goes there (FP64, on the device)
            ex._column_tables_vjp(cx.hgt, D, tzf_bar, tzi_bar, zbar, HW)
        else:
            # every column's own tables depend on that column's heights
            hp = cx.hgt
            nat.call("ffno_percol_tables_vjp", hp["z"].data_ptr(), D, HW, hp["k"].data_ptr(), live, hp["f"].data_ptr(),
                     hp["df"].data_ptr(), hp["med"].data_ptr(), tzf_bar.data_ptr(), tzi_bar.data_ptr(),
                     zbar.data_ptr(), s)
        # SI units: the feature and height gradients of ffno_fsdp_runtime's conversions, slab by slab
        fs = torch.empty(6, cd * HW, **f32)
        fb = torch.empty(6, cd * HW, **f32)
        zb = torch.empty(cd * HW, **f32)
        for d0, d1 in depth:
            Vs, o = (d1 - d0) * HW, d0 * HW
            self._rows(fs.data_ptr(), Vs * 4, cx.f_host.data_ptr() + o * 4, V * 4, Vs * 4, 6)
            self._rows(xib.data_ptr(), Vs * 4, xin_bar.data_ptr() + o * 4, V * 4, Vs * 4, 6)
            nat.call("ffno_si_input_grads", fs.data_ptr(), xib.data_ptr(), zbar[o:].data_ptr(), Vs,
                     cx.norm["std_X"].data_ptr(), fb.data_ptr(), zb.data_ptr(), cx.flags.data_ptr(), s)
            self._rows(hb["fbar"].data_ptr() + o * 4, V * 4, fb.data_ptr(), Vs * 4, Vs * 4, 6)
            self._d2h(hb["zbar"], o, zb, Vs)
        torch.cuda.current_stream().synchronize()
        flags = int(cx.flags.item())
        if flags & 1:
            raise ValueError("FFNO VJP cotangent contains NaN or Inf")
        _check(flags, "FFNO streaming VJP")
        self._check_err(cx)
        fbar = np.empty((6, D, H, W), np.float32)
        zout = np.empty((D, H, W), np.float32)
        _host_copy(fbar, hb["fbar"].numpy()[:6 * V])
        _host_copy(zout, hb["zbar"].numpy()[:V])
        return {"features": fbar, "z_scale": zout}

    # ------------------------------------------------------------------------------------------------ helpers
    def _ld_gb(self, gbs, pairs):
        """A slab loader of host buffers into the named gradient buffers of the slab's buffer set (depth slabs)."""
        n_of = lambda it: (it[1] - it[0]) * self.HW * self.C

        def load(ws, it):
            gb = gbs[ws.buf]
            for name, host in pairs:
                self._h2d(getattr(gb, name), host, it[0] * self.HW * self.C, n_of(it))
        return load

    def _st_gb(self, gbs, name, host):
        def store(ws, it):
            self._d2h(host, it[0] * self.HW * self.C, getattr(gbs[ws.buf], name), (it[1] - it[0]) * self.HW * self.C)
        return store

    def _gn_bwd_stats(self, name, mode, r, U, PRE, gamma, beta):
        """S1, S2 of the GroupNorm backward of norm `name` (u = host U, pre-activation host PRE) over the whole cube,
        from every depth slab's per-CTA partials, into self.bsums."""
        cx, G, C = self.cx, self.G, self.C
        self.nbpart = 0

        def stats(ws, it):
            gb = self.gbd[ws.buf]
            off = self.nbpart * G * 2
            nat.call("ffno_gn_bwd_stats", mode, gb.xbar.data_ptr(), r, gb.g2.data_ptr(), gamma.data_ptr(),
                     beta.data_ptr(), self.gstats[name].data_ptr(), ws.V, C, G, self.bparts[off:].data_ptr(), ws.nparts,
                     _stream())
            self.nbpart += ws.nparts

        self._run(list(self._depth_slabs()), cx.depth_ws, self._ld_gb(self.gbd, [("xbar", U), ("g2", PRE)]), stats,
                  None)
        nat.call("ffno_gn_bwd_final", self.bparts.data_ptr(), self.nbpart, G, self.bsums.data_ptr(), _stream())

    def _gn_apply(self, name, mode, r, ws, u, pre, gamma, beta, pbar, it):
        """pre_bar of the GroupNorm backward on a depth slab (u, pre: its device rows), with the depth-weight gradient
        of the slab's voxels accumulated into the cube's w_bar."""
        o = it[0] * self.HW
        nat.call("ffno_gn_bwd_apply", mode, u.data_ptr(), r, pre.data_ptr(), gamma.data_ptr(), beta.data_ptr(),
                 self.gstats[name].data_ptr(), self.bsums.data_ptr(), ws.dw.data_ptr(), ws.V, self.C, self.G, EPS,
                 pbar.data_ptr(), self.wbar[o:].data_ptr(), _stream())

    def _mlp_bwd(self, bp, a, pb, base, out, w1, w2t, w1t, pack, V, err):
        if self.ex._tc_chan():
            nat.call("ffno_mlp2_bwd_tc", a.data_ptr(), pb.data_ptr(), None if base is None else base.data_ptr(), V,
                     self.C, bp[pack].data_ptr(), out.data_ptr(), err.data_ptr(), _stream())
        else:
            nat.call("ffno_mlp2_bwd", a.data_ptr(), pb.data_ptr(), None if base is None else base.data_ptr(), V,
                     self.C, bp[w1].data_ptr(), bp[w2t].data_ptr(), bp[w1t].data_ptr(), out.data_ptr(), _stream())

    # ------------------------------------------------------------------------------------------------ one block
    def _block_bwd(self, i, X, S, hb):
        """Block i's VJP (executor.Executor._block_bwd over slabs): hb["G"] (gradient of the block output) ->
        hb["GA"] (gradient of the block input X); the block's intermediates are in S, its GroupNorm statistics in
        self.coefs / self.gstats."""
        ex, cx = self.ex, self.cx
        pk = cx.pk
        bp = pk.blocks[i]
        C, D, H, W, HW, Wf = self.C, self.D, self.H, self.W, self.HW, self.W // 2 + 1
        live, tc, tcg, s = cx.live, ex._tc(), ex._tc_chan(), _stream()
        r_f, r_pw, r_mlp = bp["res"]
        act = 2 if tc else 1      # GELU after the spec / vert GroupNorms, as the forward applied it
        act_f = 2 if ex._tc_chan() else 1   # after the fuse GroupNorm (applied by the pw MLP's prologue)
        depth = list(self._depth_slabs())
        gbd, gbr = self.gbd, self.gbr
        Gout, GA, T1, T2, T3 = hb["G"], hb["GA"], hb["T1"], hb["T2"], hb["T3"]
        ld = lambda names, hosts: (lambda ws, it: self._load(ws, names, it[0], it[1], hosts))

        def both(*loaders):
            def load(ws, it):
                for f in loaders:
                    f(ws, it)
            return load

        # out = x2 + r_mlp GN(mlp_pre), mlp_pre = mlp(x2): x2_bar = out_bar + mlp'(GN'(out_bar)) -> T1
        self._gn_bwd_stats("mlp", 0, r_mlp, Gout, S["mlp_pre"], bp["mlp_g"], bp["mlp_b"])

        def mlp_stage(ws, it):
            gb = gbd[ws.buf]
            self._gn_apply("mlp", 0, r_mlp, ws, gb.xbar, ws.mlp_pre, bp["mlp_g"], bp["mlp_b"], gb.pbar, it)
            self._mlp_bwd(bp, ws.x2, gb.pbar, gb.xbar, gb.g2, "m1", "m2t", "m1t", "tcb_mlp", ws.V, ws.err)

        self._run(depth, cx.depth_ws, both(self._ld_gb(gbd, [("xbar", Gout)]), ld(["mlp_pre", "x2"],
                  [S["mlp_pre"], S["x2"]])), mlp_stage, self._st_gb(gbd, "g2", T1))
        # x2 = x1 + r_pw GN(pw_pre), pw_pre = pw(x1) -> x1_bar in T2
        self._gn_bwd_stats("pw", 0, r_pw, T1, S["pw_pre"], bp["pw_g"], bp["pw_b"])

        def pw_stage(ws, it):
            gb = gbd[ws.buf]
            self._gn_apply("pw", 0, r_pw, ws, gb.xbar, ws.pw_pre, bp["pw_g"], bp["pw_b"], gb.pbar, it)
            self._mlp_bwd(bp, ws.x1, gb.pbar, gb.xbar, gb.g2, "pw1", "pw2t", "pw1t", "tcb_pw", ws.V, ws.err)

        self._run(depth, cx.depth_ws, both(self._ld_gb(gbd, [("xbar", T1)]), ld(["pw_pre", "x1"],
                  [S["pw_pre"], S["x1"]])), pw_stage, self._st_gb(gbd, "g2", T2))
        # x1 = x + r_f gelu(GN(fused_pre)), fused_pre = fuse(x, spec, vert) -> x_bar so far (GA), spec_bar (T1),
        # vert_bar (T3)
        self._gn_bwd_stats("fuse", act_f, r_f, T2, S["fused_pre"], bp["fuse_g"], bp["fuse_b"])

        def fuse_stage(ws, it):
            gb = gbd[ws.buf]
            self._gn_apply("fuse", act_f, r_f, ws, gb.xbar, ws.fused_pre, bp["fuse_g"], bp["fuse_b"], gb.pbar, it)
            cs, cv = self.coefs["spec"].data_ptr(), self.coefs["vert"].data_ptr()
            if tc:
                ex._fuse1_tc(ws, bp, ws.x, gb.hg)
                nat.call("ffno_fuse_bwd_a_tc", ws.spec_pre.data_ptr(), cs, ws.vert_pre.data_ptr(), cv,
                         ws.gates.data_ptr(), gb.pbar.data_ptr(), ws.V, C, bp["tcb_fuse_a"].data_ptr(),
                         gb.hfb.data_ptr(), ws.err.data_ptr(), s)
                nat.call("ffno_fuse_bwd_b_tc", ws.spec_pre.data_ptr(), cs, ws.vert_pre.data_ptr(), cv,
                         ws.gates.data_ptr(), gb.hg.data_ptr(), gb.pbar.data_ptr(), gb.hfb.data_ptr(),
                         gb.xbar.data_ptr(), ws.V, C, bp["tcb_fuse_b"].data_ptr(), gb.xacc.data_ptr(),
                         gb.sbar.data_ptr(), gb.vbar.data_ptr(), ws.err.data_ptr(), s)
            else:
                nat.call("ffno_fuse_bwd", ws.x.data_ptr(), ws.spec_pre.data_ptr(), cs, ws.vert_pre.data_ptr(), cv,
                         gb.pbar.data_ptr(), gb.xbar.data_ptr(), ws.V, C, bp["bg1"].data_ptr(), bp["bg2"].data_ptr(),
                         bp["bgb"].data_ptr(), bp["f1"].data_ptr(), bp["f2t"].data_ptr(), bp["f1t"].data_ptr(),
                         bp["bg2t"].data_ptr(), bp["bg1t"].data_ptr(), gb.xacc.data_ptr(), gb.sbar.data_ptr(),
                         gb.vbar.data_ptr(), s)

        def fuse_store(ws, it):
            for name, host in (("xacc", GA), ("sbar", T1), ("vbar", T3)):
                self._st_gb(gbd, name, host)(ws, it)

        self._run(depth, cx.depth_ws, both(self._ld_gb(gbd, [("xbar", T2)]),
                  ld(["x", "fused_pre", "spec_pre", "vert_pre"], [X, S["fused_pre"], S["spec_pre"], S["vert_pre"]])),
                  fuse_stage, fuse_store)
        # spec = gelu(GN(spec_pre)), spec_pre = post_s(ys), ys = irfft2 mix rfft2 gate_s(x): recompute ys, then back
        # through the post-MLP, the transposed transforms and the gate; x_bar accumulates in GA
        self._gn_bwd_stats("spec", act, 1.0, T1, S["spec_pre"], bp["spec_g"], bp["spec_b"])
        fq = cx.pfr[i]

        def spec_stage(ws, it):
            gb, Ds = gbd[ws.buf], it[1] - it[0]
            d = _descs(Ds, H, W, C, live)
            if tcg:
                nat.call("ffno_gate_fwd_tc", ws.x.data_ptr(), ws.V, C, bp["tc_s_gate"].data_ptr(), None, None,
                         ws.xs.data_ptr(), ws.err.data_ptr(), s)
            else:
                nat.call("ffno_gate_fwd", ws.x.data_ptr(), ws.V, C, bp["s_g1"].data_ptr(), bp["s_g2"].data_ptr(), None,
                         None, ws.xs.data_ptr(), s)
            ex._xf(cx.pln, "twf", ws.xs, ws.sa, d["wf"], ws)
            ex._xf(cx.pln, "thf", ws.sa, ws.sb, d["hf"], ws)
            ex._mix(ws, "s", bp, fq, ws.sb, ws.sa, H * Wf, Ds, C, 2 * H * Wf * C, H * Wf * C, False)
            ex._xf(cx.pln, "thi", ws.sa, ws.sb, d["hf"], ws)
            ex._xf(cx.pln, "twi", ws.sb, ws.ys, d["wi"], ws)
            self._gn_apply("spec", act, 1.0, ws, gb.sbar, ws.spec_pre, bp["spec_g"], bp["spec_b"], gb.pbar, it)
            self._mlp_bwd(bp, ws.ys, gb.pbar, None, gb.ysb, "s_p1", "s_p2t", "s_p1t", "tcb_s_post", ws.V, ws.err)
            ex._xf(cx.pln, "twi_t", gb.ysb, ws.sa, d["wf"], ws)
            ex._xf(cx.pln, "thi_t", ws.sa, ws.sb, d["hf"], ws)
            ex._mix(ws, "s", bp, fq, ws.sb, ws.sa, H * Wf, Ds, C, 2 * H * Wf * C, H * Wf * C, True)
            ex._xf(cx.pln, "thf_t", ws.sa, ws.sb, d["hf"], ws)
            ex._xf(cx.pln, "twf_t", ws.sb, gb.xsb, d["wi"], ws)
            if tcg:
                nat.call("ffno_gate_bwd_tc", ws.x.data_ptr(), gb.xsb.data_ptr(), gb.xacc.data_ptr(), ws.V, C,
                         bp["tcb_s_gate"].data_ptr(), None, gb.xacc.data_ptr(), None, ws.err.data_ptr(), s)
            else:
                gb.xvb.zero_()
                nat.call("ffno_gate_bwd", ws.x.data_ptr(), gb.xsb.data_ptr(), gb.xvb.data_ptr(), gb.xacc.data_ptr(),
                         ws.V, C, bp["s_g1"].data_ptr(), bp["s_g2"].data_ptr(), bp["s_g2t"].data_ptr(),
                         bp["s_g1t"].data_ptr(), bp["v_g1"].data_ptr(), bp["v_g2"].data_ptr(), bp["v_g2t"].data_ptr(),
                         bp["v_g1t"].data_ptr(), bp["v_zp"].data_ptr(), gb.xacc.data_ptr(), gb.wbar.data_ptr(), s)

        self._run(depth, cx.depth_ws, both(self._ld_gb(gbd, [("sbar", T1), ("xacc", GA)]),
                  ld(["x", "spec_pre"], [X, S["spec_pre"]])), spec_stage, self._st_gb(gbd, "xacc", GA))
        # vert = gelu(GN(vert_pre)): its pre-activation gradient over depth slabs (T2), then the height branch over
        # row slabs: recompute xv, its modes and yv; back through the post-MLP, the inverse transform (table gradient),
        # the adjoint mixing, the forward transform (table gradient) and the gate with z_proj
        self._gn_bwd_stats("vert", act, 1.0, T3, S["vert_pre"], bp["vert_g"], bp["vert_b"])

        def vert_pbar(ws, it):
            gb = gbd[ws.buf]
            self._gn_apply("vert", act, 1.0, ws, gb.vbar, ws.vert_pre, bp["vert_g"], bp["vert_b"], gb.pbar, it)

        self._run(depth, cx.depth_ws, both(self._ld_gb(gbd, [("vbar", T3)]), ld(["vert_pre"], [S["vert_pre"]])),
                  vert_pbar, self._st_gb(gbd, "pbar", T2))
        hq = cx.hgt["freq"][i]
        rowb = HW * C * 4

        def rows_in(ws, it):
            gb = gbr[ws.buf]
            width = (it[1] - it[0]) * W * C * 4
            for dst, host in ((ws.x, X), (gb.pbar, T2), (gb.xacc, GA)):
                self._rows(dst.data_ptr(), width, host.data_ptr() + it[0] * W * C * 4, rowb, width, D)

        def rows_out(ws, it):
            gb = gbr[ws.buf]
            width = (it[1] - it[0]) * W * C * 4
            self._rows(GA.data_ptr() + it[0] * W * C * 4, rowb, gb.xacc.data_ptr(), width, width, D)

        def vert_stage(ws, it):
            gb, rows = gbr[ws.buf], it[1] - it[0]
            RW = rows * W
            N = RW * C
            d = _descs(D, rows, W, C, live)
            zrow = self.zbar_rows[D * it[0] * W:]
            if tcg:
                nat.call("ffno_gate_fwd_tc", ws.x.data_ptr(), ws.V, C, bp["tc_v_gate"].data_ptr(), bp["v_zp"].data_ptr(),
                         ws.zr.data_ptr(), ws.xv.data_ptr(), ws.err.data_ptr(), s)
            else:
                nat.call("ffno_gate_fwd", ws.x.data_ptr(), ws.V, C, bp["v_g1"].data_ptr(), bp["v_g2"].data_ptr(),
                         bp["v_zp"].data_ptr(), ws.zr.data_ptr(), ws.xv.data_ptr(), s)
            self._vert_forward(cx, ws, it, bp, hq)
            self._mlp_bwd(bp, ws.yv, gb.pbar, None, gb.yvb, "v_p1", "v_p2t", "v_p1t", "tcb_v_post", ws.V, ws.err)
            hgt = cx.hgt
            if hgt.get("percol"):
                # the slab's columns' tables and their gradients, from its first column on
                c0 = it[0] * W
                tab = 4 * c0 * 2 * live * D
                bar = 8 * c0 * 2 * live * D
                nat.call("ffno_col_outer", gb.yvb.data_ptr(), D, ws.vb.data_ptr(), 2 * live, RW, C, N,
                         self.tzi_bar.data_ptr() + bar, 1, s)
                nat.call("ffno_xform_pt", hgt["tzi_t"].data_ptr() + tab, 2 * live * D, gb.yvb.data_ptr(),
                         ws.va.data_ptr(), d["pcf"], 0, s)
                ex._mix(ws, "v", bp, hq, ws.va, ws.vb, live, RW, RW * C, C, live * RW * C, True)
                nat.call("ffno_col_outer", ws.vb.data_ptr(), 2 * live, ws.xv.data_ptr(), D, RW, C, N,
                         self.tzf_bar.data_ptr() + bar, 1, s)
                nat.call("ffno_xform_pt", hgt["tzf_t"].data_ptr() + tab, 2 * live * D, ws.vb.data_ptr(),
                         gb.xvb.data_ptr(), d["pci"], 0, s)
            else:
                # split counts for this slab's own N (the buffer holds the counts of the largest slab, which are
                # larger)
                lib = nat.lib()
                ex._outer(ws, gb.yvb, D, ws.vb, 2 * live, N, gb.opart, lib.ffno_outer_parts(D, 2 * live, N),
                          self.tzi_bar)
                ex._xf(hgt, "tzi_t", gb.yvb, ws.va, d["zf"], ws)
                ex._mix(ws, "v", bp, hq, ws.va, ws.vb, live, RW, RW * C, C, live * RW * C, True)
                ex._outer(ws, ws.vb, 2 * live, ws.xv, D, N, gb.opart, lib.ffno_outer_parts(2 * live, D, N),
                          self.tzf_bar)
                ex._xf(hgt, "tzf_t", ws.vb, gb.xvb, d["zi"], ws)
            if tcg:
                nat.call("ffno_gate_bwd_tc", ws.x.data_ptr(), gb.xvb.data_ptr(), gb.xacc.data_ptr(), ws.V, C,
                         bp["tcb_v_gate"].data_ptr(), bp["v_zp"].data_ptr(), gb.xacc.data_ptr(), zrow.data_ptr(),
                         ws.err.data_ptr(), s)
            else:
                gb.xsb.zero_()
                nat.call("ffno_gate_bwd", ws.x.data_ptr(), gb.xsb.data_ptr(), gb.xvb.data_ptr(), gb.xacc.data_ptr(),
                         ws.V, C, bp["s_g1"].data_ptr(), bp["s_g2"].data_ptr(), bp["s_g2t"].data_ptr(),
                         bp["s_g1t"].data_ptr(), bp["v_g1"].data_ptr(), bp["v_g2"].data_ptr(), bp["v_g2t"].data_ptr(),
                         bp["v_g1t"].data_ptr(), bp["v_zp"].data_ptr(), gb.xacc.data_ptr(), zrow.data_ptr(), s)

        self._run(list(self._row_slabs()), cx.row_ws, rows_in, vert_stage, rows_out)


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
        self._vjp = None
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

    def vjp_local(self, features, z_scale, dx, dy, population_cotangent):
        """Input VJP along the population cotangent (D, H, W, L) in SI units: {"features": (6, D, H, W), "z_scale":
        (D, H, W)}, the interface of GB300Backend.vjp_local (ffno_fsdp_runtime.py:306-348), for cubes beyond HBM.
        The reference's batched backend has no VJP."""
        features = np.asarray(features, dtype=np.float32)
        if features.ndim != 4 or features.shape[0] != len(INPUT_CHANNELS):
            raise ValueError(f"expected features (6,D,H,W), got {features.shape}")
        cot = np.asarray(population_cotangent, dtype=np.float32)
        if not (np.isfinite(features).all() and np.isfinite(np.asarray(z_scale)).all()):
            raise ValueError("FFNO request contains NaN or Inf")
        if not np.isfinite(cot).all():
            raise ValueError("FFNO VJP cotangent contains NaN or Inf")
        if not (features[0] > 0).all():
            raise ValueError("FFNO request temperature must be positive")
        if self._vjp is None:
            self._vjp = StreamingVJP(self.model, self.forward.chunk_depth, self.forward.chunk_rows,
                                     self.normalization)
        return self._vjp(features, z_scale, float(dx), float(dy), cot)

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
