"""The per-column height tables built on the device (ffno_percol_tables) and their gradient (ffno_percol_tables_vjp)
against the float64 host statements in ffnoml_gb300/tables.py (numpy Filon weights; torch autograd through the same
table builder), on columns that run up and down, with tied minima, zero-length intervals and modes inside the taper's
transition band, so that every term of the gradient is exercised."""
import math

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _columns(ncol, D, seed):
    g = np.random.default_rng(seed)
    steps = g.uniform(0.25, 0.7, (ncol, D))            # median spacing ~0.47: k in (4.5, 6.7) falls in the taper band
    cols = 14.0 - np.cumsum(steps, axis=1)              # descending columns (heights from the top)
    cols[1] = cols[1][::-1].copy()                      # an ascending one
    cols[2, 5] = cols[2, 6]                             # a zero-length interval
    cols[3, -1] = cols[3, -2] = cols[3].min() - 0.5     # two tied minima
    if ncol > 4:
        cols[4] = np.sort(g.uniform(-1.0, 14.0, D))[::-1]   # irregular spacing
    return np.ascontiguousarray(cols)


def _k(length, n):
    return torch.arange(0, n, dtype=torch.float64) * 2 * math.pi / (2 * length)


def _device_tables(cols, length, k):
    from ffnoml_gb300 import _native as nat
    from ffnoml_gb300 import tables as tb
    live, f, df, med = tb.percolumn_prep(cols, length, k)
    ncol, D = cols.shape
    dev = torch.device("cuda")
    d64 = lambda a: torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device=dev)
    z, kk, fd, dfd = d64(cols), d64(k.numpy()[:live]), d64(f), d64(df)
    medd = torch.as_tensor(med, dtype=torch.int32, device=dev)
    out = [torch.empty(s, dtype=torch.float32, device=dev)
           for s in ((ncol, 2 * live, D), (ncol, D, 2 * live), (ncol, D, 2 * live), (ncol, 2 * live, D))]
    s = torch.cuda.current_stream().cuda_stream
    nat.call("ffno_percol_tables", z.data_ptr(), D, ncol, kk.data_ptr(), live, fd.data_ptr(),
             *[t.data_ptr() for t in out], s)
    torch.cuda.synchronize()
    return live, out, (z, kk, fd, dfd, medd)


@pytest.mark.parametrize("D,ncol,nk", [(40, 9, 33), (256, 5, 65), (37, 6, 12)])
def test_tables_match_host_float64(D, ncol, nk):
    from ffnoml_gb300 import tables as tb
    length = 15.0
    cols = _columns(ncol, D, D)
    k = _k(length, nk)
    live, (tzf, tzi, tzf_t, tzi_t), _ = _device_tables(cols, length, k)
    live0, tzf0, tzi0 = tb.percolumn_tables(cols, length, k)
    assert live == live0
    for got, ref in ((tzf, tzf0), (tzi, tzi0), (tzf_t, tzf0.transpose(0, 2, 1)), (tzi_t, tzi0.transpose(0, 2, 1))):
        got = got.cpu().numpy().astype(np.float64)
        # both are the float32 rounding of float64 values that agree to ~1e-15: equal or one float32 ulp apart
        assert np.all(np.abs(got - ref) <= 1.2e-7 * np.abs(ref) + 1e-12 * np.abs(ref).max())


@pytest.mark.parametrize("D,ncol,nk", [(40, 9, 33), (256, 5, 65), (37, 6, 12)])
def test_gradient_matches_host_autograd(D, ncol, nk):
    from ffnoml_gb300 import _native as nat
    from ffnoml_gb300 import tables as tb
    length = 15.0
    cols = _columns(ncol, D, D + 1)
    k = _k(length, nk)
    live, _, (z, kk, fd, dfd, medd) = _device_tables(cols, length, k)
    _, f, df, _ = tb.percolumn_prep(cols, length, k)
    # with 33 or more modes some reach the taper's transition band, so its term is live; 12 modes stay below it
    assert np.any(df != 0.0) == (nk >= 33)
    g = np.random.default_rng(D + 2)
    fb = g.normal(size=(ncol, 2 * live, D))
    ib = g.normal(size=(ncol, D, 2 * live))
    ref = tb.percolumn_tables_vjp(cols, length, k, live, fb, ib)          # [ncol][D], float64
    zbar = torch.zeros(D, ncol, dtype=torch.float32, device="cuda")
    # device copies held until the kernel has run (a temporary's memory may be handed to the next allocation)
    fbd = torch.as_tensor(fb, dtype=torch.float64, device="cuda").contiguous()
    ibd = torch.as_tensor(ib, dtype=torch.float64, device="cuda").contiguous()
    nat.call("ffno_percol_tables_vjp", z.data_ptr(), D, ncol, kk.data_ptr(), live, fd.data_ptr(), dfd.data_ptr(),
             medd.data_ptr(), fbd.data_ptr(), ibd.data_ptr(), zbar.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    got = zbar.cpu().numpy().T.astype(np.float64)                      # [ncol][D]
    want = ref.astype(np.float32).astype(np.float64)
    # float64 sums in other orders, then rounded to float32: equal to within two float32 ulps of the entry
    assert np.all(np.abs(got - want) <= 2.4e-7 * np.abs(want) + 1e-9 * np.abs(want).max()), \
        np.max(np.abs(got - want) / (np.abs(want) + 1e-30))


def test_gradient_accumulates_into_z_bar():
    """The kernel adds to z_bar (the executor accumulates the samples' other height gradients there first)."""
    from ffnoml_gb300 import _native as nat
    length, D, ncol = 15.0, 24, 4
    cols = _columns(ncol, D, 5)
    k = _k(length, 20)
    live, _, (z, kk, fd, dfd, medd) = _device_tables(cols, length, k)
    fb = torch.randn(ncol, 2 * live, D, dtype=torch.float64, device="cuda")
    ib = torch.randn(ncol, D, 2 * live, dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    args = lambda zb: (z.data_ptr(), D, ncol, kk.data_ptr(), live, fd.data_ptr(), dfd.data_ptr(), medd.data_ptr(),
                       fb.data_ptr(), ib.data_ptr(), zb.data_ptr(), s)
    a = torch.zeros(D, ncol, device="cuda")
    nat.call("ffno_percol_tables_vjp", *args(a))
    b = torch.full((D, ncol), 2.5, device="cuda")
    nat.call("ffno_percol_tables_vjp", *args(b))
    torch.cuda.synchronize()
    assert torch.equal(b, (a + 2.5))


@pytest.mark.parametrize("Ra,Rb,C,ncol", [(70, 130, 64, 5), (256, 64, 16, 3), (37, 12, 96, 4)])
def test_column_outer_products(Ra, Rb, C, ncol):
    """ffno_col_outer: out[col][i][j] (+)= sum_c A[i][col][c] B[j][col][c] with row stride rs, ragged against the
    64 x 64 output tiles, against float64; each sum over the C channels is FP32 (bounded by C ulps of sum |a b|)."""
    from ffnoml_gb300 import _native as nat
    g = torch.Generator().manual_seed(Ra + Rb + C)
    rs = (ncol + 1) * C                                 # a row holds ncol columns and a spare one
    A = torch.randn(Ra, rs, generator=g).cuda()
    B = torch.randn(Rb, rs, generator=g).cuda()
    out = torch.randn(ncol, Ra, Rb, generator=g, dtype=torch.float64).cuda()
    base = out.clone()
    s = torch.cuda.current_stream().cuda_stream
    nat.call("ffno_col_outer", A.data_ptr(), Ra, B.data_ptr(), Rb, ncol, C, rs, out.data_ptr(), 1, s)
    torch.cuda.synchronize()
    a = A[:, :ncol * C].double().reshape(Ra, ncol, C)
    b = B[:, :ncol * C].double().reshape(Rb, ncol, C)
    ref = torch.einsum("icx,jcx->cij", a, b)
    bound = C * 2.0 ** -23 * torch.einsum("icx,jcx->cij", a.abs(), b.abs())
    assert torch.all((out - base - ref).abs() <= bound + 1e-12)
    nat.call("ffno_col_outer", A.data_ptr(), Ra, B.data_ptr(), Rb, ncol, C, rs, out.data_ptr(), 0, s)
    torch.cuda.synchronize()
    assert torch.all((out - ref).abs() <= bound + 1e-12)


@pytest.mark.parametrize("D,nk", [(40, 33), (256, 65), (37, 12), (256, 700)])
def test_one_column_gradient_matches_per_column_kernel(D, nk):
    """ffno_column_tables_vjp (one column over many CTAs, the shared height grid's path) against
    ffno_percol_tables_vjp on the same column, for columns that run up and down, with a zero-length interval, tied
    minima and irregular spacing, written at a stride into z_bar."""
    from ffnoml_gb300 import _native as nat
    length = 15.0
    cols = _columns(5, D, D + 1)
    k = _k(length, nk)
    dev = torch.device("cuda")
    s = torch.cuda.current_stream().cuda_stream
    g = np.random.default_rng(D + nk)
    for c in range(cols.shape[0]):
        col = cols[c:c + 1]
        live, _, (z, kk, fd, dfd, medd) = _device_tables(col, length, k)
        fbar = torch.as_tensor(g.normal(size=(1, 2 * live, D)), device=dev)
        ibar = torch.as_tensor(g.normal(size=(1, D, 2 * live)), device=dev)
        ref = torch.zeros(D, dtype=torch.float32, device=dev)
        nat.call("ffno_percol_tables_vjp", z.data_ptr(), D, 1, kk.data_ptr(), live, fd.data_ptr(), dfd.data_ptr(),
                 medd.data_ptr(), fbar.data_ptr(), ibar.data_ptr(), ref.data_ptr(), s)
        stride = 7
        got = torch.full((D * stride,), 0.5, dtype=torch.float32, device=dev)
        got.view(D, stride)[:, 0] = 0.0
        scratch = torch.empty(3 * live * D, dtype=torch.float64, device=dev)
        nat.call("ffno_column_tables_vjp", z.data_ptr(), D, kk.data_ptr(), live, fd.data_ptr(), dfd.data_ptr(),
                 int(medd[0].item()), fbar.data_ptr(), ibar.data_ptr(), scratch.data_ptr(), got.data_ptr(), stride, s)
        torch.cuda.synchronize()
        g2 = got.view(D, stride)
        assert torch.all(g2[:, 1:] == 0.5)
        # FP64 sums in another order, rounded to float32: within a few float32 ulps of the largest entry
        err = (g2[:, 0].double() - ref.double()).abs().max().item()
        assert err <= 1e-6 * ref.abs().max().item() + 1e-30, (c, err)
