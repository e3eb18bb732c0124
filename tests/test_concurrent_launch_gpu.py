"""Kernels launched from several host threads at once with different dynamic shared memory sizes. The limit a kernel
may take is one process-wide attribute per kernel; the service runs one request per host thread, so launches of the
same kernel with different sizes overlap in time. Every launch must succeed and give the bits it gives alone."""
import threading

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _case(D, H, W, C, seed):
    """One resident-table height transform (2H x 2H table, so its shared memory grows with H) with its input."""
    from ffnoml_gb300 import _native as nat
    from ffnoml_gb300 import tables as tb
    from ffnoml_gb300.executor import TcXform, _descs
    Wf = W // 2 + 1
    _, thf, _, _ = tb.plane_dft(H, W)
    d = _descs(D, H, W, C, 1)["hf"]
    n = D * 2 * H * Wf * C
    g = torch.Generator().manual_seed(seed)
    x = torch.randn(n, generator=g).cuda()
    tx = TcXform(thf, torch.device("cuda"))
    assert len(tx.slices) == 1
    r0, rows, c0, cols, _, res = tx.slices[0]
    assert res is not None and r0 == 0 and c0 == 0
    dd = nat.XformDesc.from_buffer_copy(d)
    dd.M, dd.K = rows, cols
    return dict(tx=tx, res=res, x=x, dd=dd, n=n)


def _run(case, out, err, stream):
    from ffnoml_gb300 import _native as nat
    res = case["res"]
    nat.call("ffno_xform_tcr", res[0].data_ptr(), res[1], res[2], case["x"].data_ptr(), out.data_ptr(), case["dd"], 0,
             err.data_ptr(), stream.cuda_stream)


def test_overlapping_launches_with_different_shared_memory():
    # resident tables of 48 x 48 and 128 x 128: about 138 KiB and 193 KiB of dynamic shared memory per block
    cases = [_case(8, 24, 20, 16, 1), _case(4, 64, 40, 16, 2)]
    assert cases[0]["res"][1:] != cases[1]["res"][1:]
    alone = []
    for c in cases:
        s = torch.cuda.Stream()
        out = torch.zeros(c["n"], device="cuda")
        err = torch.zeros(1, dtype=torch.int32, device="cuda")
        _run(c, out, err, s)
        s.synchronize()
        assert int(err.item()) == 0
        alone.append(out.cpu())
    failures, results = [], {}

    def worker(i):
        c = cases[i % 2]
        s = torch.cuda.Stream()
        out = torch.zeros(c["n"], device="cuda")
        err = torch.zeros(1, dtype=torch.int32, device="cuda")
        try:
            for _ in range(200):
                _run(c, out, err, s)
            s.synchronize()
        except Exception as e:                     # the status of a refused launch, raised by the binding
            failures.append((i, repr(e)))
            s.synchronize()
            return
        results[i] = (int(err.item()), out.cpu())

    ts = [threading.Thread(target=worker, args=(i,)) for i in range(6)]
    [t.start() for t in ts]
    [t.join() for t in ts]
    assert not failures, failures
    for i, (e, out) in results.items():
        assert e == 0
        assert torch.equal(out, alone[i % 2]), i
