"""The GB300 service end to end: PREDICT and VJP over the wire against the float64 oracle at the service level (SI
units, linear populations), and each request's result identical alone and in a concurrent mix of uneven sizes."""
import threading

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

MEAN_X = np.array([4.75, 0.0, 0.0, 0.0, 17.5, -8.0], np.float32)
STD_X = np.array([2.5 / 12 ** 0.5, 5.0, 5.0, 5.0, 7.0 / 12 ** 0.5, 8.0 / 12 ** 0.5], np.float32)


def _model(precision):
    from ffnoml_gb300 import create_ffno3d
    torch.manual_seed(0)
    m = create_ffno3d(6, 12, atoms=["H", "CA"], width=32, n_layers=2, hidden_spectral=32, hidden_vertical=32,
                      z_min_wavelength=40.0 / 15)
    with torch.no_grad():
        for n, p in m.named_parameters():
            if ".freq_u." in n:
                p.normal_(0.0, 0.1)
    m.set_normalization(MEAN_X, STD_X, np.zeros(12), np.ones(12))
    m.eval()
    return m.set_precision(precision)


def _request(shape, seed):
    D, H, W = shape
    g = np.random.default_rng(seed)
    f = np.empty((6, D, H, W), np.float32)
    f[0] = 10.0 ** g.uniform(3.5, 6.0, (D, H, W))
    f[1:4] = g.normal(0.0, 5e3, (3, D, H, W))
    f[4] = g.uniform(14.0, 21.0, (D, H, W))
    f[5] = g.uniform(-12.0, -4.0, (D, H, W))
    z = np.broadcast_to(np.linspace(14e6, -1e6, D, dtype=np.float32)[:, None, None], (D, H, W)).copy()
    return f, z


@pytest.fixture(scope="module")
def served():
    from ffnoml_gb300.runtime import GB300Backend
    from ffnoml_gb300.service import Server
    model = _model("fp32")
    state = {k: v.detach().clone() for k, v in model.state_dict().items()}
    backend = GB300Backend(model, [f"l{i}" for i in range(12)])
    srv = Server({"HCA": backend}, "tok", slots=3)
    srv.start()
    yield srv, state
    srv.shutdown()


def _oracle(state):
    from ffnoml_gb300.config import species_of
    from oracle.ffno_oracle import OracleFFNO3D
    cfg = dict(width=32, n_layers=2, hidden_spectral=32, hidden_vertical=32, z_min_wavelength=40.0 / 15,
               species=species_of(["H", "CA"]), in_channels=6, out_channels=12)
    return OracleFFNO3D(state, cfg, torch.float64)


def test_predict_and_vjp_match_the_oracle(served):
    from ffnoml_gb300.service import Client
    srv, state = served
    c = Client(srv.port, "tok")
    f, z = _request((16, 12, 10), 1)
    pop = c.request("PREDICT", "HCA", f, z, 48e3, 48e3, 12)
    orc = _oracle(state)
    ft = torch.from_numpy(f).double()[None].requires_grad_(True)
    zt = torch.from_numpy(z).double()[None].requires_grad_(True)
    ref = orc.forward_si(ft, zt, 48e3, 48e3)[0].permute(1, 2, 3, 0)
    rel = np.abs(pop / ref.detach().numpy() - 1).max()
    assert rel < 1e-4, rel                                 # |d log10 n| ~ 4e-5
    cot = np.random.default_rng(2).normal(size=pop.shape).astype(np.float32) / pop
    out = c.request("VJP", "HCA", f, z, 48e3, 48e3, 12, cot)
    fb, zb = torch.autograd.grad(ref, (ft, zt), torch.from_numpy(cot).double())
    fb = fb[0].numpy()
    for ch in range(6):
        e = np.abs(out["features"][ch] - fb[ch]).max() / np.abs(fb[ch]).max()
        assert e < 1e-3, (ch, e)
    assert np.abs(out["z_scale"] - zb[0].numpy()).max() / np.abs(zb[0].numpy()).max() < 1e-2
    c.close()


def test_results_are_the_same_alone_and_in_a_mix(served):
    from ffnoml_gb300.service import Client
    srv, _ = served
    shapes = [(24, 16, 16), (16, 32, 32), (32, 8, 24), (8, 16, 8)]
    reqs = [_request(s, 10 + i) for i, s in enumerate(shapes)]
    alone = []
    c = Client(srv.port, "tok")
    for f, z in reqs:
        alone.append(c.request("PREDICT", "HCA", f, z, 48e3, 48e3, 12))
    c.close()
    mixed = [None] * len(reqs)

    def run(i):
        cl = Client(srv.port, "tok")
        for _ in range(2):
            mixed[i] = cl.request("PREDICT", "HCA", reqs[i][0], reqs[i][1], 48e3, 48e3, 12)
        cl.close()

    ts = [threading.Thread(target=run, args=(i,)) for i in range(len(reqs))]
    [t.start() for t in ts]
    [t.join() for t in ts]
    for a, b in zip(alone, mixed):
        assert np.array_equal(a, b)


@pytest.fixture(scope="module")
def served_bf16():
    from ffnoml_gb300.runtime import GB300Backend
    from ffnoml_gb300.service import Server
    backend = GB300Backend(_model("bf16"), [f"l{i}" for i in range(12)])
    srv = Server({"HCA": backend}, "tok", slots=4)
    srv.start()
    yield srv
    srv.shutdown()


def test_bf16_results_are_the_same_alone_and_in_a_mix(served_bf16):
    """The service's default precision (split-BF16 tensor cores): PREDICT and VJP requests of uneven sizes give the
    same bits alone and while other requests run on the device beside them (each request has its own workspace and
    the kernels' reductions run in a fixed order)."""
    from ffnoml_gb300.service import Client
    srv = served_bf16
    shapes = [(40, 32, 32), (24, 48, 40), (64, 16, 24), (16, 24, 16), (32, 40, 40)]
    reqs = []
    for i, s in enumerate(shapes):
        f, z = _request(s, 30 + i)
        op = "VJP" if i % 2 else "PREDICT"
        cot = (np.random.default_rng(40 + i).normal(size=s + (12,)) * 1e-15).astype(np.float32) if op == "VJP" else None
        reqs.append((op, f, z, cot))

    def ask(cl, op, f, z, cot):
        out = cl.request(op, "HCA", f, z, 48e3, 48e3, 12, cot)
        return [out] if op == "PREDICT" else [out["features"], out["z_scale"]]

    c = Client(srv.port, "tok")
    alone = [ask(c, *r) for r in reqs]
    c.close()
    mixed = [None] * len(reqs)

    def run(i):
        cl = Client(srv.port, "tok")
        for _ in range(3):
            mixed[i] = ask(cl, *reqs[i])
        cl.close()

    ts = [threading.Thread(target=run, args=(i,)) for i in range(len(reqs))]
    [t.start() for t in ts]
    [t.join() for t in ts]
    for i, (a, b) in enumerate(zip(alone, mixed)):
        for x, y in zip(a, b):
            assert np.array_equal(x, y), (i, reqs[i][0])
