"""A forward through tables reloaded from the on-disk store equals one through freshly built tables, bit for bit."""
import pytest
import torch

from golden_io import load, model_config

pytestmark = pytest.mark.gpu


def _model(meta, state, store):
    from ffnoml_gb300 import FFNO3D
    m = FFNO3D(**model_config(meta))
    m.load_state_dict({k: v.float() for k, v in state.items()}, strict=True)
    m = m.cuda().eval()
    m.executor().tables = store
    return m


@pytest.mark.parametrize("name", ["hca_stretched", "w32_m16"])
def test_forward_with_reloaded_tables(name, tmp_path):
    from ffnoml_gb300.table_store import NoStore, TableStore
    meta, state, a = load(name)
    x, z = a["x"].float().cuda(), a["z"].float().cuda()
    with torch.no_grad():
        y0 = _model(meta, state, NoStore())(x, z, meta["dx"], meta["dy"])
        s1 = TableStore(tmp_path)
        y1 = _model(meta, state, s1)(x, z, meta["dx"], meta["dy"])
        s2 = TableStore(tmp_path)
        y2 = _model(meta, state, s2)(x, z, meta["dx"], meta["dy"])
    assert s1.builds > 0 and s1.hits == 0
    assert s2.builds == 0 and s2.hits == s1.builds
    assert torch.equal(y0, y1) and torch.equal(y1, y2)
