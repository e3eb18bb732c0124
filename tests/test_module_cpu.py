"""The drop-in module's parameter tree, constructor checks and seeded initialisation against the reference's."""
import pytest
import torch

from golden_io import ATOMS, load, model_config
from ffnoml_gb300 import FFNO3D, create_ffno3d


def test_state_dict_matches_reference_keys_and_shapes():
    meta, state, _ = load("hca_stretched")
    model = FFNO3D(**model_config(meta))
    sd = model.state_dict()
    assert list(sd) == list(state)
    assert all(tuple(sd[k].shape) == tuple(state[k].shape) for k in sd)
    model.load_state_dict({k: v.float() for k, v in state.items()}, strict=True)


def test_seeded_init_equals_reference():
    # the fixtures were built by torch.manual_seed(seed) + the reference constructor; only freq_u and the total rows
    # of proj2 were perturbed afterwards
    meta, state, _ = load("h_uniform")
    torch.manual_seed(meta["seed"])
    model = FFNO3D(**model_config(meta))
    for k, v in model.state_dict().items():
        if ".freq_u." in k or k.startswith("proj2") or k in ("mean_X", "std_X", "mean_Y", "std_Y"):
            continue
        assert torch.equal(v, state[k].to(v.dtype)), k


def test_factory_defaults_are_the_final_model():
    m = create_ffno3d(6, 6)
    assert m.width == 96 and m.n_layers == 4 and m.blocks[0].vertical.modes == 1001
    assert m.proj2.out_channels == 7
    m2 = create_ffno3d(6, 12, atoms=["H", "CA"], width=16, n_layers=1)
    assert m2.proj2.out_channels == 14


def test_needs_species_and_matching_levels():
    with pytest.raises(ValueError):
        FFNO3D(out_channels=6, width=16, n_layers=1)
    with pytest.raises(ValueError):
        FFNO3D(out_channels=12, species=[ATOMS["H"]], width=16, n_layers=1)


def test_cpu_tensors_are_refused():
    m = create_ffno3d(6, 6, width=16, n_layers=1, hidden_spectral=16, hidden_vertical=16)
    x = torch.zeros(1, 6, 4, 4, 4)
    z = torch.zeros(1, 4, 4, 4)
    with pytest.raises(RuntimeError):
        m(x, z, 48e3, 48e3)


def test_diagnostic_arguments_are_outside_the_path():
    m = create_ffno3d(6, 6, width=16, n_layers=1, hidden_spectral=16, hidden_vertical=16)
    with pytest.raises(NotImplementedError):
        m(torch.zeros(1, 6, 4, 4, 4), torch.zeros(1, 4, 4, 4), 48e3, 48e3, collect_stats=True)
