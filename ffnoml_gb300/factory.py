"""create_ffno3d, the drop-in for ffno_model_factory.create_ffno3d (harshmathur1990/FFNOML ffno_model_factory.py:6-19)."""
from .config import MODEL_CONFIG, species_of
from .model import FFNO3D


def create_ffno3d(Cin, Cout, device="cpu", atoms=None, **overrides):
    """FFNO3D from MODEL_CONFIG + overrides; atoms (e.g. ["CA"]) picks the level-fraction head's species. The module is
    built on the CPU, as the reference's is; move it with .to(device) / .cuda()."""
    configuration = dict(MODEL_CONFIG)
    configuration.update(overrides)
    if atoms is not None:
        configuration["species"] = species_of(atoms)
    configuration["in_channels"] = int(Cin)
    configuration["out_channels"] = int(Cout)
    return FFNO3D(**configuration)
