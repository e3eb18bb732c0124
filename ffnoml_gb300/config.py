"""Model and atom constants of the path (harshmathur1990/FFNOML config.py:150-220, 294-311): the level-fraction data of
the H and Ca II atoms and the final (zaug) model's defaults."""
import math

ATOM_CONFIG = {
    "H": {
        "levels": 6,
        "log10_particle_mass": float(math.log10(2.2697e-27)),  # kg
        "multi3d_lte": dict(g=[2.0, 8.0, 18.0, 32.0, 50.0, 1.0], ion=[1, 1, 1, 1, 1, 2],
                            ev=[0.0, 10.198673740091325, 12.087318311066094, 12.748311674749516, 13.054262568222963,
                                13.60794573029334]),
    },
    "CA": {
        "levels": 6,
        "log10_particle_mass": float(math.log10(1.0375e-21)),  # kg
        "multi3d_lte": dict(g=[2.0, 4.0, 6.0, 2.0, 4.0, 1.0], ion=[2, 2, 2, 2, 2, 3],
                            ev=[0.0, 1.69242903005873, 1.6999489817497997, 3.12337806212316, 3.151018087686871,
                                11.87181686885173]),
    },
}

MODEL_CONFIG = dict(
    in_channels=6,
    out_channels=6,
    width=96,
    n_layers=4,
    dropout=0.0,
    spec_dropout=0.08,
    vertical_dropout=0.08,
    spec_dropout_layers=[0, 1, 2, 3],
    vertical_dropout_layers=[0, 1, 2, 3],
    hidden_spectral=128,
    hidden_vertical=128,
    checkpoint_blocks=True,
    freq_mix_rank=8,
    z_reference_length=40.0,
    z_min_wavelength=0.04,
    z_feature_wavelength=0.3,
    species=[{k: ATOM_CONFIG["H"][k] for k in ("levels", "log10_particle_mass", "multi3d_lte")}],
)


def species_of(atoms):
    return [{k: ATOM_CONFIG[a][k] for k in ("levels", "log10_particle_mass", "multi3d_lte")} for a in atoms]
