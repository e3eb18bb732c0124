"""Loading helpers for the golden fixtures in tests/golden/ (written by tests/golden/make_golden.py)."""
import json
import math
import os

import numpy as np
import torch

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ("h_uniform", "hca_stretched", "per_column", "tall_box", "batch2", "w32_m16", "w64_m32")

# config.ATOM_CONFIG's level-fraction data (harshmathur1990/FFNOML config.py:150-220)
ATOMS = {
    "H": dict(levels=6, log10_particle_mass=math.log10(2.2697e-27),
              multi3d_lte=dict(g=[2.0, 8.0, 18.0, 32.0, 50.0, 1.0], ion=[1, 1, 1, 1, 1, 2],
                               ev=[0.0, 10.198673740091325, 12.087318311066094, 12.748311674749516,
                                   13.054262568222963, 13.60794573029334])),
    "CA": dict(levels=6, log10_particle_mass=math.log10(1.0375e-21),
               multi3d_lte=dict(g=[2.0, 4.0, 6.0, 2.0, 4.0, 1.0], ion=[2, 2, 2, 2, 2, 3],
                                ev=[0.0, 1.69242903005873, 1.6999489817497997, 3.12337806212316, 3.151018087686871,
                                    11.87181686885173])),
}


def load(name):
    data = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(str(data["meta"]))
    state = {k[len("state/"):]: torch.from_numpy(data[k]) for k in data.files if k.startswith("state/")}
    arrays = {k: torch.from_numpy(data[k]) for k in data.files if not k.startswith("state/") and k != "meta"}
    return meta, state, arrays


def model_config(meta):
    cfg = dict(meta["config"] if "config" in meta else meta)
    atoms = cfg.pop("atoms")
    cfg["species"] = [ATOMS[a] for a in atoms]
    cfg["in_channels"] = 6
    cfg["out_channels"] = sum(s["levels"] for s in cfg["species"])
    return cfg
