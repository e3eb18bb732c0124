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


# ------------------------------------------------------------------------------------------------ recipe fixtures
# The fixtures at the benchmark configurations hold only the reference's outputs. Their weights and inputs come from
# the integer-hash recipe below, which gives the same float32 values on any machine and any numpy / torch version:
# SplitMix64 (S. Vigna's generator, as in java.util.SplittableRandom) over a per-element counter, uniforms from its
# top 53 bits, and only IEEE additions, multiplications and divisions after that (no transcendental function, whose
# last bit may differ between platforms). Normal-like values are Irwin-Hall sums of four uniforms, scaled to unit
# variance. tests/golden/make_golden.py loads the same values into the reference's FFNO3D.

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(x):
    with np.errstate(over="ignore"):
        z = x + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def recipe_uniform(seed, stream, n):
    """n uniforms in [0, 1) (float64) of counter stream `stream` under `seed`."""
    with np.errstate(over="ignore"):
        base = _splitmix64(np.uint64(seed) * np.uint64(0x632BE59BD9B4E019) + np.uint64(stream) * np.uint64(0x9E3779B1))
        h = _splitmix64(base + np.arange(n, dtype=np.uint64))
    return (h >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def recipe_normal(seed, stream, n):
    """n values of zero mean and unit variance: (u1 + u2 + u3 + u4 - 2) * sqrt(3)."""
    u = recipe_uniform(seed, stream, 4 * n).reshape(4, n)
    return ((u[0] + u[1]) + (u[2] + u[3]) - 2.0) * 1.7320508075688772


def _param_values(name, shape, seed, stream):
    n = int(np.prod(shape))
    u = 2.0 * recipe_uniform(seed, stream, n) - 1.0                  # U(-1, 1)
    if name.endswith("weight_real") or name.endswith("weight_imag"):
        a = math.sqrt(3.0 / shape[0])                                 # std 1/sqrt(C), as scale * randn
    elif ".freq_u." in name:
        a = 0.1 * math.sqrt(3.0)                                      # the low-rank U made live, std 0.1
    elif len(shape) >= 2:
        a = 1.0 / math.sqrt(int(np.prod(shape[1:])))                  # nn.Conv3d / nn.Linear init bound
    elif name.endswith("res_fused") or name.endswith("res_pw") or name.endswith("res_mlp"):
        init = 1.0 if name.endswith("res_fused") else 0.5
        return (init * (1.0 + 0.2 * u)).reshape(shape)
    elif ("norm_" in name or name.startswith("lift.1.")) and name.endswith(".weight"):
        return (1.0 + 0.2 * u).reshape(shape)                         # GroupNorm gamma near 1
    else:
        a = 0.1                                                       # biases, GroupNorm beta
    return (a * u).reshape(shape)


def recipe_state(named_shapes, seed):
    """float32 values for every parameter {name: shape} of an FFNO3D (sorted by name, one counter stream each)."""
    out = {}
    for i, name in enumerate(sorted(named_shapes)):
        out[name] = _param_values(name, tuple(named_shapes[name]), seed, 1000 + i).astype(np.float32)
    return out


def recipe_digest(state):
    """SHA-256 of the recipe values (sorted names, float32 bytes): the fixture records it, the tests check it."""
    import hashlib
    h = hashlib.sha256()
    for name in sorted(state):
        h.update(name.encode())
        h.update(np.ascontiguousarray(state[name], dtype=np.float32).tobytes())
    return h.hexdigest()


MEAN_X = np.array([4.75, 0.0, 0.0, 0.0, 17.5, -8.0], np.float64)
STD_X = np.array([2.5 / math.sqrt(12), 5.0, 5.0, 5.0, 7.0 / math.sqrt(12), 8.0 / math.sqrt(12)], np.float64)


def recipe_inputs(shape, seed):
    """Normalised inputs [1, 6, D, H, W] (float32 values, as float64) of the synthetic distributions: log10 T ~
    U(3.5, 6), v ~ 5 km/s x unit-variance, log10 ne ~ U(14, 21), log10 rho ~ U(-12, -4), z-scored with their
    analytic moments; heights z = linspace(14, -1, D) Mm per column, top first, as float32 values."""
    _, _, D, H, W = shape
    V = D * H * W
    raw = np.empty((6, V))
    raw[0] = 3.5 + 2.5 * recipe_uniform(seed, 1, V)
    for c in (1, 2, 3):
        raw[c] = 5.0 * recipe_normal(seed, 1 + c, V)
    raw[4] = 14.0 + 7.0 * recipe_uniform(seed, 5, V)
    raw[5] = -12.0 + 8.0 * recipe_uniform(seed, 6, V)
    x = ((raw - MEAN_X[:, None]) / STD_X[:, None]).astype(np.float32).astype(np.float64)
    col = np.array([14.0 - 15.0 * d / (D - 1) for d in range(D)], np.float32).astype(np.float64)
    z = np.broadcast_to(col[:, None, None], (D, H, W))[None].copy()
    return x.reshape(1, 6, D, H, W), z


def recipe_cotangent(shape, levels, seed):
    """A unit-variance cotangent on the normalised output [1, levels, D, H, W] (float32 values, as float64)."""
    _, _, D, H, W = shape
    n = levels * D * H * W
    return recipe_normal(seed, 7, n).astype(np.float32).astype(np.float64).reshape(1, levels, D, H, W)


def recipe_normalisation(levels):
    """mean_Y, std_Y of the recipe fixtures (the same as the other fixtures')."""
    return np.linspace(0.5, 1.5, levels), np.linspace(1.0, 2.0, levels)


def recipe_model(meta, device="cuda"):
    """The drop-in FFNO3D of a recipe fixture, with the recipe's weights (checked against the fixture's digest)."""
    from ffnoml_gb300 import FFNO3D
    cfg = model_config(meta)
    model = FFNO3D(**cfg)
    state = recipe_state({k: tuple(p.shape) for k, p in model.named_parameters()}, meta["seed"])
    if recipe_digest(state) != meta["digest"]:
        raise AssertionError("the weight recipe does not reproduce the fixture's weights on this machine")
    with torch.no_grad():
        for k, p in model.named_parameters():
            p.copy_(torch.from_numpy(state[k]))
    mean_y, std_y = recipe_normalisation(cfg["out_channels"])
    model.set_normalization(MEAN_X.astype(np.float32), STD_X.astype(np.float32), mean_y, std_y)
    return model.eval().to(device)


def recipe_arrays(meta):
    """Inputs and cotangent of a recipe fixture (float64 tensors holding float32 values)."""
    shape = meta["shape"]
    x, z = recipe_inputs(shape, meta["seed"] + 1)
    L = model_config(meta)["out_channels"]
    cot = recipe_cotangent(shape, L, meta["seed"] + 2)
    return torch.from_numpy(x), torch.from_numpy(z), torch.from_numpy(cot)


RECIPE_CASES = ("cfg0", "cfg1_sub", "w96_p_d64", "w96_p_d256", "w64_p_d256")


def load_recipe(name):
    """(meta, arrays) of a recipe fixture: the reference's outputs plus the recipe's inputs x, z and cotangent cot."""
    data = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(str(data["meta"]))
    arrays = {k: torch.from_numpy(data[k]) for k in data.files if k != "meta"}
    arrays["x"], arrays["z"], arrays["cot"] = recipe_arrays(meta)
    return meta, arrays


def recipe_fp32_bound(meta):
    """The FP32 path's bound on max |d log10 n| against float64: 1e-5, or 1.5 x the reference's own FP32 error where
    that exceeds 1e-5 (the production height operator at D = 256)."""
    return max(1e-5, 1.5 * meta["env32"])
