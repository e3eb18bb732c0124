"""MULTI3D LTE level tables for the level-fraction head (models/ffno_model.py:111-128, MULTI3D calc_lte_populations):
per level ln(g_i/g_1), E_i [eV], the Debye-lowering stage multiple ndxi(ion_i) and ion_i - ion_1."""
import math

# MULTI3D constants, cgs (models/ffno_model.py:111-112)
EE, HH, EM, BK, PI_M3D = 1.602189e-12, 6.626176e-27, 9.109534e-28, 1.380662e-16, 3.14159265359


def tables(atom, levels):
    g = [float(v) for v in atom["g"]]
    ev = [float(v) for v in atom["ev"]]
    ion = [int(v) for v in atom["ion"]]
    if not len(g) == len(ev) == len(ion) == levels:
        raise ValueError(f"multi3d_lte atom data has {len(g)}, {len(ev)}, {len(ion)} entries for {levels} levels")
    # cumulative stage offsets 0, 0, 1, 3, 6, ...; MULTI3D subtracts the first level's entry in a loop that zeroes that
    # entry on the way, so stages above the first level's keep their absolute values
    stage = [0] * 21
    for i in range(2, 21):
        stage[i] = stage[i - 1] + (i - 1)
    first = stage[ion[0]]
    stage = [s - first if i <= ion[0] else s for i, s in enumerate(stage)]
    return ([math.log(v / g[0]) for v in g], ev, [float(stage[i]) for i in ion],
            [float(max(i - ion[0], 0)) for i in ion])
