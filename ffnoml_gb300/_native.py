"""ctypes binding of libffnoml_gb300.so (the C ABI declared in include/ffnoml_gb300.h).

The library is built in-tree by ffnoml_gb300.build (or __graft_entry__.build()). There is no fallback: if the library
is missing or fails to load, every operation raises.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libffnoml_gb300.so")

P = ctypes.c_void_p
I = ctypes.c_int
L = ctypes.c_long
F = ctypes.c_float
D = ctypes.c_double

FFNO_MAX_LEVELS = 32
FFNO_MAX_SPECIES = 4

ERRORS = {1: "invalid argument", 2: "kernel launch failed", 3: "workspace too small", 4: "device wait timed out",
          5: "request exceeds the fixed capacity of a non-allocating entry point"}


class HeadParams(ctypes.Structure):
    _fields_ = [
        ("nspecies", I),
        ("levels", I * FFNO_MAX_SPECIES),
        ("rho_channel", I), ("temperature_channel", I), ("ne_channel", I),
        ("in_channels", I),
        ("total_bound", F),
        ("log10_particle_mass", F * FFNO_MAX_SPECIES),
        ("mean_x", F * 8), ("std_x", F * 8),
        ("mean_y", F * FFNO_MAX_LEVELS), ("std_y", F * FFNO_MAX_LEVELS),
        ("log_g", D * FFNO_MAX_LEVELS), ("ev", D * FFNO_MAX_LEVELS), ("ndxi", D * FFNO_MAX_LEVELS),
        ("dion", D * FFNO_MAX_LEVELS),
        ("math32", I),
    ]


class XformDesc(ctypes.Structure):
    _fields_ = [
        ("nb", L), ("nb2", L),
        ("in_b1", L), ("in_b2", L), ("out_b1", L), ("out_b2", L),
        ("K", I), ("M", I),
        ("N", L),
        ("in_split", I),
        ("in_hi", L), ("in_lo", L),
        ("out_split", I),
        ("out_hi", L), ("out_lo", L),
    ]


# name -> argument types (all return int status)
PROTOTYPES = {
    "ffno_stats_parts": [L],
    "ffno_depth_weights": [P, I, L, P, P],
    "ffno_column_info": [P, I, L, P, P],
    "ffno_lift_fwd": [P, I, L, I, P, P, P, P, I, I, P],
    "ffno_gn_finalize": [P, I, I, I, P, P, F, P, P, P],
    "ffno_gn_act": [P, P, L, I, I, P, P],
    "ffno_gate_fwd": [P, L, I, P, P, P, P, P, P],
    "ffno_mlp2_fwd": [I, P, P, P, F, P, L, I, P, P, P, P, P, I, I, P],
    "ffno_fuse_fwd": [P, P, P, P, P, L, I, P, P, P, P, P, P, P, P, I, I, P],
    "ffno_resid_out": [P, P, P, F, L, I, P, P],
    "ffno_head_fwd": [P, P, L, I, P, P, P, I, I, ctypes.POINTER(HeadParams), P, P, P],
    "ffno_xform": [P, P, P, ctypes.POINTER(XformDesc), I, P],
    "ffno_xform_pt": [P, L, P, P, ctypes.POINTER(XformDesc), I, P],
    "ffno_col_outer": [P, I, P, I, L, I, L, P, I, P],
    "ffno_percol_tables": [P, I, L, P, I, P, P, P, P, P, P],
    "ffno_percol_tables_vjp": [P, I, L, P, I, P, P, P, P, P, P, P],
    "ffno_column_tables_vjp": [P, I, P, I, P, P, I, P, P, P, P, L, P],
    "ffno_spectral_mix": [P, P, L, L, L, L, L, I, P, P, P, P, I, P],
    "ffno_gn_bwd_stats": [I, P, F, P, P, P, P, L, I, I, P, I, P],
    "ffno_gn_bwd_final": [P, I, I, P, P],
    "ffno_gn_bwd_apply": [I, P, F, P, P, P, P, P, P, L, I, I, F, P, P, P],
    "ffno_mlp2_bwd": [P, P, P, L, I, P, P, P, P, P],
    "ffno_fuse_bwd": [P, P, P, P, P, P, P, L, I, P, P, P, P, P, P, P, P, P, P, P, P],
    "ffno_gate_bwd": [P, P, P, P, L, I, P, P, P, P, P, P, P, P, P, P, P, P],
    "ffno_lift_bwd": [P, I, L, I, P, P, P],
    "ffno_head_bwd": [P, P, P, L, I, P, P, P, P, P, I, ctypes.POINTER(HeadParams), P, P, P],
    "ffno_depth_weights_bwd": [P, P, I, L, P, P],
    "ffno_proj_fwd": [P, L, I, P, P, P, I, I, P, P],
    "ffno_head_output": [P, P, L, I, ctypes.POINTER(HeadParams), P, P],
    "ffno_proj_bwd": [P, P, L, I, P, P, P, P, P, I, I, P, P],
    "ffno_head_output_bwd": [P, P, P, L, I, ctypes.POINTER(HeadParams), P, P, P],
    "ffno_outer_parts": [I, I, L],
    "ffno_outer": [P, L, I, P, L, I, L, P, I, P, I, P],
    "ffno_outer_noalloc": [P, L, I, P, L, I, L, P, I, P],
    "ffno_si_inputs": [P, P, L, P, P, P, P, P, P],
    "ffno_si_populations": [P, L, I, P, P, P, P, P],
    "ffno_si_population_cotangent": [P, P, L, I, P, P, P, P, P],
    "ffno_si_input_grads": [P, P, P, L, P, P, P, P, P],
    "ffno_tc_selftest": [P, P, I, I, I, P, P, P],
    "ffno_tc_parts": [L],
    "ffno_tc_width_supported": [I],
    "ffno_tc_channel_width_supported": [I],
    "ffno_fuse_hidden_tc": [P, P, P, P, P, L, I, P, P, P, P],
    "ffno_fuse_out_tc": [P, P, P, P, P, P, L, I, P, P, P, P, I, I, P, P],
    "ffno_fuse_bwd_h_tc": [P, P, L, I, P, P, P, P],
    "ffno_fuse_bwd_q_tc": [P, P, P, P, P, P, P, L, I, P, P, P, P, P, P],
    "ffno_fuse_bwd_x_tc": [P, P, P, L, I, P, P, P, P, P, P],
    "ffno_tc_set_prefetch_tiles": [I],
    "ffno_copy2d": [P, L, P, L, L, L, P],
    "ffno_reverse_axes4": [P, L, L, L, L, P, P],
    "ffno_shear_levels": [P, I, L, L, P, P, P, P, I, P, P],
    "ffno_mesh_refine": [P, L, I, D, D, D, D, D, P, P],
    "ffno_mesh_features": [P, P, L, I, P, I, I, P, P, P],
    "ffno_mesh_features_vjp": [P, P, L, I, P, I, I, P, P, P, P, P],
    "ffno_mesh_features_jvp": [P, P, L, I, P, I, I, P, P, P, P],
    "ffno_mesh_backmap": [P, P, I, P, L, I, I, P, P],
    "ffno_mesh_backmap_vjp": [P, P, I, P, L, I, I, P, P, P, P],
    "ffno_mesh_backmap_jvp": [P, P, P, I, P, L, I, I, P, P],
    "ffno_mlp2_fwd_tc": [I, P, P, P, F, P, L, I, P, P, P, P, I, I, P, P],
    "ffno_gate_fwd_tc": [P, L, I, P, P, P, P, P, P],
    "ffno_fuse1_tc": [P, P, P, P, P, L, I, P, P, P, P, P, P],
    "ffno_fuse2_tc": [P, P, P, P, P, L, I, P, P, P, P, I, I, P, P],
    "ffno_mlp2_bwd_tc": [P, P, P, L, I, P, P, P, P],
    "ffno_gate_bwd_tc": [P, P, P, L, I, P, P, P, P, P, P],
    "ffno_fuse_bwd_a_tc": [P, P, P, P, P, P, L, I, P, P, P, P],
    "ffno_fuse_bwd_b_tc": [P, P, P, P, P, P, P, P, P, L, I, P, P, P, P, P, P],
    "ffno_outer_tc": [P, L, I, P, L, I, L, P, I, P, I, P, P],
    "ffno_outer_tc_ld": [P, L, I, P, L, I, L, P, I, P, L, I, P, P],
    "ffno_head_fwd_tc": [P, P, L, I, P, P, I, I, ctypes.POINTER(HeadParams), P, P, P, P],
    "ffno_head_bwd_tc": [P, P, P, L, I, P, P, I, ctypes.POINTER(HeadParams), P, P, P, P],
    "ffno_gn_jvp_stats": [P, P, P, P, L, I, I, P, I, P],
    "ffno_gn_jvp_apply": [P, P, P, P, P, P, I, P, F, L, I, I, P, P],
    "ffno_gate_jvp": [P, P, L, I, P, P, P, P],
    "ffno_mlp2_jvp": [P, P, L, I, P, P, P, P],
    "ffno_fuse_jvp": [P, P, P, P, P, P, P, P, L, I, P, P, P, P, P, P, P],
    "ffno_head_jvp": [P, P, P, P, L, I, P, P, P, I, ctypes.POINTER(HeadParams), P, P],
    "ffno_si_input_tangent": [P, P, L, P, P, P, P],
    "ffno_si_population_tangent": [P, P, L, I, P, P, P, P, P],
    "ffno_xform_tc_pack_bytes": [I, I],
    "ffno_xform_tcr_max_table_bytes": [],
    "ffno_xform_tcr": [P, I, I, P, P, ctypes.POINTER(XformDesc), I, P, P],
    "ffno_xform_tc": [P, P, P, ctypes.POINTER(XformDesc), I, P, P],
    "ffno_spectral_mix_tc": [P, P, L, L, L, L, L, I, P, P, P, P, I, P, P],
}

_lib = None


class NativeError(RuntimeError):
    pass


def lib():
    """The loaded library; raises if it was not built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise NativeError(f"{LIB_PATH} is missing: build it with `python -m ffnoml_gb300.build` "
                              "(or __graft_entry__.build()); ffnoml_gb300 has no fallback path")
        handle = ctypes.CDLL(LIB_PATH)
        for name, args in PROTOTYPES.items():
            fn = getattr(handle, name)
            fn.argtypes = args
            fn.restype = I
        handle.ffno_version.restype = ctypes.c_char_p
        handle.ffno_version.argtypes = []
        _lib = handle
    return _lib


class _Counter:
    """Launch accounting: number of entry-point calls, and optional per-call CUDA-event timing (for the benchmark's
    kernel breakdown)."""

    def __init__(self):
        self.calls = 0
        self.timing = None      # list of (name, start_event, end_event) while timing is on


counter = _Counter()


def call(name, *args, tag=None):
    """Call an entry point and raise on a non-zero status. tag names the call site in the timing breakdown."""
    counter.calls += 1
    if counter.timing is not None:
        import torch
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        status = getattr(lib(), name)(*args)
        b.record()
        counter.timing.append((name + (":" + tag if tag else ""), a, b, args))
    else:
        status = getattr(lib(), name)(*args)
    if status:
        raise NativeError(f"{name} failed: {ERRORS.get(status, status)} (status {status})")
    return status


def exported_symbols():
    return list(PROTOTYPES) + ["ffno_version"]
