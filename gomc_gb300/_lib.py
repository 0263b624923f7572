"""ctypes binding of the C ABI in include/gomc_gb300.h.

The library is the in-tree ``gomc_gb300/_build/libgomc_gb300.so`` built by
``gomc_gb300.build``.  There is no fallback: if the library is missing or
cannot load, :func:`lib` raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

_LIB = None

STATUS = {0: "GB_OK", 1: "GB_ERR_ARG", 2: "GB_ERR_CUDA", 3: "GB_ERR_NOMEM",
          4: "GB_ERR_CAPACITY", 5: "GB_ERR_TIMEOUT", 6: "GB_ERR_STATE",
          7: "GB_ERR_UNSUPPORTED"}

GB_FP64 = 0
GB_MIXED = 1


class GbError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("%s: %s" % (STATUS.get(code, code), msg))
        self.code = code


class SystemDesc(C.Structure):
    _fields_ = [("n_atoms", C.c_int32), ("n_mol", C.c_int32),
                ("n_kinds", C.c_int32),
                ("pos", C.POINTER(C.c_double)),
                ("atom_kind", C.POINTER(C.c_int32)),
                ("atom_charge", C.POINTER(C.c_double)),
                ("mol_start", C.POINTER(C.c_int32)),
                ("kind_epsilon", C.POINTER(C.c_double)),
                ("kind_sigma", C.POINTER(C.c_double)),
                ("kind_n", C.POINTER(C.c_double)),
                ("box", C.c_double * 3)]


class Config(C.Structure):
    _fields_ = [("temperature", C.c_double), ("rcut", C.c_double),
                ("rcut_low", C.c_double), ("rcut_coulomb", C.c_double),
                ("tolerance", C.c_double), ("ewald", C.c_int32),
                ("electrostatic", C.c_int32), ("precision", C.c_int32),
                ("device", C.c_int32), ("sc_alpha", C.c_double),
                ("sc_sigma", C.c_double), ("sc_power", C.c_int32),
                ("sc_coul", C.c_int32)]


class McParams(C.Structure):
    _fields_ = [("seed", C.c_uint32), ("frac", C.c_double * 3),
                ("adj_steps", C.c_int32), ("use_scales", C.c_int32),
                ("scales", C.c_double * 4), ("recompute_freq", C.c_int32),
                ("cluster_size", C.c_int32), ("flush_every", C.c_int32),
                ("move_buffer", C.c_int32), ("unit_lanes", C.c_int32),
                ("grid_ctas", C.c_int32), ("writer_kchunk", C.c_int32),
                ("moves_in_flight", C.c_int32)]


class McShape(C.Structure):
    _fields_ = [("ctas", C.c_int32), ("unit_lanes", C.c_int32),
                ("writer_kchunk", C.c_int32), ("moves_in_flight", C.c_int32),
                ("max_concurrent", C.c_int32),
                ("us_per_move", C.c_double)]


class ServerConfig(C.Structure):
    _fields_ = [("device", C.c_int32), ("quantum", C.c_int32),
                ("mem_budget", C.c_int64), ("max_resident", C.c_int32)]


# every function the header declares: name -> (restype, argtypes)
class GemcDesc(C.Structure):
    """gb_gemc_desc (include/gomc_gb300.h)."""
    _fields_ = [("n0", C.c_int32), ("n1", C.c_int32),
                ("pos0", C.POINTER(C.c_double)),
                ("pos1", C.POINTER(C.c_double)),
                ("box0", C.c_double * 3), ("box1", C.c_double * 3),
                ("epsilon", C.c_double), ("sigma", C.c_double),
                ("n_mie", C.c_double)]


class GemcConfig(C.Structure):
    """gb_gemc_config (include/gomc_gb300.h)."""
    _fields_ = [("temperature", C.c_double), ("rcut", C.c_double),
                ("rcut_low", C.c_double), ("frac", C.c_double * 3),
                ("adj_steps", C.c_int32), ("cbmc_first", C.c_int32),
                ("precision", C.c_int32), ("device", C.c_int32),
                ("cluster_size", C.c_int32), ("seed", C.c_uint32)]


B2, M16, MP2 = 2, 16, 2


class GomcChk(C.Structure):
    """gb_gomc_chk (include/gomc_gb300.h): the Monte Carlo loop state of a
    GOMC checkpoint file (src/Checkpoint.h)."""
    _fields_ = [("step", C.c_uint64), ("true_step", C.c_uint64),
                ("mt_state", C.c_uint32 * 624), ("mt_left", C.c_uint32),
                ("seed_location", C.c_uint32), ("seed_left", C.c_uint32),
                ("seed_value", C.c_uint32),
                ("n_box", C.c_int32), ("n_move", C.c_int32),
                ("n_kind", C.c_int32),
                ("scale", (C.c_double * M16) * B2),
                ("accept_percent", (C.c_double * M16) * B2),
                ("accepted", (C.c_uint32 * M16) * B2),
                ("tries", (C.c_uint32 * M16) * B2),
                ("temp_accepted", (C.c_uint32 * M16) * B2),
                ("temp_tries", (C.c_uint32 * M16) * B2),
                ("mp_tries", (C.c_uint32 * MP2) * B2),
                ("mp_accepted", (C.c_uint32 * MP2) * B2),
                ("mp_interval_accepted", (C.c_uint32 * MP2) * B2),
                ("mp_interval_tries", (C.c_uint32 * MP2) * B2),
                ("mp_t_max", C.c_double * B2), ("mp_r_max", C.c_double * B2),
                ("single_move_accepted", C.c_int32 * B2),
                ("records_offset", C.c_int64)]


_P = C.c_void_p
_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int32)
_L = C.POINTER(C.c_int64)
SIGNATURES = {
    "gb_version": (C.c_char_p, []),
    "gb_last_error": (C.c_char_p, [_P]),
    "gb_box_create": (C.c_int, [C.POINTER(SystemDesc), C.POINTER(Config),
                                C.POINTER(_P)]),
    "gb_box_destroy": (None, [_P]),
    "gb_system_total": (C.c_int, [_P, _D]),
    "gb_box_inter": (C.c_int, [_P, _D, _D]),
    "gb_molecule_inter": (C.c_int, [_P, C.c_int32, _D, _D, _D, _I]),
    "gb_single_molecule_inter": (C.c_int, [_P, C.c_int32, _D, _D]),
    "gb_virial": (C.c_int, [_P, _D]),
    "gb_checkpoint_size": (C.c_int, [_P, _L]),
    "gb_checkpoint_save": (C.c_int, [_P, _P, C.c_int64]),
    "gb_checkpoint_load": (C.c_int, [_P, _P, C.c_int64]),
    "gb_particle_inter": (C.c_int, [_P, C.c_int32, C.c_int32, _D,
                                    C.c_int32, _D, _D, _I]),
    "gb_cell_remove_mol": (C.c_int, [_P, C.c_int32]),
    "gb_cell_add_mol": (C.c_int, [_P, C.c_int32]),
    "gb_box_force": (C.c_int, [_P, _D, _D, _D, _D]),
    "gb_calculate_torque": (C.c_int, [_P, _D]),
    "gb_num_kvectors": (C.c_int, [_P, _I, _I]),
    "gb_get_kvectors": (C.c_int, [_P, _D]),
    "gb_get_sums_new": (C.c_int, [_P, _D, _D]),
    "gb_box_reciprocal_setup": (C.c_int, [_P]),
    "gb_box_reciprocal_sums": (C.c_int, [_P]),
    "gb_box_reciprocal": (C.c_int, [_P, C.c_int32, _D]),
    "gb_box_reciprocal_sums_coords": (C.c_int, [_P, _D]),
    "gb_box_reciprocal_setup_coords": (C.c_int, [_P, _D]),
    "gb_recip_init": (C.c_int, [_P, _D, _I]),
    "gb_update_recip_vec": (C.c_int, [_P]),
    "gb_set_box": (C.c_int, [_P, _D, _D, _D]),
    "gb_box_edges": (C.c_int, [_P, _D]),
    "gb_box_inter_coords": (C.c_int, [_P, _D, _D, _D, _D]),
    "gb_box_force_coords": (C.c_int, [_P, _D, _D, _D, _D, _D]),
    "gb_swap_self": (C.c_int, [_P, C.c_int32, _D]),
    "gb_swap_correction": (C.c_int, [_P, C.c_int32, _D, _D]),
    "gb_mol_reciprocal": (C.c_int, [_P, C.c_int32, _D, _D]),
    "gb_swap_dest_recip": (C.c_int, [_P, C.c_int32, _D, _D]),
    "gb_swap_source_recip": (C.c_int, [_P, C.c_int32, _D, _D]),
    "gb_update_recip": (C.c_int, [_P]),
    "gb_copy_recip": (C.c_int, [_P]),
    "gb_box_self": (C.c_int, [_P, _D]),
    "gb_mol_correction": (C.c_int, [_P, C.c_int32, _D]),
    "gb_box_force_reciprocal": (C.c_int, [_P, _D, _D]),
    "gb_grid_all": (C.c_int, [_P]),
    "gb_cell_membership": (C.c_int, [_P, _I, _I]),
    "gb_get_coords": (C.c_int, [_P, _D, _D]),
    "gb_set_coords": (C.c_int, [_P, _D, _D]),
    "gb_get_energy": (C.c_int, [_P, _D]),
    "gb_set_energy": (C.c_int, [_P, _D]),
    "gb_mc_init": (C.c_int, [_P, C.POINTER(McParams)]),
    "gb_mc_run": (C.c_int, [_P, C.c_int64, C.c_int64, _I, _I, _I, _D]),
    "gb_mc_state": (C.c_int, [_P, _D, _L]),
    "gb_mc_run_batch": (C.c_int, [C.POINTER(_P), C.c_int32, C.c_int64,
                                  C.c_int64]),
    "gb_mc_timing": (C.c_int, [_P, C.c_int32, _D, _L, _L, _D, _L]),
    "gb_mc_profile": (C.c_int, [_P, C.c_int32, _D, _L]),
    "gb_mc_set_wait_limit": (C.c_int, [_P, C.c_int64]),
    "gb_gomc_checkpoint_read": (C.c_int, [C.c_void_p, C.c_int64,
                                          C.POINTER(GomcChk)]),
    "gb_gomc_checkpoint_write": (C.c_int, [C.c_void_p, C.c_int64,
                                           C.POINTER(GomcChk), C.c_void_p,
                                           C.c_int64, _L]),
    "gb_mc_get_gomc_state": (C.c_int, [_P, C.POINTER(GomcChk)]),
    "gb_mc_set_gomc_state": (C.c_int, [_P, C.POINTER(GomcChk)]),
    "gb_box_stream": (C.c_int, [_P, C.POINTER(_P)]),
    "gb_mc_layout": (C.c_int, [_P, _I, _I, _L]),
    "gb_mc_shape_get": (C.c_int, [_P, C.POINTER(McShape)]),
    "gb_mc_autotune": (C.c_int, [_P, C.c_int32, C.c_int32,
                                 C.POINTER(McShape), C.POINTER(McShape),
                                 C.c_int32, _I]),
    "gb_mc_drift": (C.c_int, [_P, _D, _D, _L]),
    "gb_recip_energy_noalloc": (C.c_int, [_P, _P, _P, C.c_int32, _P, _P]),
    "gb_gemc_create": (C.c_int, [C.POINTER(GemcDesc), C.POINTER(GemcConfig),
                                 C.POINTER(_P)]),
    "gb_gemc_destroy": (None, [_P]),
    "gb_gemc_error": (C.c_char_p, [_P]),
    "gb_gemc_run": (C.c_int, [_P, C.c_int64, C.c_int64, _I, _D]),
    "gb_gemc_state": (C.c_int, [_P, _D, _D, _I, _D, _L, _D]),
    "gb_gemc_coords": (C.c_int, [_P, _D, _D, _I]),
    "gb_gemc_system_total": (C.c_int, [_P, _D]),
    "gb_gemc_profile": (C.c_int, [_P, C.c_int32, _D, _L]),
    "gb_server_create": (C.c_int, [C.POINTER(ServerConfig), C.POINTER(_P)]),
    "gb_server_destroy": (None, [_P]),
    "gb_server_submit": (C.c_int, [_P, C.POINTER(SystemDesc),
                                   C.POINTER(Config), C.POINTER(McParams),
                                   C.c_int64, C.c_int64, _L]),
    "gb_server_estimate": (C.c_int, [_P, C.POINTER(SystemDesc),
                                     C.POINTER(Config), C.POINTER(McParams),
                                     _L, _I]),
    "gb_server_step": (C.c_int, [_P, _I]),
    "gb_server_start": (C.c_int, [_P]),
    "gb_server_drain": (C.c_int, [_P, C.c_double]),
    "gb_server_job": (C.c_int, [_P, C.c_int64, _I, _L, _D]),
    "gb_server_result": (C.c_int, [_P, C.c_int64, _D, _D, _D]),
    "gb_server_stats": (C.c_int, [_P, _D]),
    "gb_server_occupancy": (C.c_int, [_P, _D]),
    "gb_server_error": (C.c_char_p, [_P]),
}

# fixed scratch of gb_recip_energy_noalloc (include/gomc_gb300.h)
RECIP_NOALLOC_MAX_K = 256 * 1024


def lib_path() -> str:
    return _build.LIB


def lib(build_if_missing: bool = False):
    """Load the library (optionally building it first); raise if absent."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError("libgomc_gb300.so is not built (%s); run "
                               "python -m gomc_gb300.build" % path)
        _build.build()
    L = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _LIB = L
    return L


def check(rc: int, box=None) -> None:
    if rc != 0:
        msg = lib().gb_last_error(box)
        raise GbError(rc, msg.decode() if msg else "")
