"""ctypes binding of the C ABI (include/cusat_fec.h).

Loads the in-tree ``cusat_gb300/_lib/libcusat_fec.so``.  There is no CPU
fallback: if the library is missing or was built for another machine, the
first use raises.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libcusat_fec.so")

_c_int_p = ctypes.POINTER(ctypes.c_int32)
_lib = None

# name -> (restype, argtypes)
_SIGS = {
    "cusat_last_error": (ctypes.c_char_p, []),
    "cusat_ldpc_decoder_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                  ctypes.POINTER(ctypes.c_void_p)]),
    "cusat_ldpc_decoder_destroy": (None, [ctypes.c_void_p]),
    "cusat_ldpc_decoder_info": (ctypes.c_int, [ctypes.c_void_p, _c_int_p]),
    "cusat_ldpc_decoder_frames_per_cta": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "cusat_ldpc_decoder_set_frames_per_cta": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "cusat_rx_fec_set_frames_per_cta": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "cusat_ldpc_decoder_set_weights": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    "cusat_ldpc_decoder_set_max_ctas": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "cusat_ldpc_decode_launch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                                ctypes.c_void_p, ctypes.c_void_p]),
    "cusat_ldpc_decode_batch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.c_int, ctypes.c_void_p]),
    "cusat_ldpc_decode_batch_d2h": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                   ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "cusat_ldpc_decoder_results": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                  ctypes.c_int]),
    "cusat_demapper_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                             ctypes.POINTER(ctypes.c_void_p)]),
    "cusat_demapper_destroy": (None, [ctypes.c_void_p]),
    "cusat_demapper_info": (ctypes.c_int, [ctypes.c_void_p, _c_int_p]),
    "cusat_demapper_capped_llr_gain": (ctypes.c_float, [ctypes.c_void_p, ctypes.c_float]),
    "cusat_demapper_soft_out_dev": (ctypes.c_void_p, [ctypes.c_void_p]),
    "cusat_demap_launch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_float,
                                          ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p]),
    "cusat_demap_batch_async": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_float,
                                               ctypes.c_float, ctypes.c_void_p]),
    "cusat_demap_batch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_float,
                                         ctypes.c_float]),
    "cusat_bch_checker_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_uint,
                                                ctypes.POINTER(ctypes.c_void_p)]),
    "cusat_bch_checker_create_for_code": (ctypes.c_int, [ctypes.c_int, ctypes.c_int,
                                                         ctypes.POINTER(ctypes.c_void_p)]),
    "cusat_bch_checker_destroy": (None, [ctypes.c_void_p]),
    "cusat_bch_checker_n_bytes": (ctypes.c_uint, [ctypes.c_void_p]),
    "cusat_bch_check_launch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                              ctypes.c_int, ctypes.c_void_p]),
    "cusat_rx_fec_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_void_p)]),
    "cusat_rx_fec_destroy": (None, [ctypes.c_void_p]),
    "cusat_rx_fec_info": (ctypes.c_int, [ctypes.c_void_p, _c_int_p]),
    "cusat_rx_fec_set_weights": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    "cusat_rx_fec_capped_llr_gain": (ctypes.c_float, [ctypes.c_void_p, ctypes.c_float]),
    "cusat_rx_fec_launch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_float,
                                           ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_void_p]),
    "cusat_server_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_size_t,
                                           ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "cusat_server_destroy": (None, [ctypes.c_void_p]),
    "cusat_server_now": (ctypes.c_double, [ctypes.c_void_p]),
    "cusat_server_set_weights": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]),
    "cusat_server_submit": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    "cusat_server_poll": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "cusat_server_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]),
    "cusat_bb_extractor_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "cusat_bb_extractor_destroy": (None, [ctypes.c_void_p]),
    "cusat_pl_layout": (ctypes.c_int, [ctypes.c_int, ctypes.c_void_p]),
    "cusat_ldpc_encode": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    "cusat_pl_rotation_index": (ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_int]),
    "cusat_pl_extractor_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                                 ctypes.POINTER(ctypes.c_void_p)]),
    "cusat_pl_extractor_destroy": (None, [ctypes.c_void_p]),
    "cusat_pl_extract": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "cusat_bb_extract": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "cusat_bb_extract_frames": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                               ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                               ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "cusat_generator_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                              ctypes.POINTER(ctypes.c_void_p)]),
    "cusat_generator_destroy": (None, [ctypes.c_void_p]),
    "cusat_generator_info": (ctypes.c_int, [ctypes.c_void_p, _c_int_p]),
    "cusat_generate": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_void_p]),
    "cusat_nms_trainer_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                 ctypes.POINTER(ctypes.c_void_p)]),
    "cusat_nms_trainer_destroy": (None, [ctypes.c_void_p]),
    "cusat_nms_trainer_info": (ctypes.c_int, [ctypes.c_void_p, _c_int_p]),
    "cusat_nms_trainer_degree_counts": (ctypes.c_int, [ctypes.c_void_p, _c_int_p]),
    "cusat_nms_train_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_void_p]),
    "cusat_ldpc_decode_noalloc": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                                 ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "cusat_batch_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.POINTER(ctypes.c_void_p)]),
    "cusat_batch_destroy": (None, [ctypes.c_void_p]),
    "cusat_batch_info": (ctypes.c_int, [ctypes.c_void_p, _c_int_p]),
    "cusat_batch_set_weights": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]),
    "cusat_batch_set_max_ctas": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "cusat_batch_tuned": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    "cusat_batch_launch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "cusat_batch_tune": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_void_p, ctypes.POINTER(ctypes.c_float)]),
    "cusat_batch_capture": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "cusat_batch_replay": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "cusat_decode_budget_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "cusat_decode_budget_destroy": (None, [ctypes.c_void_p]),
    "cusat_decode_budget_info": (ctypes.c_int, [ctypes.c_void_p, _c_int_p]),
    "cusat_dd_snr": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                    ctypes.c_int, ctypes.POINTER(ctypes.c_float)]),
    "cusat_rx_chain_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "cusat_rx_chain_destroy": (None, [ctypes.c_void_p]),
    "cusat_rx_chain_info": (ctypes.c_int, [ctypes.c_void_p, _c_int_p]),
    "cusat_rx_chain_set_weights": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    "cusat_rx_chain_set_decode_budget": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "cusat_rx_chain_set_launch_lock": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                      ctypes.c_void_p]),
    "cusat_rx_chain_set_block_when_full": (None, [ctypes.c_void_p, ctypes.c_int]),
    "cusat_rx_chain_set_copy_threads": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "cusat_rx_pool_set_copy_threads": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "cusat_rx_chain_update_snr": (None, [ctypes.c_void_p, ctypes.c_float]),
    "cusat_rx_chain_submit_xfecframe": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    "cusat_rx_chain_drain_completed": (ctypes.c_int, [ctypes.c_void_p]),
    "cusat_rx_chain_get_gse_output": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    "cusat_rx_chain_gse_dfl_sizes": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    "cusat_rx_chain_launch_partial": (ctypes.c_int, [ctypes.c_void_p]),
    "cusat_rx_chain_flush": (ctypes.c_int, [ctypes.c_void_p]),
    "cusat_rx_chain_reset": (ctypes.c_int, [ctypes.c_void_p]),
    "cusat_rx_chain_warmup": (ctypes.c_int, [ctypes.c_void_p]),
    "cusat_rx_chain_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]),
    "cusat_rx_pool_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "cusat_rx_pool_create_mixed": (ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                                  ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                  ctypes.POINTER(ctypes.c_void_p)]),
    "cusat_rx_pool_destroy": (None, [ctypes.c_void_p]),
    "cusat_rx_pool_chain": (ctypes.c_void_p, [ctypes.c_void_p, ctypes.c_int]),
    "cusat_rx_pool_submit": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "cusat_rx_pool_get_gse_output": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    "cusat_rx_pool_gse_dfl_sizes": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]),
    "cusat_rx_pool_drain_all_completed": (ctypes.c_int, [ctypes.c_void_p]),
    "cusat_rx_pool_finish_all_pending": (ctypes.c_int, [ctypes.c_void_p]),
    "cusat_rx_pool_launch_stale": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double]),
    "cusat_rx_pool_reset_all": (ctypes.c_int, [ctypes.c_void_p]),
    "cusat_rx_pool_warmup_all": (ctypes.c_int, [ctypes.c_void_p]),
    "cusat_rx_pool_update_snr": (None, [ctypes.c_void_p, ctypes.c_int, ctypes.c_float]),
    "cusat_rx_pool_set_launch_lock": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                     ctypes.c_void_p]),
    "cusat_rx_pool_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]),
    "cusat_rx_pool_modcod_counters": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int,
                                                     ctypes.POINTER(ctypes.c_uint64),
                                                     ctypes.POINTER(ctypes.c_uint64)]),
    "cusat_code_info": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _c_int_p]),
    "cusat_gen_encode": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_int]),
    "cusat_gen_map": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                     ctypes.c_void_p]),
    "cusat_modcod_info": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                         ctypes.c_void_p, _c_int_p]),
    "cusat_modcod_capped_llr_gain": (ctypes.c_float, [ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                      ctypes.c_float]),
}


class PlFrame(ctypes.Structure):
    """cusat_pl_frame of include/cusat_fec.h."""
    _fields_ = [("payload", ctypes.c_void_p), ("data", ctypes.c_void_p), ("slot_rot", ctypes.c_void_p),
                ("pls_code", ctypes.c_int32), ("gold", ctypes.c_int32)]


class Frame(ctypes.Structure):
    """cusat_frame of include/cusat_fec.h."""
    _fields_ = [("modcod", ctypes.c_int32), ("noise_var", ctypes.c_float), ("llr_gain", ctypes.c_float),
                ("reserved", ctypes.c_int32), ("sym", ctypes.c_void_p), ("hard", ctypes.c_void_p),
                ("trials", ctypes.c_void_p), ("bch_valid", ctypes.c_void_p)]


class Request(ctypes.Structure):
    """cusat_request of include/cusat_fec.h."""
    _fields_ = [("modcod", ctypes.c_int32), ("noise_var", ctypes.c_float), ("llr_gain", ctypes.c_float),
                ("flags", ctypes.c_int32), ("sym", ctypes.c_void_p), ("hard_host", ctypes.c_void_p),
                ("tag", ctypes.c_uint64), ("arrival_s", ctypes.c_double)]


class Result(ctypes.Structure):
    """cusat_result of include/cusat_fec.h."""
    _fields_ = [("tag", ctypes.c_uint64), ("modcod", ctypes.c_int32), ("trials", ctypes.c_int32),
                ("bch_valid", ctypes.c_int32), ("reserved", ctypes.c_int32), ("arrival_s", ctypes.c_double),
                ("admit_s", ctypes.c_double), ("done_s", ctypes.c_double)]


class CusatError(RuntimeError):
    """A C-ABI call returned an error code."""

    def __init__(self, code, msg):
        super().__init__(f"cusat error {code}: {msg}")
        self.code = code


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run __graft_entry__.build() "
                              f"(or python cusat_gb300/build.py) on this machine first")
        l = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(l, name)
            fn.restype = res
            fn.argtypes = args
        _lib = l
    return _lib


def check(rc):
    if rc != 0:
        raise CusatError(rc, lib().cusat_last_error().decode())
    return rc


def exported_symbols():
    return list(_SIGS)
