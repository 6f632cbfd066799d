"""ctypes binding of libvahana_gb300.so (the C ABI in include/vahana_gb300.h).

The library is built in-tree (vahana.jl_gb300/build.py).  There is no CPU
fallback: importing this module without the library raises ImportError.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(os.path.dirname(HERE), "libvahana_gb300.so")

VG_OK, VG_ERR_ASSERT, VG_ERR_ARG, VG_ERR_CUDA, VG_ERR_NOMEM, VG_ERR_DEVICE, VG_ERR_STATE = range(7)

DTYPES = {"bool": 1, "u8": 2, "i8": 3, "u16": 4, "i16": 5, "u32": 6, "i32": 7,
          "u64": 8, "i64": 9, "f32": 10, "f64": 11}
NP_DTYPES = {"bool": "bool", "u8": "uint8", "i8": "int8", "u16": "uint16", "i16": "int16",
             "u32": "uint32", "i32": "int32", "u64": "uint64", "i64": "int64",
             "f32": "float32", "f64": "float64"}

HINTS = {":Immortal": 0x01, ":Independent": 0x02, ":Stateless": 0x10, ":IgnoreFrom": 0x20,
         ":SingleType": 0x40, ":SingleEdge": 0x80, ":IgnoreSourceState": 0x100,
         ":NumEdgesOnly": 0x200, ":HasEdgeOnly": 0x400}

OPS = {"+": 1, "*": 2, "max": 3, "min": 4, "&": 5, "|": 6}
MAPS = {"field": 0, "==": 1, "!=": 2, "<": 3, ">": 4}
METRICS = {"chebyshev": 0, "euclidean": 1, "manhatten": 2}


def VG_EDGE(e):
    return 0x10000 | e


class VahanaError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("[%d] %s" % (code, msg))
        self.code = code


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIBPATH):
            raise ImportError("libvahana_gb300.so is not built (run vahana.jl_gb300/build.py)")
        _lib = C.CDLL(LIBPATH)
        _declare(_lib)
    return _lib


def check(rc):
    if rc == VG_OK:
        return
    msg = lib().vg_last_error().decode()
    if rc == VG_ERR_ASSERT:
        raise AssertionError(msg)
    raise VahanaError(rc, msg)


P = C.c_void_p
I = C.c_int
U64 = C.c_uint64
I64 = C.c_int64
D = C.c_double
PP = C.POINTER(C.c_void_p)
PU64 = C.POINTER(C.c_uint64)
PI64 = C.POINTER(C.c_int64)
PI = C.POINTER(C.c_int)
CP = C.c_char_p

SIGNATURES = {
    "vg_last_error": (C.c_char_p, []),
    "vg_version": (I, []),
    "vg_device_count": (I, [PI]),
    "vg_model_create": (I, [C.POINTER(P)]),
    "vg_model_destroy": (None, [P]),
    "vg_model_register_agenttype": (I, [P, CP, I, C.POINTER(CP), PI, C.c_uint, PI]),
    "vg_model_register_edgetype": (I, [P, CP, I, C.POINTER(CP), PI, C.c_uint, I, I64, PI]),
    "vg_model_register_param": (I, [P, CP, D]),
    "vg_bind_param": (I, [P, CP, I, I, CP]),
    "vg_unbind_params": (I, [P, CP]),
    "vg_model_register_global": (I, [P, CP, D]),
    "vg_model_finalize": (I, [P, CP]),
    "vg_model_edge_hints": (I, [P, I, C.POINTER(C.c_uint)]),
    "vg_model_type_by_name": (I, [P, CP, PI]),
    "vg_sim_create": (I, [P, CP, P, C.POINTER(P)]),
    "vg_sim_destroy": (I, [P]),
    "vg_sim_copy": (I, [P, C.POINTER(P)]),
    "vg_finish_init": (I, [P]),
    "vg_sim_num_transitions": (I, [P, PI64]),
    "vg_sim_set_stream": (I, [P, P]),
    "vg_sim_synchronize": (I, [P]),
    "vg_sim_set_async": (I, [P, I]),
    "vg_write_agents": (I, [P, I, PP, U64]),
    "vg_sim_device_bytes": (I, [P, PU64]),
    "vg_disable_transition_checks": (I, [P, I]),
    "vg_set_param": (I, [P, CP, D]),
    "vg_param": (I, [P, CP, C.POINTER(D)]),
    "vg_set_global": (I, [P, CP, D]),
    "vg_get_global": (I, [P, CP, C.POINTER(D)]),
    "vg_push_global": (I, [P, CP, D]),
    "vg_global_series": (I, [P, CP, C.POINTER(D), U64, PU64]),
    "vg_add_agents": (I, [P, I, U64, PP, PU64]),
    "vg_add_agent_per_process": (I, [P, I, PP, PU64]),
    "vg_agentstate": (I, [P, U64, I, PP]),
    "vg_num_agents": (I, [P, I, PU64]),
    "vg_agent_slots": (I, [P, I, PU64]),
    "vg_all_agents": (I, [P, I, PP, PU64, U64, PU64]),
    "vg_read_agents": (I, [P, I, PP, C.POINTER(C.c_uint8), U64, PU64]),
    "vg_agent_field_device_ptr": (I, [P, I, I, C.POINTER(P)]),
    "vg_add_edges": (I, [P, I, U64, PU64, PU64, PP]),
    "vg_remove_edges": (I, [P, I, U64, PU64, PU64]),
    "vg_edges": (I, [P, U64, I, PU64, PP, U64, PI64]),
    "vg_neighborids": (I, [P, U64, I, PU64, U64, PI64]),
    "vg_edgestates": (I, [P, U64, I, PP, U64, PI64]),
    "vg_num_edges": (I, [P, U64, I, PI64]),
    "vg_has_edge": (I, [P, U64, I, PI]),
    "vg_num_edges_total": (I, [P, I, I, PU64]),
    "vg_read_edges": (I, [P, I, I, PU64, PU64, PP, PU64, PU64]),
    "vg_apply": (I, [P, CP, PI, I, PI, I, PI, I, PI, I, I, C.POINTER(D), I]),
    "vg_apply_prepare": (I, [P, CP, PI, I, PI, I, PI, I, PI, I, I, C.POINTER(D), I,
                             C.POINTER(P)]),
    "vg_apply_call_run": (I, [P]),
    "vg_apply_call_destroy": (I, [P]),
    "vg_apply_host": (I, [P, CP, PI, I, PI, I, PI, I, PI, I, I, C.POINTER(D), I, I, PP, PP, U64]),
    "vg_transition_names": (C.c_char_p, []),
    "vg_mapreduce_agents": (I, [P, I, I, I, D, I, I, I, D, P]),
    "vg_mapreduce_edges": (I, [P, I, I, I, D, I, I, I, D, P]),
    "vg_add_raster": (I, [P, CP, I, PI64, I, PP, PU64]),
    "vg_connect_raster_neighbors": (I, [P, CP, I, PP, D, I, I, I]),
    "vg_move_to": (I, [P, CP, U64, PI64, I, PP, I, PP, D, I, I, I]),
    "vg_cellid": (I, [P, CP, PI64, PU64]),
    "vg_raster_dims": (I, [P, CP, PI64, PI]),
    "vg_rastervalues": (I, [P, CP, I, P]),
    "vg_gen_uniform_out_edges": (I, [P, I, I, C.c_uint32, U64]),
    "vg_gen_chung_lu_edges": (I, [P, I, I, U64, D, D, D, U64, I]),
    "vg_read_staged_edges": (I, [P, I, PU64, PU64, PP, U64, PU64]),
    "vg_selftest_fp64": (I, [U64, U64, PU64]),
    "vg_selftest_sort": (I, [U64, I, I, I, I, U64, PU64]),
    "vg_selftest_scan": (I, [U64, I, I, U64, PU64]),
    "vg_selftest_scan_timeout": (I, [PI, C.POINTER(D)]),
    "vg_selftest_barrier_timeout": (I, [PI, C.POINTER(D)]),
    "vg_selftest_rate": (I, [I, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(D),
                             C.POINTER(D)]),
    "vg_sir_step_noalloc": (I, [P, P, P, P, P, P, U64, C.c_uint32, D, C.c_int32, U64,
                                C.c_uint32, P]),
    "vg_batch_create_sir": (I, [I, PI64, C.POINTER(C.c_int32), C.POINTER(D),
                                C.POINTER(C.c_int32), PU64, I64, P, C.POINTER(P)]),
    "vg_batch_step": (I, [P, I, I]),
    "vg_batch_step_one": (I, [P, I, I]),
    "vg_batch_read_states": (I, [P, I, C.POINTER(C.c_uint8), C.POINTER(C.c_int32), U64, PU64]),
    "vg_batch_read_graph": (I, [P, I, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), PU64, PU64]),
    "vg_batch_destroy": (I, [P]),
    "vg_batch_read_states2": (I, [P, I, I, C.POINTER(C.c_uint8), C.POINTER(C.c_int32), U64, PU64]),
    "vg_batch_info": (I, [P, PU64, PU64, PI, PI, PU64]),
    "vg_batch_tuning": (I, [P, PI, PI, C.POINTER(C.c_uint32), PU64, C.POINTER(D),
                            C.POINTER(D), C.POINTER(D)]),
    "vg_batch_set_launch": (I, [P, I, I, C.c_uint32]),
    "vg_batch_set_lanes": (I, [P, I, I]),
    "vg_batch_lanes": (I, [P, PI, PI]),
    "vg_batch_set_cluster": (I, [P, I, I, I]),
    "vg_batch_cluster": (I, [P, PI, PI, PI, C.POINTER(C.c_uint)]),
    "vg_add_graph": (I, [P, I, U64, PP, I, U64, PU64, PU64, I, PP, PU64]),
    "vg_sim_save": (I, [P, CP]),
    "vg_sim_load": (I, [P, CP, P, C.POINTER(P)]),
    "vg_serve_create": (I, [U64, I, C.POINTER(P)]),
    "vg_serve_submit": (I, [P, P, PI64]),
    "vg_serve_poll": (I, [P, P, U64, PU64]),
    "vg_serve_job_state": (I, [P, I64, P, U64, PU64]),
    "vg_serve_stats": (I, [P, PU64, PU64, PU64, PU64, PU64, PU64]),
    "vg_serve_drain": (I, [P]),
    "vg_serve_destroy": (I, [P]),
}


def _declare(L):
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name, None)
        if f is None:
            continue
        f.restype = res
        f.argtypes = args


def exported_symbols():
    return list(SIGNATURES)
