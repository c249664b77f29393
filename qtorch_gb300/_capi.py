"""ctypes declarations of the C ABI in include/qtorch_gb300.h."""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libqtorch_gb300.so")

c_int, c_int32, c_int64, c_uint64, c_double, c_char_p, c_void_p, c_size_t, c_uint8 = (
    ctypes.c_int, ctypes.c_int32, ctypes.c_int64, ctypes.c_uint64, ctypes.c_double, ctypes.c_char_p,
    ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint8)
P = ctypes.POINTER
PP = lambda: P(c_void_p)  # noqa: E731


class LaunchPolicy(ctypes.Structure):
    """qt_launch_policy"""
    _fields_ = [("ws_smem_cap", c_int32), ("stage_cap", c_int32), ("ctas_per_sm", c_int32),
                ("static_schedule", c_int32), ("kernel_ctas", c_int32)]


class LaunchInfo(ctypes.Structure):
    """qt_launch_info"""
    _fields_ = [("grid", c_int32), ("n_grouped", c_int32), ("n_stepwise", c_int32), ("dynamic_schedule", c_int32),
                ("n_ws_smem", c_int32), ("n_staged", c_int32), ("smem_bytes", ctypes.c_uint32),
                ("ws_smem_bytes", ctypes.c_uint32), ("stage_bytes", ctypes.c_uint32), ("tile_bytes", ctypes.c_uint32),
                ("ws_slab_bytes", c_uint64), ("kernel_ctas", c_int32), ("pad", c_int32)]


# (name, restype, argtypes)
SIGNATURES = [
    ("qt_status_string", c_char_p, [c_int]),
    ("qt_ctx_create", c_int, [c_int, c_void_p, P(c_void_p)]),
    ("qt_ctx_destroy", c_int, [c_void_p]),
    ("qt_ctx_synchronize", c_int, [c_void_p]),
    ("qt_last_error", c_size_t, [c_void_p, c_char_p, c_size_t]),
    ("qt_ctx_set_memory_budget", c_int, [c_void_p, c_uint64]),
    ("qt_ctx_set_deadline", c_int, [c_void_p, c_double]),
    ("qt_ctx_kernel_launches", c_uint64, [c_void_p]),
    ("qt_ctx_tensor_core_steps", c_uint64, [c_void_p]),
    ("qt_ctx_stream_steps", c_uint64, [c_void_p]),
    ("qt_debug_stream_fault", c_int, [c_void_p, c_int, ctypes.c_uint32]),
    ("qt_debug_gemm_fault", c_int, [c_void_p, c_int, ctypes.c_uint32]),
    ("qt_debug_staging_fault", c_int, [c_void_p, c_int, ctypes.c_uint32]),
    ("qt_ctx_memory_stats", c_int, [c_void_p, P(c_uint64), P(c_uint64), P(c_uint64)]),
    ("qt_tensor_create", c_int, [c_void_p, c_int, c_int, P(c_void_p)]),
    ("qt_tensor_free", c_int, [c_void_p, c_void_p]),
    ("qt_tensor_upload", c_int, [c_void_p, c_void_p, c_void_p, c_size_t]),
    ("qt_tensor_download", c_int, [c_void_p, c_void_p, c_void_p, c_size_t]),
    ("qt_tensor_rank", c_int, [c_void_p]),
    ("qt_tensor_dtype", c_int, [c_void_p]),
    ("qt_tensor_device_ptr", c_void_p, [c_void_p]),
    ("qt_contract_pair", c_int, [c_void_p, c_void_p, c_void_p, c_int, P(c_uint8), P(c_int32), c_int, P(c_int32),
                                 P(c_int32), P(c_void_p)]),
    ("qt_contract_pair_device", c_int, [c_void_p, c_void_p, c_int, c_void_p, c_int, c_int, P(c_uint8), P(c_int32),
                                        c_int, P(c_int32), P(c_int32), c_void_p]),
    ("qt_tensor_permute", c_int, [c_void_p, c_void_p, P(c_int32), P(c_void_p)]),
    ("qt_permute_device", c_int, [c_void_p, c_void_p, c_int, c_int, P(c_int32), c_void_p]),
    ("qt_contract_pair_host", c_int, [c_void_p, P(c_double), c_int, P(c_double), c_int, c_int, P(c_uint8),
                                      P(c_int32), c_int, P(c_int32), P(c_int32), P(c_double)]),
    ("qt_network_create", c_int, [c_void_p, c_char_p, c_char_p, c_char_p, P(c_void_p)]),
    ("qt_network_create_from_files", c_int, [c_void_p, c_char_p, c_char_p, P(c_void_p)]),
    ("qt_network_free", c_int, [c_void_p]),
    ("qt_network_reset", c_int, [c_void_p]),
    ("qt_network_num_qubits", c_int, [c_void_p]),
    ("qt_network_num_nodes", c_int, [c_void_p]),
    ("qt_network_num_uncontracted", c_int, [c_void_p]),
    ("qt_network_node_rank", c_int, [c_void_p, c_int]),
    ("qt_network_is_done", c_int, [c_void_p]),
    ("qt_network_contract_nodes", c_int, [c_void_p, c_int, c_int, c_int, P(c_int)]),
    ("qt_network_contract_sequence", c_int, [c_void_p, P(c_int32), c_int]),
    ("qt_network_contract_user_sequence", c_int, [c_void_p, c_char_p]),
    ("qt_network_contract_stochastic", c_int, [c_void_p, c_uint64]),
    ("qt_network_contract_linegraph", c_int, [c_void_p]),
    ("qt_network_contract_wire_order", c_int, [c_void_p, P(c_int32), c_int]),
    ("qt_network_reduce", c_int, [c_void_p]),
    ("qt_network_final_value", c_int, [c_void_p, P(c_double)]),
    ("qt_network_flops", c_int64, [c_void_p]),
    ("qt_network_created_from", c_int, [c_void_p, P(c_int32), c_int]),
    ("qt_network_node_values", c_int64, [c_void_p, c_int, P(c_double), c_int64]),
    ("qt_network_linegraph_order", c_int, [c_void_p, P(c_int32), c_int]),
    ("qt_run_inp", c_int, [c_void_p, c_char_p, P(c_double), P(c_int64)]),
    ("qt_plan_build", c_int, [c_void_p, c_char_p, c_char_p, c_char_p, c_int, c_uint64, P(c_int32), c_int,
                              P(c_void_p)]),
    ("qt_plan_build_search", c_int, [c_void_p, c_char_p, c_char_p, c_char_p, c_uint64, c_int, c_int64, P(c_void_p),
                                     P(c_uint64)]),
    ("qt_plan_free", c_int, [c_void_p]),
    ("qt_plan_num_steps", c_int, [c_void_p]),
    ("qt_plan_item_descriptors", c_int64, [c_void_p]),
    ("qt_plan_num_leaves", c_int, [c_void_p]),
    ("qt_plan_peak_rank", c_int, [c_void_p]),
    ("qt_plan_workspace_bytes", c_uint64, [c_void_p, c_int]),
    ("qt_plan_flops", c_int64, [c_void_p]),
    ("qt_plan_algorithmic_bytes", c_uint64, [c_void_p, c_int]),
    ("qt_plan_sequence", c_int, [c_void_p, P(c_int32), c_int]),
    ("qt_plan_leaf_elems", c_uint64, [c_void_p]),
    ("qt_plan_leaf_values", c_int, [c_void_p, P(c_double), c_uint64]),
    ("qt_plan_execute", c_int, [c_void_p, c_void_p, c_int, P(c_double)]),
    ("qt_plan_execute_static", c_int, [c_void_p, c_void_p, c_int, c_void_p, P(c_double)]),
    ("qt_plan_num_rotations", c_int, [c_void_p]),
    ("qt_plan_rotation_angles", c_int, [c_void_p, P(c_double), c_int]),
    ("qt_plan_step_info", c_int, [c_void_p, c_int, P(c_int32), c_int]),
    ("qt_batch_set_rotations", c_int, [c_void_p, P(c_double), c_int64]),
    ("qt_batch_set_rotations_device", c_int, [c_void_p, P(c_double), c_int64]),
    # the optimiser's inner loop: raw addresses, no ctypes pointer objects per call
    ("qt_batch_evaluate", c_int, [c_void_p, c_void_p, c_int64, c_void_p]),
    ("qt_batch_create", c_int, [c_void_p, P(c_void_p)]),
    ("qt_batch_free", c_int, [c_void_p]),
    ("qt_batch_add", c_int, [c_void_p, c_void_p, P(c_double), P(c_int)]),
    ("qt_batch_size", c_int, [c_void_p]),
    ("qt_batch_execute", c_int, [c_void_p, c_int, P(c_double)]),
    ("qt_batch_prepare", c_int, [c_void_p, c_int]),
    ("qt_batch_run", c_int, [c_void_p]),
    ("qt_batch_fetch", c_int, [c_void_p, P(c_double)]),
    ("qt_batch_set_leaves", c_int, [c_void_p, c_int, P(c_double)]),
    ("qt_batch_upload", c_int, [c_void_p]),
    ("qt_batch_use_graph", c_int, [c_void_p, c_int]),
    ("qt_batch_use_resident", c_int, [c_void_p, c_double]),
    ("qt_plan_slice", c_int, [c_void_p, c_void_p, c_int, c_uint64, c_int, P(c_void_p)]),
    ("qt_sliced_num_cuts", c_int, [c_void_p]),
    ("qt_sliced_plan", c_void_p, [c_void_p]),
    ("qt_sliced_execute", c_int, [c_void_p, c_int, P(c_double)]),
    ("qt_sliced_execute_leaves", c_int, [c_void_p, c_void_p, c_int, P(c_double), P(c_double)]),
    ("qt_sliced_free", c_int, [c_void_p]),
    ("qt_batch_resident_starts", c_uint64, [c_void_p]),
    ("qt_batch_h2d_bytes", c_uint64, [c_void_p]),
    ("qt_batch_d2h_bytes", c_uint64, [c_void_p]),
    ("qt_batch_launches_per_run", c_int, [c_void_p]),
    ("qt_batch_set_launch_policy", c_int, [c_void_p, P(LaunchPolicy)]),
    ("qt_batch_get_launch_policy", c_int, [c_void_p, P(LaunchPolicy)]),
    ("qt_batch_launch_info", c_int, [c_void_p, P(LaunchInfo)]),
    ("qt_batch_autotune", c_int, [c_void_p, c_int, P(LaunchPolicy), P(c_double)]),
    ("qt_qaoa_term_text", c_int64, [c_char_p, c_int, P(c_double), c_int, c_char_p, c_int64, c_char_p, c_int64]),
    ("qt_qaoa_num_edges", c_int, [c_char_p]),
    ("qt_qaoa_circuit_text", c_int64, [c_char_p, c_int, P(c_double), c_char_p, c_int64]),
    ("qt_maxcut_final_string", c_int, [c_void_p, c_char_p, c_int, P(c_double), c_int, c_int, c_uint64,
                                       P(c_int32), c_int, P(c_int), P(c_int), P(c_double), P(c_double)]),
    ("qt_random_regular_graph", c_int64, [c_int, c_int, c_uint64, c_char_p, c_int64]),
    ("qt_server_create", c_int, [c_void_p, c_int, c_int, P(c_void_p)]),
    ("qt_server_free", c_int, [c_void_p]),
    ("qt_server_submit", c_int, [c_void_p, c_void_p, P(c_double), P(c_int64)]),
    ("qt_server_poll", c_int, [c_void_p, c_int64, P(c_double), P(c_double)]),
    ("qt_server_poll_detail", c_int, [c_void_p, c_int64, P(c_double), P(c_double), P(c_double), P(c_int)]),
    ("qt_server_set_max_macs", c_int, [c_void_p, c_int64]),
    ("qt_server_refused", c_int64, [c_void_p]),
    ("qt_server_oom_retries", c_int64, [c_void_p]),
    ("qt_server_drain", c_int, [c_void_p]),
    ("qt_server_stats", c_int, [c_void_p, P(c_double), P(c_double), P(c_int64), P(c_int64)]),
    ("qt_server_wave_stats", c_int, [c_void_p, P(c_int64), P(c_int64), P(c_double)]),
]

_lib = None


def load(path=None):
    """Load the shared library and declare every entry point (no GPU needed)."""
    global _lib
    if _lib is None:
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise OSError(f"libqtorch_gb300.so is not built ({p}); run qtorch_gb300.build.build()")
        lib = ctypes.CDLL(p)
        for name, res, args in SIGNATURES:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib
