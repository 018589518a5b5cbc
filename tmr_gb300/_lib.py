"""ctypes binding of the native library ``libtmrg.so`` (C ABI in include/tmrg.h).

The library is the only compute path: if it has not been built this module
raises on first use rather than falling back to anything else.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libtmrg.so")

c_int = ctypes.c_int
c_i64 = ctypes.c_int64
c_u64 = ctypes.c_uint64
c_dbl = ctypes.c_double
c_vp = ctypes.c_void_p
P = ctypes.POINTER

# name -> argtypes (all return int status unless listed in _RESTYPE)
_SIGS = {
    "tmrg_last_error": [],
    "tmrg_version": [],
    "tmrg_kernel_launch_count": [],
    "tmrg_host_sync_count": [],
    "tmrg_device_alloc_count": [],
    "tmrg_tune_reset": [c_int],
    "tmrg_tune_report": [c_vp, c_i64],
    "tmrg_tune_force": [c_int, c_int],
    "tmrg_profile_begin": [],
    "tmrg_profile_end": [c_vp, c_i64],
    "tmrg_measure_fp64_peak": [P(c_dbl)],
    "tmrg_forest_create": [c_int, c_int, c_vp, P(c_vp)],
    "tmrg_forest_destroy": [c_vp],
    "tmrg_forest_set_connectivity": [c_vp, c_int, c_vp, c_int],
    "tmrg_forest_set_mesh_order": [c_vp, c_int, c_int],
    "tmrg_forest_get_mesh_order": [c_vp, P(c_int), P(c_int)],
    "tmrg_forest_get_interp_knots": [c_vp, c_vp],
    "tmrg_forest_create_trees": [c_vp, c_int],
    "tmrg_forest_refine": [c_vp, c_vp, c_i64, c_int, c_int],
    "tmrg_forest_refine_device": [c_vp, c_vp, c_i64, c_int, c_int],
    "tmrg_forest_coarsen": [c_vp, P(c_vp)],
    "tmrg_forest_duplicate": [c_vp, P(c_vp)],
    "tmrg_forest_balance": [c_vp, c_int],
    "tmrg_forest_repartition": [c_vp, c_int],
    "tmrg_forest_create_nodes": [c_vp],
    "tmrg_forest_num_octants": [c_vp, P(c_i64)],
    "tmrg_forest_get_octants": [c_vp, c_vp, c_i64],
    "tmrg_forest_octants_device": [c_vp, P(c_vp), P(c_vp), P(c_vp), P(c_vp), P(c_vp), P(c_vp)],
    "tmrg_forest_node_sizes": [c_vp, c_vp],
    "tmrg_forest_get_node_conn": [c_vp, c_vp, c_i64],
    "tmrg_forest_get_node_numbers": [c_vp, c_vp, c_i64],
    "tmrg_forest_get_dep_node_conn": [c_vp, c_vp, c_vp, c_vp],
    "tmrg_forest_node_conn_device": [c_vp, P(c_vp)],
    "tmrg_forest_dep_node_conn_device": [c_vp, P(c_vp), P(c_vp), P(c_vp)],
    "tmrg_forest_octants_host": [c_vp, P(c_vp), P(c_i64)],
    "tmrg_forest_node_conn_host": [c_vp, P(c_vp), P(c_i64)],
    "tmrg_forest_dep_node_conn_host": [c_vp, P(c_vp), P(c_vp), P(c_vp), P(c_i64)],
    "tmrg_host_pool_trim": [],
    "tmrg_forest_set_full_connectivity": [c_vp, c_int, c_int, c_int, c_int, c_vp, c_vp, c_vp],
    "tmrg_forest_get_connectivity": [c_vp, P(c_int), P(c_int), P(c_int), P(c_int),
                                     P(c_vp), P(c_vp), P(c_vp), P(c_vp)],
    "tmrg_forest_get_inverse_connectivity": [c_vp, P(c_vp), P(c_vp), P(c_vp), P(c_vp),
                                             P(c_vp), P(c_vp)],
    "tmrg_forest_create_random_trees": [c_vp, c_int, c_int, c_int, c_u64],
    "tmrg_forest_get_local_node_number": [c_vp, c_int, P(c_int)],
    "tmrg_forest_set_block_boxes": [c_vp, c_vp, c_int],
    "tmrg_forest_get_points": [c_vp, c_vp, c_i64],
    "tmrg_eval_interp": [c_int, c_int, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp],
    "tmrg_forest_eval_interp": [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp],
    "tmrg_eval_interp2": [c_int, c_int, c_vp, c_vp] + [c_vp] * 10,
    "tmrg_forest_eval_interp2": [c_vp, c_vp] + [c_vp] * 10,
    "tmrg_forest_find_enclosing": [c_vp, c_int, c_vp, c_vp, c_i64, c_vp],
    "tmrg_forest_transform_nodes": [c_vp, c_vp, c_i64, c_int, c_vp, c_vp],
    "tmrg_bump_indicator_device": [c_vp, c_vp, c_int, c_vp, c_dbl, c_dbl, c_int, c_int, c_vp],
    "tmrg_batch_refinement_device": [c_vp, c_int, c_vp, c_vp, c_vp, c_vp, c_u64, c_u64, c_vp,
                                     c_vp],
    "tmrg_interp_create": [c_vp, c_vp, P(c_vp)],
    "tmrg_interp_destroy": [c_vp],
    "tmrg_topo_weights_create": [c_vp, c_vp, P(c_vp)],
    "tmrg_interp_sizes": [c_vp, c_vp],
    "tmrg_interp_apply_nnz": [c_vp, c_vp],
    "tmrg_interp_get_csr": [c_vp, c_vp, c_vp, c_vp],
    "tmrg_interp_mult": [c_vp, c_vp, c_vp, c_int],
    "tmrg_interp_mult_transpose": [c_vp, c_vp, c_vp, c_int],
    "tmrg_interp_mult_weight_transpose": [c_vp, c_vp, c_vp, c_int],
    "tmrg_interp_mult_device": [c_vp, c_vp, c_vp, c_int],
    "tmrg_interp_mult_transpose_device": [c_vp, c_vp, c_vp, c_int],
    "tmrg_interp_mult_weight_transpose_device": [c_vp, c_vp, c_vp, c_int],
    "tmrg_filter_create": [c_vp, c_dbl, c_dbl, c_int, P(c_vp)],
    "tmrg_filter_create_quad": [c_vp, c_dbl, c_dbl, c_int, P(c_vp)],
    "tmrg_filter_destroy": [c_vp],
    "tmrg_filter_sizes": [c_vp, c_vp],
    "tmrg_filter_get_matrix": [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp],
    "tmrg_filter_apply": [c_vp, c_int, c_vp, c_vp],
    "tmrg_filter_apply_transpose": [c_vp, c_int, c_vp, c_vp],
    "tmrg_filter_apply_device": [c_vp, c_int, c_vp, c_vp],
    "tmrg_filter_apply_transpose_device": [c_vp, c_int, c_vp, c_vp],
    "tmrg_filter_apply_f32_device": [c_vp, c_int, c_vp, c_vp],
    "tmrg_filter_apply_transpose_f32_device": [c_vp, c_int, c_vp, c_vp],
    "tmrg_filter_apply_static_device": [c_vp, c_int, c_int, c_vp, c_vp],
    "tmrg_qforest_create": [c_int, c_int, c_vp, P(c_vp)],
    "tmrg_qforest_destroy": [c_vp],
    "tmrg_qforest_set_connectivity": [c_vp, c_int, c_vp, c_int],
    "tmrg_qforest_set_full_connectivity": [c_vp, c_int, c_int, c_int, c_vp, c_vp],
    "tmrg_qforest_get_connectivity": [c_vp, c_vp, c_vp, c_vp],
    "tmrg_qforest_set_mesh_order": [c_vp, c_int, c_int],
    "tmrg_qforest_get_mesh_order": [c_vp, c_vp, c_vp, c_vp],
    "tmrg_qforest_create_trees": [c_vp, c_int],
    "tmrg_qforest_create_random_trees": [c_vp, c_int, c_int, c_int, c_u64],
    "tmrg_qforest_refine": [c_vp, c_vp, c_i64, c_int, c_int],
    "tmrg_qforest_refine_device": [c_vp, c_vp, c_i64, c_int, c_int],
    "tmrg_qforest_coarsen": [c_vp, P(c_vp)],
    "tmrg_qforest_duplicate": [c_vp, P(c_vp)],
    "tmrg_qforest_balance": [c_vp, c_int],
    "tmrg_qforest_create_nodes": [c_vp],
    "tmrg_qforest_num_quadrants": [c_vp, c_vp],
    "tmrg_qforest_get_quadrants": [c_vp, c_vp],
    "tmrg_qforest_sizes": [c_vp, c_vp],
    "tmrg_qforest_get_node_conn": [c_vp, c_vp],
    "tmrg_qforest_get_dep_node_conn": [c_vp, c_vp, c_vp, c_vp],
    "tmrg_qforest_create_interpolation": [c_vp, c_vp, P(c_vp)],
    "tmrg_qforest_set_face_boxes": [c_vp, c_vp, c_int],
    "tmrg_qforest_get_points": [c_vp, c_vp],
    "tmrg_stl_triangles": [c_vp, c_vp, c_int, c_int, c_dbl, c_vp, c_vp, c_i64],
    "tmrg_stl_triangles_device": [c_vp, c_vp, c_int, c_int, c_dbl, c_vp, c_vp, c_i64],
    "tmrg_generate_bin_file": [ctypes.c_char_p, c_vp, c_vp, c_int, c_int, c_dbl],
    "tmrg_convert_bin_to_stl": [ctypes.c_char_p, ctypes.c_char_p],
    "tmrg_helmholtz_create": [c_vp, c_int, c_dbl, P(c_vp)],
    "tmrg_helmholtz_create_quad": [c_vp, c_int, c_dbl, P(c_vp)],
    "tmrg_helmholtz_destroy": [c_vp],
    "tmrg_helmholtz_sizes": [c_vp, c_vp, c_vp],
    "tmrg_helmholtz_apply": [c_vp, c_int, c_vp, c_vp],
    "tmrg_helmholtz_apply_transpose": [c_vp, c_int, c_vp, c_vp],
    "tmrg_helmholtz_apply_device": [c_vp, c_int, c_vp, c_vp],
    "tmrg_helmholtz_apply_transpose_device": [c_vp, c_int, c_vp, c_vp],
    "tmrg_helmholtz_set_tolerances": [c_vp, c_dbl, c_dbl, c_int],
    "tmrg_helmholtz_last_solve": [c_vp, c_vp, c_vp, c_int],
    "tmrg_helmholtz_set_smoother": [c_vp, c_int, c_int, c_dbl, c_dbl, c_dbl],
    "tmrg_helmholtz_mult_device": [c_vp, c_int, c_int, c_int, c_vp, c_vp],
    "tmrg_random_refinement_device": [c_u64, c_u64, c_dbl, c_vp, c_i64, c_vp],
}
_RESTYPE = {
    "tmrg_last_error": ctypes.c_char_p,
    "tmrg_version": ctypes.c_char_p,
    "tmrg_kernel_launch_count": c_i64,
    "tmrg_host_sync_count": c_i64,
    "tmrg_device_alloc_count": c_i64,
}

STATUS = {
    0: "TMRG_OK", 1: "TMRG_ERR_ARG", 2: "TMRG_ERR_STATE", 3: "TMRG_ERR_CUDA",
    4: "TMRG_ERR_NOMEM", 5: "TMRG_ERR_KEY_RANGE", 6: "TMRG_ERR_UNSUPPORTED",
    7: "TMRG_ERR_INTERNAL",
}


class TMRGError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS.get(status, status), msg))
        self.status = status


_lib = None


def lib():
    """Load libtmrg.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                "libtmrg.so is not built (%s); run tmr_gb300.build.build()" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, args in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = _RESTYPE.get(name, c_int)
        _lib = L
    return _lib


def check(status):
    if status != 0:
        raise TMRGError(status, lib().tmrg_last_error().decode())


def call(name, *args):
    check(getattr(lib(), name)(*args))
