"""ctypes bindings of ``include/laml_gb300.h`` (the C ABI of liblaml_gb300.so).

The library is loaded on first use; a missing library raises immediately --
there is no Python fallback for any compute entry point.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
# LAML_GB300_LIB selects another build of the library (tile-setting variants)
LIB_PATH = os.environ.get("LAML_GB300_LIB") or os.path.join(HERE, "_lib", "liblaml_gb300.so")

i32, i64, u8, u32, f32, f64 = C.c_int32, C.c_int64, C.c_uint8, C.c_uint32, C.c_float, C.c_double
P = C.POINTER
vp = C.c_void_p

LAML_OK = 0
ERRORS = {-1: "LAML_ERR_ARG", -2: "LAML_ERR_CUDA", -3: "LAML_ERR_PARSE", -4: "LAML_ERR_PRIOR",
          -5: "LAML_ERR_TIMEOUT", -6: "LAML_ERR_NOT_BINARY", -7: "LAML_ERR_LEAF"}
TREE_ACTIVE, TREE_CONVERGED, TREE_NAN, TREE_MAXITER, TREE_INFEASIBLE = 0, 1, 2, 3, 4
MODE_LINEAR, MODE_LOG = 0, 1
MSTEP_FP64_POLISH, MSTEP_ULTRAMETRIC, MSTEP_ULTRA_BARRIER = 1, 2, 4
MSTEP_ULTRA_PD_SHORT = 8
MSTEP_LBFGS = 16
LBFGS_SLOTS = 25   # LAML_LBFGS_SLOTS: floats per node and tree parameter of nd_lbfgs
UWORK_SLOTS = 17   # LAML_UWORK_SLOTS: doubles per node of nd_uwork
OUT_POSTERIORS, OUT_TRUE_ROOT = 1, 2


class LamlError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class DatasetInfo(C.Structure):
    _fields_ = [("n_leaves", i32), ("n_sites", i32), ("n_sites_pad", i32), ("n_groups", i32),
                ("group_sites", i32), ("row_len", i64), ("max_states", i32),
                ("n_missing", i64), ("n_silenced", i64)]


class PlanInput(C.Structure):
    _fields_ = [("n_trees", i32), ("tree_nodes", vp), ("tree_leaves", vp), ("tree_dataset", vp),
                ("child0", vp), ("child1", vp), ("n_datasets", i32), ("ds_groups", vp),
                ("ds_sites_pad", vp), ("ds_row_len", vp), ("ds_group_base", vp), ("group_C", vp),
                ("ds_sites", vp), ("ds_leaves", vp), ("group_off", vp)]


class PlanSizes(C.Structure):
    _fields_ = [("n_nodes", i64), ("part_floats", i64), ("scalar_len", i64), ("site_len", i64),
                ("count_floats", i64), ("post_len", i64), ("n_in_levels", i32),
                ("n_out_levels", i32), ("n_in_items", i64), ("n_out_items", i64),
                ("n_root_items", i64), ("n_groups_total", i64)]


PLAN_OUT_FIELDS = ["tr_node_base", "tr_root", "tr_quirk", "tr_site_base", "tr_cnt_base",
                   "tr_post_base", "nd_tree", "nd_c0", "nd_c1", "nd_parent", "nd_sib",
                   "nd_leafrow", "nd_prow", "nd_srow", "in_level_off", "in_items",
                   "out_level_off", "out_items", "root_items", "in_desc", "out_desc",
                   "grp_desc", "in_lnodes", "out_lnodes"]


class PlanOutput(C.Structure):
    _fields_ = [(n, vp) for n in PLAN_OUT_FIELDS]


# laml_batch: (name, ctype) in header order
BATCH_FIELDS = [
    ("group_sites", i32), ("compat", i32), ("n_trees", i32), ("n_datasets", i32),
    ("n_nodes", i64), ("n_in_levels", i32), ("n_out_levels", i32),
    ("n_in_items", i64), ("n_out_items", i64), ("n_root_items", i64),
    ("ds_sites", vp), ("ds_sites_pad", vp), ("ds_groups", vp), ("ds_group_base", vp),
    ("ds_site_base", vp), ("ds_q_base", vp), ("ds_code_base", vp), ("ds_missing", vp),
    ("ds_silenced", vp), ("group_off", vp), ("group_C", vp), ("site_C", vp),
    ("site_sumq", vp), ("q", vp), ("codes", vp),
    ("tr_ds", vp), ("tr_node_base", vp), ("tr_nodes", vp), ("tr_leaves", vp), ("tr_root", vp),
    ("tr_quirk", vp), ("tr_site_base", vp), ("tr_cnt_base", vp), ("tr_post_base", vp),
    ("tr_nu", vp), ("tr_phi", vp), ("tr_prev", vp), ("tr_fix", vp), ("tr_llh", vp),
    ("tr_llh_prev", vp), ("tr_iter", vp), ("tr_status", vp),
    ("tr_mode", vp),
    ("nd_tree", vp), ("nd_c0", vp), ("nd_c1", vp), ("nd_parent", vp), ("nd_sib", vp),
    ("nd_leafrow", vp), ("nd_prow", vp), ("nd_srow", vp), ("nd_d", vp), ("nd_d_prev", vp),
    ("nd_mask", vp), ("nd_bt", vp), ("nd_cnt", vp), ("nd_stage", vp),
    ("in_part", vp), ("out_part", vp), ("in_dot", vp), ("in_x", vp), ("in_h", vp),
    ("out_x", vp), ("out_h", vp), ("llh_site", vp), ("root_lr", vp), ("root_x", vp),
    ("cnt_part", vp), ("post0", vp), ("post1", vp),
    ("in_level_off", vp), ("in_items", vp), ("out_level_off", vp), ("out_items", vp),
    ("root_items", vp), ("in_desc", vp), ("out_desc", vp), ("grp_desc", vp),
    ("h_in_level_off", vp), ("h_out_level_off", vp),
    ("barrier", vp), ("error", vp), ("max_states", i32), ("max_tree_nodes", i32),
    ("tr_leaf", vp), ("nd_uorder", vp), ("nd_uwork", vp),
    ("plan_part_floats", i64), ("plan_scalar_len", i64), ("tr_mstats", vp),
    ("wide_chunk", i32), ("wait_limit_ns", i64), ("nd_lbfgs", vp), ("wide_pc", i32),
    ("in_lnodes", vp), ("out_lnodes", vp),
]


class Batch(C.Structure):
    _fields_ = BATCH_FIELDS


EXPORTS = {
    "laml_newick_size": (i32, [C.c_char_p, P(i32), P(i32), P(i64)]),
    "laml_newick_encode": (i32, [C.c_char_p, P(C.c_char_p), i32, vp, vp, vp, vp, vp, vp, vp]),
    "laml_newick_batch_measure": (i32, [i32, P(C.c_char_p), P(i64)]),
    "laml_newick_encode_batch": (i32, [i32, P(C.c_char_p), P(C.c_char_p), i32, i32, vp, vp, vp,
                                       vp, vp, vp, vp]),
    "laml_dataset_measure": (i32, [i32, i32, vp, vp, vp, vp, i32, i32, P(DatasetInfo)]),
    "laml_dataset_encode": (i32, [i32, i32, vp, vp, vp, vp, i32, i32, vp, vp, vp, vp, vp, vp, vp,
                                  vp, vp]),
    "laml_plan_measure": (i32, [P(PlanInput), P(PlanSizes)]),
    "laml_plan_fill": (i32, [P(PlanInput), P(PlanOutput)]),
    "laml_ultra_order": (i32, [vp, i32, vp, i64, P(i64)]),
    "laml_nni_candidates": (i32, [i32, i32, vp, vp, vp, vp, vp, i32, vp, i32, vp, vp, vp, vp,
                                  vp]),
    "laml_supported_group_sites": (i32, []),
    "laml_plan_descriptors": (i32, [P(Batch), vp, vp, vp, vp]),
    "laml_branch_terms": (i32, [P(Batch), vp]),
    "laml_inside": (i32, [P(Batch), i32, vp]),
    "laml_outside": (i32, [P(Batch), i32, vp]),
    "laml_mstep": (i32, [P(Batch), i32, i32, vp]),
    "laml_gradient": (i32, [P(Batch), vp, vp, vp]),
    "laml_em_run": (i32, [P(Batch), i32, i32, f64, i32, i32, vp]),
    "laml_em_run_levels": (i32, [P(Batch), i32, i32, f64, i32, i32, vp]),
    "laml_inside_noalloc": (i32, [P(Batch), i64, i64, vp]),
    "laml_em_graph_create": (i32, [P(Batch), i32, i32, f64, i32, i32, i32, P(vp)]),
    "laml_em_graph_loop_create": (i32, [P(Batch), i32, i32, f64, i32, i32, i32, vp, P(vp)]),
    "laml_graph_launch": (i32, [vp, vp]),
    "laml_graph_destroy": (None, [vp]),
    "laml_last_error": (C.c_char_p, []),
}

_lib = None


def lib():
    """Load liblaml_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"laml_gb300 native library not built: {LIB_PATH} "
                               "(run python -m laml_gb300.build)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in EXPORTS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc):
    if rc != LAML_OK:
        msg = lib().laml_last_error().decode(errors="replace")
        raise LamlError(rc, msg)
    return rc


def ptr(a):
    """Address of a numpy array or torch tensor (None -> NULL)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data
