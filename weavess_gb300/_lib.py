"""ctypes binding of libweavess_gpu.so (the C ABI in include/weavess_gpu.h).

There is no fallback: if the library is missing or a call fails, this raises.
"""
from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np

from . import build as _build

_lib = None

HEADER = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "include", "weavess_gpu.h")

u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")


class WeavessError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class Counters(C.Structure):
    _fields_ = [("dist_count", C.c_ulonglong), ("hop_count", C.c_ulonglong)]


class LearnParams(C.Structure):
    _fields_ = [("clusters", C.c_uint32), ("kmeans_iters", C.c_uint32), ("list_len", C.c_uint32),
                ("L_trace", C.c_uint32), ("epochs", C.c_uint32), ("batch", C.c_uint32), ("lr", C.c_float),
                ("lam", C.c_float), ("L_min", C.c_uint32), ("L_max", C.c_uint32), ("target_agreement", C.c_float),
                ("fallback_p", C.c_float), ("seed", C.c_uint32)]


class PlanParams(C.Structure):
    _fields_ = [("nq_max", C.c_uint32), ("L_max", C.c_uint32), ("K_max", C.c_uint32), ("out_stride", C.c_uint32),
                ("mode", C.c_int)]


class PlanShape(C.Structure):
    _fields_ = [("warps_per_block", C.c_int), ("hash_words", C.c_uint32), ("wide_hash", C.c_int), ("blocks", C.c_int),
                ("ms", C.c_float), ("query_warps", C.c_int)]


class TuneReport(C.Structure):
    _fields_ = [("n", C.c_int), ("chosen", C.c_int), ("tried", PlanShape * 32)]


class IndexInfo(C.Structure):
    _fields_ = [("max_out", C.c_uint32), ("min_out", C.c_uint32), ("avg_out", C.c_double), ("conn", C.c_uint32),
                ("quality", C.c_double)]


class LearnReport(C.Structure):
    _fields_ = [("loss_ce", C.c_float), ("loss_mse", C.c_float), ("margin", C.c_float),
                ("val_agreement", C.c_float), ("ms", C.c_float), ("mean_label_L", C.c_float),
                ("steps", C.c_uint32), ("labelled", C.c_uint32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class BuildStats(C.Structure):
    _fields_ = [("rand_draws", C.c_ulonglong), ("offers", C.c_ulonglong), ("pairs", C.c_ulonglong),
                ("chunks", C.c_uint), ("ms_join", C.c_float), ("ms_update", C.c_float), ("ms_total", C.c_float),
                ("levels", C.c_uint), ("ep", C.c_uint), ("conn_added", C.c_uint)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def declared_functions():
    """Names of every function the C header declares."""
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(wv_\w+)\s*\(", txt, re.M)))


def load(build_if_needed: bool = True):
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build_if_needed:
        path = _build.build()
    if not os.path.exists(path):
        raise WeavessError(-1, f"{path} is missing: build it with weavess_gb300.build.build()")
    L = C.CDLL(path)
    vp = C.c_void_p
    L.wv_ctx_create.argtypes = [C.POINTER(vp), C.c_int]
    L.wv_ctx_destroy.argtypes = [vp]
    L.wv_last_error.argtypes = [vp]
    L.wv_last_error.restype = C.c_char_p
    L.wv_srand.argtypes = [vp, C.c_uint]
    L.wv_set_rand_source.argtypes = [vp, vp]
    L.wv_rand.argtypes = [vp, C.POINTER(C.c_int)]
    L.wv_set_stream.argtypes = [vp, vp]
    L.wv_upload_base.argtypes = [vp, f32p, C.c_uint32, C.c_uint32]
    L.wv_upload_graph.argtypes = [vp, u32p, u32p, C.c_uint32, C.c_uint32, C.c_uint32]
    L.wv_set_eps.argtypes = [vp, vp, C.c_uint32]
    L.wv_load_hnsw.argtypes = [vp, u32p, C.c_size_t]
    L.wv_search_hnsw.argtypes = [vp, f32p, C.c_uint32, C.c_int, C.c_uint32, C.c_uint32, u32p, vp,
                                 C.POINTER(Counters)]
    L.wv_get_eps.argtypes = [vp, C.c_int, vp, C.c_uint32, C.POINTER(C.c_uint32)]
    L.wv_search.argtypes = [vp, f32p, C.c_uint32, C.c_int, C.c_uint32, C.c_uint32, vp, u32p, vp,
                            C.POINTER(Counters)]
    L.wv_search_batch.argtypes = [vp, f32p, C.c_uint32, C.c_int, u32p, u32p, C.c_uint32, u32p, vp,
                                  C.POINTER(Counters)]
    L.wv_search_device.argtypes = [vp, vp, C.c_uint32, C.c_uint32, C.c_uint32, vp, vp, vp, C.POINTER(Counters)]
    L.wv_draw_seeds.argtypes = [vp, C.c_uint32, C.c_int, C.c_uint32, u32p]
    L.wv_draw_seeds_device.argtypes = [vp, C.c_uint32, C.c_uint32, vp, C.c_uint32]
    L.wv_set_graph.argtypes = [vp, u32p, vp, u32p, C.c_uint32, C.c_uint32, C.c_uint32]
    L.wv_graph_width.argtypes = [vp, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
    L.wv_get_graph.argtypes = [vp, vp, vp, vp, C.c_uint32]
    L.wv_load_built_graph.argtypes = [vp]
    L.wv_init_random.argtypes = [vp, C.c_uint32, C.POINTER(BuildStats)]
    L.wv_init_rand.argtypes = [vp, C.c_uint32, C.POINTER(BuildStats)]
    L.wv_init_kdt.argtypes = [vp, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(BuildStats)]
    L.wv_nnd_refine.argtypes = [vp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                                C.POINTER(BuildStats)]
    L.wv_vamana_refine.argtypes = [vp, C.c_uint32, C.c_uint32, C.c_float, C.c_uint32, C.POINTER(BuildStats)]
    L.wv_set_build_mode.argtypes = [vp, C.c_int]
    L.wv_efanna_refine.argtypes = [vp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                                   C.POINTER(BuildStats)]
    L.wv_nsg_refine.argtypes = [vp, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(BuildStats)]
    L.wv_ssg_refine.argtypes = [vp, C.c_uint32, C.c_uint32, C.c_float, C.c_uint32, vp, C.POINTER(BuildStats)]
    L.wv_set_search_precision.argtypes = [vp, C.c_int, C.c_uint32]
    L.wv_set_search_expansion.argtypes = [vp, C.c_uint32]
    L.wv_candidate_distances.argtypes = [vp, f32p, C.c_uint32, u32p, C.c_uint32, f32p]
    L.wv_learn_default_params.argtypes = [C.POINTER(LearnParams)]
    L.wv_learn_default_params.restype = None
    L.wv_learn_fit.argtypes = [vp, f32p, C.c_uint32, C.POINTER(LearnParams), C.POINTER(LearnReport)]
    L.wv_search_learned.argtypes = [vp, f32p, C.c_uint32, C.c_uint32, u32p, vp, C.POINTER(Counters), vp]
    L.wv_search_learned_device.argtypes = [vp, vp, C.c_uint32, C.c_uint32, vp, vp, vp, C.POINTER(Counters)]
    L.wv_learn_set_margin.argtypes = [vp, C.c_float]
    L.wv_learn_plain_beam.argtypes = [vp, C.POINTER(C.c_uint32)]
    L.wv_learn_set_fallback.argtypes = [vp, C.c_float, C.c_uint32]
    L.wv_learn_predict.argtypes = [vp, f32p, C.c_uint32, u32p, f32p, f32p]
    L.wv_learn_assign.argtypes = [vp, u32p, C.c_uint32, u32p]
    L.wv_learn_param_count.argtypes = [C.c_uint32, C.c_uint32, C.POINTER(C.c_ulonglong)]
    L.wv_learn_grad.argtypes = [vp, f32p, u32p, f32p, C.c_uint32, C.c_uint32, f32p, C.c_float, f32p, f32p]
    L.wv_debug_sort.argtypes = [vp, f32p, u32p, u32p, C.c_uint32, C.c_int]
    u16p = np.ctypeslib.ndpointer(np.uint16, flags="C_CONTIGUOUS")
    L.wv_debug_gemm.argtypes = [vp, C.c_int, C.c_uint32, C.c_uint32, C.c_uint32, u16p, C.c_longlong, C.c_longlong,
                                u16p, C.c_longlong, C.c_longlong, f32p]
    L.wv_search_noalloc.argtypes = [vp, C.c_uint32, C.c_uint32, vp, vp, C.c_uint32, vp, C.c_uint32, vp, C.c_uint32,
                                    C.c_uint32, vp, vp, vp]
    L.wv_save_graph.argtypes = [vp, C.c_char_p, C.c_int]
    L.wv_load_graph.argtypes = [vp, C.c_char_p, C.c_int]
    L.wv_index_info.argtypes = [vp, C.c_int, vp, vp, C.c_uint32, C.POINTER(IndexInfo)]
    L.wv_plan_create.argtypes = [vp, C.POINTER(PlanParams), vp, vp, vp, vp, vp, vp, C.POINTER(vp)]
    L.wv_plan_run.argtypes = [vp, C.c_uint32]
    L.wv_plan_wait.argtypes = [vp, C.POINTER(Counters)]
    L.wv_plan_tune.argtypes = [vp, C.c_uint32, C.POINTER(TuneReport)]
    L.wv_plan_shape_of.argtypes = [vp, C.POINTER(PlanShape)]
    L.wv_plan_search_ms.argtypes = [vp, C.POINTER(C.c_float)]
    L.wv_plan_set_shape.argtypes = [vp, C.POINTER(PlanShape)]
    L.wv_plan_destroy.argtypes = [vp]
    _lib = L
    return L
