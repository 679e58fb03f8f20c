"""Python host mirror of the xavs2 GB300 hot-path library.

The product is the C-ABI shared library ``libxavs2gpu.so`` (declared in
include/xavs2_gb300.h).  This module loads it with ctypes and mirrors the
reference's primitive tables and the batched entry points for Python callers
(tests, bench).  There is no fallback: if the library is missing or no GPU is
present, loading fails with an exception.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("XAVS2GPU_LIB") or os.path.join(HERE, "libxavs2gpu.so")

# LumaPU order (source/common/pixel.h:50-65)
PU_W = [4, 8, 16, 32, 64, 8, 4, 16, 8, 32, 16, 64, 32, 16, 12, 16, 4, 32, 24, 32, 8, 64, 48, 64, 16]
PU_H = [4, 8, 16, 32, 64, 4, 8, 8, 16, 16, 32, 32, 64, 12, 16, 4, 16, 24, 32, 8, 32, 48, 64, 16, 64]
TU_PARTS = [0, 1, 2, 3, 4, 15, 16, 19, 20, 23, 24]

_P = ctypes.c_void_p
_I = ctypes.c_int
_S = ctypes.c_ssize_t


class MeParams(ctypes.Structure):
    _fields_ = [("search_range", ctypes.c_int32), ("lambda_factor", ctypes.c_int32),
                ("use_hadamard", ctypes.c_int32), ("fractional_me", ctypes.c_int32),
                ("fast_sub_me", ctypes.c_int32), ("enable_pmvr", ctypes.c_int32)]


class Pu(ctypes.Structure):
    _fields_ = [("x", ctypes.c_int16), ("y", ctypes.c_int16), ("part", ctypes.c_uint8),
                ("ref", ctypes.c_uint8), ("mvp_x", ctypes.c_int16), ("mvp_y", ctypes.c_int16),
                ("min_x", ctypes.c_int16), ("min_y", ctypes.c_int16),
                ("max_x", ctypes.c_int16), ("max_y", ctypes.c_int16)]


PU_DTYPE = np.dtype([("x", "<i2"), ("y", "<i2"), ("part", "u1"), ("ref", "u1"),
                     ("mvp_x", "<i2"), ("mvp_y", "<i2"), ("min_x", "<i2"), ("min_y", "<i2"),
                     ("max_x", "<i2"), ("max_y", "<i2")])
RESULT_DTYPE = np.dtype([("bmv_x", "<i2"), ("bmv_y", "<i2"), ("bcost", "<i4"), ("mvcost", "<i4"),
                         ("imv_x", "<i2"), ("imv_y", "<i2"), ("icost", "<i4")])
TQ_DTYPE = np.dtype([("offset", "<i8"), ("coef_offset", "<i8"), ("part", "<i4"), ("qp", "<i4"),
                     ("flags", "<i4"), ("pad_", "<i4")])
COST_JOB_DTYPE = np.dtype([("off1", "<i8"), ("off2", "<i8"), ("s1", "<i4"), ("s2", "<i4"),
                           ("part", "<i4"), ("pad_", "<i4")])

_SIGS = {
    "xavs2gpu_init": (_I, [_I]),
    "xavs2gpu_get_status": (_I, []),
    "xavs2gpu_get_error": (ctypes.c_char_p, []),
    "xavs2gpu_clear_error": (None, []),
    "xavs2gpu_set_abort_on_error": (None, [_I]),
    "xavs2gpu_set_percall_mode": (None, [_I]),
    "xavs2gpu_percall_in_place": (_I, []),
    "xavs2gpu_kernel_launches": (ctypes.c_uint64, []),
    "xavs2gpu_version": (ctypes.c_char_p, []),
    "xavs2gpu_copy_d2h": (_I, [_P, _P, ctypes.c_size_t]),
    "xavs2gpu_copy_h2d": (_I, [_P, _P, ctypes.c_size_t]),
    "xavs2gpu_pixel_init": (None, [ctypes.c_uint32, _P]),
    "xavs2gpu_mad_init": (None, [ctypes.c_uint32, _P]),
    "xavs2gpu_dct_init": (None, [ctypes.c_uint32, _P]),
    "xavs2gpu_quant_init": (None, [ctypes.c_uint32, _P]),
    "xavs2gpu_get_block_ssd": (_I, [_P, _S, _P, _S, _I, _I]),
    "xavs2gpu_pixel_average": (None, [_P, _I, _P, _I, _P, _I, _I, _I]),
    "xavs2gpu_mad_NxN": (_I, [_P, _I, _I]),
    "xavs2gpu_intpl_luma_hor": (None, [_P, _I, _P, _I, _P, _I, _I, _I, _P]),
    "xavs2gpu_intpl_luma_ver": (None, [_P, _I, _P, _I, _I, _I, _P]),
    "xavs2gpu_intpl_luma_ext": (None, [_P, _I, _P, _I, _I, _I, _P]),
    "xavs2gpu_intpl_luma_ver_x3": (None, [_P, _I, _P, _I, _I, _I, _P]),
    "xavs2gpu_intpl_luma_hor_x3": (None, [_P, _I, _P, _I, _P, _I, _I, _I, _P]),
    "xavs2gpu_intpl_luma_ext_x3": (None, [_P, _I, _P, _I, _I, _I, _P]),
    "xavs2gpu_intpl_luma_block_hor": (None, [_P, _I, _P, _I, _I, _I, _P]),
    "xavs2gpu_intpl_luma_block_ver": (None, [_P, _I, _P, _I, _I, _I, _P]),
    "xavs2gpu_intpl_luma_block_ext": (None, [_P, _I, _P, _I, _I, _I, _P, _P]),
    "xavs2gpu_intpl_chroma_block_hor": (None, [_P, _I, _P, _I, _I, _I, _P]),
    "xavs2gpu_intpl_chroma_block_ver": (None, [_P, _I, _P, _I, _I, _I, _P]),
    "xavs2gpu_intpl_chroma_block_ext": (None, [_P, _I, _P, _I, _I, _I, _P, _P]),
    "xavs2gpu_dct_32x32_half": (None, [_P, _P, _I]),
    "xavs2gpu_dct_64x64_half": (None, [_P, _P, _I]),
    "xavs2gpu_transform_4x4_2nd": (None, [_P, _I]),
    "xavs2gpu_inv_transform_4x4_2nd": (None, [_P, _I]),
    "xavs2gpu_transform_2nd": (None, [_P, _I, _I, _I, _I]),
    "xavs2gpu_inv_transform_2nd": (None, [_P, _I, _I, _I, _I]),
    "xavs2gpu_quant": (_I, [_P, _I, _I, _I, _I]),
    "xavs2gpu_dequant": (None, [_P, _I, _I, _I]),
    "xavs2gpu_quant_weighted": (_I, [_P, _I, _I, _I, _I, _P]),
    "xavs2gpu_abs_coeff": (None, [_P, _P, _I]),
    "xavs2gpu_add_sign": (_I, [_P, _P, _I]),
    "xavs2gpu_cost_batch": (_I, [_I, _P, _I, _P, _P, _P, _P]),
    "xavs2gpu_interpolate_frame": (_I, [_P, _I, _I, _I, _I, _P, _I, _P]),
    "xavs2gpu_tq_batch_host": (_I, [_P, _I, _P, _P, _P, _P, _I]),
    "xavs2gpu_expand_border": (_I, [_P, _I, _I, _I, _I, _P]),
    "xavs2gpu_tq_batch": (_I, [_P, _I, _P, _P, _P, _P, _P]),
    "xavs2gpu_pu_set_limits": (None, [_P, _I, _I, _I, _I]),
    "xavs2gpu_me_create": (_P, [_I, _I, _I, _I]),
    "xavs2gpu_me_destroy": (None, [_P]),
    "xavs2gpu_me_set_picture_host": (_I, [_P, _I, _P, _S]),
    "xavs2gpu_me_set_picture_device": (_I, [_P, _I, _P, _S]),
    "xavs2gpu_me_set_pus": (_I, [_P, _P, _I]),
    "xavs2gpu_me_run": (_I, [_P, _P]),
    "xavs2gpu_me_get_results": (_I, [_P, _P]),
    "xavs2gpu_me_sync": (_I, [_P]),
    "xavs2gpu_me_results_device": (_P, [_P]),
    "xavs2gpu_me_plane_device": (_P, [_P, _I, _I]),
    "xavs2gpu_me_plane_stride": (_I, [_P]),
    "xavs2gpu_me_plane_pad": (_I, [_P]),
    "xavs2gpu_me_window_tma": (_I, [_P]),
    "xavs2gpu_me_stream": (_P, [_P]),
    "xavs2gpu_me_plan_stats": (None, [_P, _P, _P, _P]),
    "xavs2gpu_me_get_plane": (_I, [_P, _I, _I, _P, _S]),
    "xavs2gpu_me_set_profiling": (None, [_P, _I]),
    "xavs2gpu_me_phase_ms": (_I, [_P, _P]),
    "xavs2gpu_me_set_tuning": (_I, [_P, _P]),
    "xavs2gpu_me_get_tuning": (_I, [_P, _P]),
    "xavs2gpu_me_prepare": (_I, [_P, _P]),
    "xavs2gpu_me_autotune": (_I, [_P, _P, _I, _P]),
    "xavs2gpu_me_session_info": (None, [_P, _P, _P, _P, _P]),
    "xavs2gpu_me_session_pus": (_I, [_P, _P]),
    "xavs2gpu_chain_create": (_P, [_P, _P, _I, _I, _I]),
    "xavs2gpu_chain_destroy": (None, [_P]),
    "xavs2gpu_chain_source": (_P, [_P, _I]),
    "xavs2gpu_chain_run": (_I, [_P, _P]),
    "xavs2gpu_chain_capture": (_I, [_P, _P]),
    "xavs2gpu_chain_launch": (_I, [_P]),
    "xavs2gpu_chain_get_outputs": (_I, [_P, _P]),
    "xavs2gpu_chain_autotune": (_I, [_P, _P, _I, _P]),
    "xavs2gpu_chain_get_tuning": (_I, [_P, _P]),
    "xavs2gpu_chain_set_tuning": (_I, [_P, _P]),
    "xavs2gpu_chain_graph_kernels": (_I, [_P]),
    "xavs2gpu_me_batch_create": (_P, []),
    "xavs2gpu_me_batch_destroy": (None, [_P]),
    "xavs2gpu_me_batch_run": (_I, [_P, _P, _I, _P, _P]),
    "xavs2gpu_me_set_stream": (_I, [_P, _P]),
    "xavs2gpu_me_rotate_refs": (_I, [_P]),
    "xavs2gpu_me_plane_table_device": (_P, [_P]),
    "xavs2gpu_server_create": (_P, [_P]),
    "xavs2gpu_server_destroy": (None, [_P]),
    "xavs2gpu_server_open_stream": (_I, [_P, _I, _I, _P, _I, _P, _I, _I]),
    "xavs2gpu_server_submit": (_I, [_P, _I, _P, _S, ctypes.c_int64]),
    "xavs2gpu_server_poll": (_I, [_P, _P, _I, _I]),
    "xavs2gpu_server_stats": (None, [_P, _P, _P, _P, _P]),
    "xavs2gpu_server_timing": (None, [_P, _P, _P]),
    "xavs2gpu_intra_pred_dc": (None, [_P, _P, _I, _I, _I, _I]),
    "xavs2gpu_intra_pred_plane": (None, [_P, _P, _I, _I, _I, _I]),
    "xavs2gpu_intra_pred_bilinear": (None, [_P, _P, _I, _I, _I, _I]),
    "xavs2gpu_intra_pred_ver": (None, [_P, _P, _I, _I, _I, _I]),
    "xavs2gpu_intra_pred_hor": (None, [_P, _P, _I, _I, _I, _I]),
    "xavs2gpu_intra_pred_ang": (None, [_P, _P, _I, _I, _I, _I]),
    "xavs2gpu_intra_pred_init": (None, [ctypes.c_uint32, _P]),
    "xavs2gpu_intra_rmd_batch": (_I, [_P, _I, _P, _P, _I, _P, _P, _P]),
    "xavs2gpu_intra_fill_edges": (_I, [_P, _I, _P, _I, _I, _I, _P, ctypes.c_int64, _P]),
    "xavs2gpu_deblock_luma_ver": (None, [_P, _I, _I, _I, _P]),
    "xavs2gpu_deblock_luma_hor": (None, [_P, _I, _I, _I, _P]),
    "xavs2gpu_deblock_chroma_ver": (None, [_P, _P, _I, _I, _I, _P]),
    "xavs2gpu_deblock_chroma_hor": (None, [_P, _P, _I, _I, _I, _P]),
    "xavs2gpu_deblock_init": (None, [ctypes.c_uint32, _P]),
    "xavs2gpu_sao_block": (None, [_P, _I, _P, _I, _I, _I, _P, _P]),
    "xavs2gpu_sao_init": (None, [ctypes.c_uint32, _P]),
    "xavs2gpu_deblock_picture": (_I, [_P, _I, _P, _P, _I, _I, _I, _I, _P, _P]),
    "xavs2gpu_lowres_filter": (None, [_P, _I, _P, _I, _I, _I]),
    "xavs2gpu_loopfilter_picture": (_I, [_P, _P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _P, _P, _P]),
    "xavs2gpu_skip_costs": (_I, [_P, _P, _I, ctypes.c_double, _I, _P, _P, _P, _P]),
    "xavs2gpu_lowres_picture": (_I, [_P, _I, _P, _I, _I, _I, _P]),
    "xavs2gpu_lookahead_picture": (_I, [_P, _I, _I, _I, _P, _I, _P, _P, _P, _P]),
    "xavs2gpu_sao_picture": (_I, [_P, _P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _P, _I, _P]),
}

_PIXEL_CMP = ["sad", "satd", "sa8d", "ssd"]
_lib = None


def _shape(part):
    return "%dx%d" % (PU_W[part], PU_H[part])


def load():
    """Load libxavs2gpu.so (fails loudly if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libxavs2gpu.so is not built; run __graft_entry__.build() first")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in _SIGS.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    for part in range(25):
        s = _shape(part)
        for k in _PIXEL_CMP:
            f = getattr(lib, "xavs2gpu_pixel_%s_%s" % (k, s))
            f.restype, f.argtypes = _I, [_P, _S, _P, _S]
        for k, args in (("sad_x3", [_P, _P, _P, _P, _S, _P]), ("sad_x4", [_P, _P, _P, _P, _P, _S, _P]),
                        ("avg", [_P, _S, _P, _S, _P, _S, _I]), ("sub_ps", [_P, _S, _P, _P, _S, _S]),
                        ("add_ps", [_P, _S, _P, _P, _S, _S])):
            f = getattr(lib, "xavs2gpu_pixel_%s_%s" % (k, s))
            f.restype, f.argtypes = None, args
        for k in ("pp", "ps", "sp", "ss"):
            f = getattr(lib, "xavs2gpu_blockcopy_%s_%s" % (k, s))
            f.restype, f.argtypes = None, [_P, _S, _P, _S]
    for part in TU_PARTS:
        s = _shape(part)
        for k in ("dct", "idct"):
            f = getattr(lib, "xavs2gpu_%s_%s" % (k, s))
            f.restype, f.argtypes = None, [_P, _P, _I]
    if lib.xavs2gpu_init(0) != 0:
        raise RuntimeError("xavs2gpu_init failed: %s" % lib.xavs2gpu_get_error())
    _lib = lib
    return lib


def fn(name):
    return getattr(load(), name)


def pixel_fn(kind, part):
    """The drop-in for table entry `kind` (sad, satd, ..., copy_pp) and shape."""
    s = _shape(part)
    if kind.startswith("copy_"):
        return fn("xavs2gpu_blockcopy_%s_%s" % (kind[5:], s))
    return fn("xavs2gpu_pixel_%s_%s" % (kind, s))


def dct_fn(kind, part):
    return fn("xavs2gpu_%s_%s" % (kind, _shape(part)))


def ptr(a, off=0):
    return ctypes.c_void_p(a.ctypes.data + off * a.itemsize)


class MeSession:
    """Batched full-search + sub-pel motion search over a PU list."""

    def __init__(self, width, height, num_refs, max_pus):
        self.lib = load()
        self.h = self.lib.xavs2gpu_me_create(width, height, num_refs, max_pus)
        if not self.h:
            raise RuntimeError("xavs2gpu_me_create failed: %s" % self.lib.xavs2gpu_get_error())
        self.width, self.height, self.num_refs = width, height, num_refs
        self.n = 0

    def close(self):
        if self.h:
            self.lib.xavs2gpu_me_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc != 0:
            raise RuntimeError("%s failed (%d): %s" % (what, rc, self.lib.xavs2gpu_get_error()))

    def set_picture(self, slot, img):
        img = np.ascontiguousarray(img, dtype=np.uint8)
        self._check(self.lib.xavs2gpu_me_set_picture_host(self.h, slot, ptr(img), img.shape[1]), "set_picture")

    def set_picture_device(self, slot, dev_ptr, stride):
        self._check(self.lib.xavs2gpu_me_set_picture_device(self.h, slot, ctypes.c_void_p(dev_ptr), stride),
                    "set_picture_device")

    def set_pus(self, pus):
        pus = np.ascontiguousarray(pus, dtype=PU_DTYPE)
        self._pus = pus
        self.n = len(pus)
        self._check(self.lib.xavs2gpu_me_set_pus(self.h, ptr(pus), len(pus)), "set_pus")

    def run(self, params):
        self._check(self.lib.xavs2gpu_me_run(self.h, ctypes.byref(params)), "run")

    def results(self, out=None):
        """The results (one per PU) into `out` (e.g. a page-locked array) or a new array."""
        if out is None:
            out = np.zeros(self.n, RESULT_DTYPE)
        self._check(self.lib.xavs2gpu_me_get_results(self.h, ptr(out)), "get_results")
        return out

    def sync(self):
        self._check(self.lib.xavs2gpu_me_sync(self.h), "sync")

    def plane_ptr(self, slot, k):
        return self.lib.xavs2gpu_me_plane_device(self.h, slot, k)

    def get_plane(self, slot, k, pad=80):
        """Plane k of a slot including its `pad`-pixel margin, as a numpy array."""
        out = np.zeros((self.height + 2 * pad, self.width + 2 * pad), np.uint8)
        self._check(self.lib.xavs2gpu_me_get_plane(self.h, slot, k, ptr(out), out.shape[1]), "get_plane")
        return out

    def plane_stride(self):
        return self.lib.xavs2gpu_me_plane_stride(self.h)

    def stream(self):
        return self.lib.xavs2gpu_me_stream(self.h)

    def window_tma(self):
        """Whether the CTU search copies its windows with the TMA."""
        return bool(self.lib.xavs2gpu_me_window_tma(self.h))

    def set_profiling(self, on=True):
        self.lib.xavs2gpu_me_set_profiling(self.h, 1 if on else 0)

    def phase_ms(self):
        out = (ctypes.c_float * 4)()
        self._check(self.lib.xavs2gpu_me_phase_ms(self.h, out), "phase_ms")
        return list(out)

    def autotune(self, params, reps=2):
        """Picks the fastest refinement launch shapes (results unchanged)."""
        ms = ctypes.c_float()
        self._check(self.lib.xavs2gpu_me_autotune(self.h, ctypes.byref(params), reps, ctypes.byref(ms)), "autotune")
        t = MeTuning()
        self.lib.xavs2gpu_me_get_tuning(self.h, ctypes.byref(t))
        return ms.value, (t.refine_split_px, t.refine_block, t.cu_groups)

    def set_stream(self, stream):
        self._check(self.lib.xavs2gpu_me_set_stream(self.h, ctypes.c_void_p(stream) if stream else None),
                    "set_stream")

    def rotate_refs(self):
        self._check(self.lib.xavs2gpu_me_rotate_refs(self.h), "rotate_refs")

    def plan_stats(self):
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self.lib.xavs2gpu_me_plan_stats(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
        return a.value, b.value, c.value


class MeBatch:
    """Several sessions searched by one launch of each kernel."""

    def __init__(self):
        self.lib = load()
        self.h = self.lib.xavs2gpu_me_batch_create()

    def run(self, sessions, params, stream=None):
        arr = (ctypes.c_void_p * len(sessions))(*[s.h for s in sessions])
        rc = self.lib.xavs2gpu_me_batch_run(self.h, arr, len(sessions), ctypes.byref(params),
                                            ctypes.c_void_p(stream) if stream else None)
        if rc != 0:
            raise RuntimeError("me_batch_run failed (%d): %s" % (rc, self.lib.xavs2gpu_get_error()))

    def close(self):
        if self.h:
            self.lib.xavs2gpu_me_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_int64), ("max_batch_pixels", ctypes.c_int64),
                ("max_batch_frames", ctypes.c_int32), ("qp", ctypes.c_int32), ("me", MeParams),
                ("hbm_reserve_bytes", ctypes.c_int64), ("batch_pixels_target", ctypes.c_int64)]


SERVER_RESULT_DTYPE = np.dtype([("stream", "<i4"), ("frame", "<i4"), ("tag", "<i8"), ("t_submit_ns", "<i8"),
                                ("t_done_ns", "<i8"), ("hash", "<u8"), ("batch_frames", "<i4"),
                                ("ref_only", "<i4")])


def output_hash(recon, coef, results):
    """The serving checksum of a picture (xavs2gpu_server_result_t.hash):
    sum over the 32-bit words w_i of [reconstruction | levels | search
    results] of (w_i + 1) * (2 i + 1), modulo 2^64."""
    words = np.concatenate([np.ascontiguousarray(recon).view(np.uint32).ravel(),
                            np.ascontiguousarray(coef).view(np.uint32).ravel(),
                            np.ascontiguousarray(results).view(np.uint32).ravel()]).astype(np.uint64)
    idx = np.arange(len(words), dtype=np.uint64)
    with np.errstate(over="ignore"):
        return int(np.sum((words + np.uint64(1)) * (np.uint64(2) * idx + np.uint64(1)), dtype=np.uint64))


class Server:
    """Continuous-batching server over many streams (xavs2gpu_server_*)."""

    def __init__(self, cfg):
        self.lib = load()
        self.cfg = cfg
        self.h = self.lib.xavs2gpu_server_create(ctypes.byref(cfg))
        if not self.h:
            raise RuntimeError("xavs2gpu_server_create failed: %s" % self.lib.xavs2gpu_get_error())
        self._keep = []

    def open_stream(self, width, height, pus, cus, ring=8):
        pus = np.ascontiguousarray(pus, dtype=PU_DTYPE)
        cus = np.ascontiguousarray(cus, dtype=CU_DTYPE)
        sid = self.lib.xavs2gpu_server_open_stream(self.h, width, height, ptr(pus), len(pus), ptr(cus), len(cus),
                                                   ring)
        return sid

    def submit(self, sid, img, tag=0):
        img = np.ascontiguousarray(img, dtype=np.uint8)
        return self.lib.xavs2gpu_server_submit(self.h, sid, ptr(img), img.shape[1], tag)

    def poll(self, max_results=4096, timeout_ms=0):
        out = np.zeros(max_results, SERVER_RESULT_DTYPE)
        k = self.lib.xavs2gpu_server_poll(self.h, ptr(out), max_results, timeout_ms)
        if k < 0:
            raise RuntimeError("server_poll failed (%d)" % k)
        return out[:k]

    def stats(self):
        v = [ctypes.c_int64() for _ in range(4)]
        self.lib.xavs2gpu_server_stats(self.h, *[ctypes.byref(x) for x in v])
        g, h = ctypes.c_double(), ctypes.c_double()
        self.lib.xavs2gpu_server_timing(self.h, ctypes.byref(g), ctypes.byref(h))
        return {"hbm_used": v[0].value, "batches": v[1].value, "frames": v[2].value, "pending": v[3].value,
                "gpu_ms": g.value, "host_enqueue_ms": h.value}

    def close(self):
        if self.h:
            self.lib.xavs2gpu_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MeTuning(ctypes.Structure):
    _fields_ = [("refine_split_px", ctypes.c_int32), ("refine_block", ctypes.c_int32), ("cu_groups", ctypes.c_int32),
                ("pad_", ctypes.c_int32)]


class ChainTuning(ctypes.Structure):
    _fields_ = [("me", MeTuning), ("tq_warps", ctypes.c_int32), ("pad_", ctypes.c_int32)]


class ChainOutputs(ctypes.Structure):
    _fields_ = [("coef", _P), ("recon_residual", _P), ("nnz", _P), ("blocks", _P), ("recon", _P),
                ("choice", _P), ("n_residual", ctypes.c_int64), ("n_coef", ctypes.c_int64),
                ("cands", _P), ("cand_cost", _P), ("dist", _P), ("n_cands", ctypes.c_int64)]


INTRA_BLOCK_DTYPE = np.dtype([("edge_offset", "<i8"), ("fenc_offset", "<i8"), ("width", "<i2"), ("height", "<i2"),
                              ("dc_avail", "<i2"), ("mpm", "i1", (2,)), ("num_for_rdo", "<i4"), ("pad_", "<i4")])
INTRA_RESULT_DTYPE = np.dtype([("cost", "<f8", (33,)), ("cand_cost", "<f8", (9,)), ("cand_mode", "<i4", (9,)),
                               ("num_for_rdo", "<i4")])
# xavs2gpu_intra_edge_job_t; avail = MD_I_* bits (0 left, 1 top, 2 left-down, 3 top-right, 4 top-left)
INTRA_EDGE_JOB_DTYPE = np.dtype([("edge_offset", "<i8"), ("x", "<i4"), ("y", "<i4"), ("width", "<i2"),
                                 ("height", "<i2"), ("avail", "<i4")])


DEBLOCK_SCU_DTYPE = np.dtype([("type", "u1", (2,)), ("flag", "u1", (2, 2)), ("alpha", "u1", (2,)),
                              ("beta", "u1", (2,)), ("alpha_c", "u1", (2,)), ("beta_c", "u1", (2,)),
                              ("pad_", "u1", (2,))])
SKIP_CAND_DTYPE = np.dtype([("x", "<i2"), ("y", "<i2"), ("size_log2", "u1"), ("n_pu", "u1"), ("pad_", "<i2"),
                            ("cu", "<i4"), ("rate", "<i4"), ("ref", "i1", (4, 2)), ("mv", "<i2", (4, 2, 2))])
SAO_LCU_DTYPE = np.dtype([("type", "i1", (3,)), ("avail", "u1"), ("offset", "i1", (3, 32))])


class IntraParams(ctypes.Structure):
    _fields_ = [("lambda_", ctypes.c_double), ("use_hadamard", ctypes.c_int32), ("rough", ctypes.c_int32),
                ("dist2", ctypes.c_int32), ("dist1", ctypes.c_int32)]


# xavs2gpu_cu_choice_t: chosen candidate, its partition mode and TU variant
CHOICE_DTYPE = np.dtype([("cand", "<i4"), ("mode", "<i2"), ("split", "<i2")])
# xavs2gpu_cand_t
CAND_DTYPE = np.dtype([("cu", "<i4"), ("mode", "i1"), ("split_type", "i1"), ("pad_", "<i2"),
                       ("res_offset", "<i8"), ("coef_offset", "<i8")])


class Chain:
    """One P picture of the hot path over leaf CUs (xavs2gpu_chain_*): the
    session `sess` must hold the PU list `cus` refers to."""

    def __init__(self, sess, cus, qp, feedback=False):
        self.lib = load()
        self.sess = sess
        self.cus = np.ascontiguousarray(cus, dtype=CU_DTYPE)
        self.h = self.lib.xavs2gpu_chain_create(sess.h, ptr(self.cus), len(self.cus), qp, 1 if feedback else 0)
        if not self.h:
            raise RuntimeError("xavs2gpu_chain_create failed: %s" % self.lib.xavs2gpu_get_error())

    def close(self):
        if self.h:
            self.lib.xavs2gpu_chain_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc != 0:
            raise RuntimeError("%s failed (%d): %s" % (what, rc, self.lib.xavs2gpu_get_error()))

    def source(self, idx):
        """Device pointer of source picture idx (0: current, 1 + r: reference r)."""
        return self.lib.xavs2gpu_chain_source(self.h, idx)

    def run(self, params):
        self._check(self.lib.xavs2gpu_chain_run(self.h, ctypes.byref(params)), "chain_run")

    def capture(self, params):
        self._check(self.lib.xavs2gpu_chain_capture(self.h, ctypes.byref(params)), "chain_capture")

    def launch(self):
        self._check(self.lib.xavs2gpu_chain_launch(self.h), "chain_launch")

    def graph_kernels(self):
        return self.lib.xavs2gpu_chain_graph_kernels(self.h)

    def autotune(self, params, reps=2):
        ms = ctypes.c_float()
        self._check(self.lib.xavs2gpu_chain_autotune(self.h, ctypes.byref(params), reps, ctypes.byref(ms)),
                    "chain_autotune")
        return ms.value

    def tuning(self):
        t = ChainTuning()
        self._check(self.lib.xavs2gpu_chain_get_tuning(self.h, ctypes.byref(t)), "chain_get_tuning")
        return t

    def set_tuning(self, t):
        self._check(self.lib.xavs2gpu_chain_set_tuning(self.h, ctypes.byref(t)), "chain_set_tuning")

    def outputs(self):
        o = ChainOutputs()
        self._check(self.lib.xavs2gpu_chain_get_outputs(self.h, ctypes.byref(o)), "chain_get_outputs")
        return o

    def download(self):
        """Every output of the last picture on the host (after a session
        sync): candidate table, TU descriptors, nnz, levels, reconstructed
        residual, candidate search costs and SSDs, per-CU choices and the
        reconstructed picture."""
        o = self.outputs()
        self.lib.xavs2gpu_me_sync(self.sess.h)
        n = int(o.n_cands)
        W, H = self.sess.width, self.sess.height

        def d2h(p, count, dtype):
            out = np.zeros(count, dtype)
            if count:
                rc = self.lib.xavs2gpu_copy_d2h(out.ctypes.data_as(ctypes.c_void_p), ctypes.c_void_p(p), out.nbytes)
                self._check(rc, "copy_d2h")
            return out
        return {"cands": d2h(o.cands, n, CAND_DTYPE), "blocks": d2h(o.blocks, 5 * n, TQ_DTYPE),
                "nnz": d2h(o.nnz, 5 * n, np.int32), "coef": d2h(o.coef, int(o.n_coef), np.int16),
                "rres": d2h(o.recon_residual, int(o.n_residual), np.int16),
                "cost": d2h(o.cand_cost, n, np.int32), "dist": d2h(o.dist, 2 * n, np.int32).reshape(n, 2),
                "choice": d2h(o.choice, len(self.cus), CHOICE_DTYPE),
                "recon": d2h(o.recon, W * H, np.uint8).reshape(H, W)}


def set_limits(pus, width, height, vmin=-2048, vmax=2047):
    """Fill min/max search limits of a PU array as pred_inter_search_single
    does (md_inter.c:910-926)."""
    w = np.array(PU_W)[pus["part"]]
    h = np.array(PU_H)[pus["part"]]
    x = pus["x"].astype(np.int64)
    y = pus["y"].astype(np.int64)
    mn = np.clip((-64 - x) * 4, -8192, 8191)
    mx = np.clip((width + 64 - x - w) * 4, -8192, 8191)
    pus["min_x"] = (mn >> 2) + 6
    pus["max_x"] = (mx >> 2) - 6
    mn = np.clip((-64 - y) * 4, vmin, vmax)
    mx = np.clip((height + 64 - y - h) * 4, vmin, vmax)
    pus["min_y"] = (mn >> 2) + 6
    pus["max_y"] = (mx >> 2) - 6
    return pus


# CU-quadtree PU set of a 64x64 CTU (the slots of the shared-window kernel):
# for CU sizes 64/32/16 the 13 PUs of 2Nx2N, 2NxN, Nx2N, 2NxnU, 2NxnD,
# nLx2N, nRx2N; for 8x8 CUs 8x8, 8x4 x2, 4x8 x2 and the four 4x4 blocks.
def _part(w, h):
    for i in range(25):
        if PU_W[i] == w and PU_H[i] == h:
            return i
    raise ValueError((w, h))


def _cu_modes(n, cx, cy):
    h2, q, q3 = n // 2, n // 4, 3 * n // 4
    return [(cx, cy, n, n), (cx, cy, n, h2), (cx, cy + h2, n, h2), (cx, cy, h2, n), (cx + h2, cy, h2, n),
            (cx, cy, n, q), (cx, cy + q, n, q3), (cx, cy, n, q3), (cx, cy + q3, n, q),
            (cx, cy, q, n), (cx + q, cy, q3, n), (cx, cy, q3, n), (cx + q3, cy, q, n)]


def ctu_pu_layout():
    out = []
    for cy in range(0, 64, 8):
        for cx in range(0, 64, 8):
            out += [(cx, cy, 8, 8), (cx, cy, 8, 4), (cx, cy + 4, 8, 4), (cx, cy, 4, 8), (cx + 4, cy, 4, 8),
                    (cx, cy, 4, 4), (cx + 4, cy, 4, 4), (cx, cy + 4, 4, 4), (cx + 4, cy + 4, 4, 4)]
    for n in (16, 32, 64):
        for cy in range(0, 64, n):
            for cx in range(0, 64, n):
                out += _cu_modes(n, cx, cy)
    return out


def frame_pus(width, height, num_refs, mvp=(0, 0), vmin=-2048, vmax=2047):
    """Every PU of the CU-quadtree layout of each CTU that lies fully inside
    the picture, for each reference, with search limits set."""
    lay = np.array([(x, y, _part(w, h), w, h) for (x, y, w, h) in ctu_pu_layout()], np.int32)
    rows = []
    for ref in range(num_refs):
        for y0 in range(0, height, 64):
            for x0 in range(0, width, 64):
                x = lay[:, 0] + x0
                y = lay[:, 1] + y0
                ok = (x + lay[:, 3] <= width) & (y + lay[:, 4] <= height)
                n = int(ok.sum())
                a = np.zeros(n, PU_DTYPE)
                a["x"], a["y"], a["part"], a["ref"] = x[ok], y[ok], lay[ok, 2], ref
                a["mvp_x"], a["mvp_y"] = mvp
                rows.append(a)
    pus = np.concatenate(rows)
    return set_limits(pus, width, height, vmin, vmax)


# ---- CU quadtree from a split map (full-frame chain) ------------------------
CU_DTYPE = np.dtype([("x", "<i2"), ("y", "<i2"), ("size", "<i2"), ("pad_", "<i2"), ("pu", "<i4", (4,)),
                     ("offset", "<i8"), ("coef_offset", "<i8")])
_SQUARE_PART = {4: 0, 8: 1, 16: 2, 32: 3, 64: 4}


def split_map_cus(width, height, seed, p_split=(0.5, 0.5, 0.5)):
    """Leaf CUs (x, y, size) of every CTU from a seeded split map: a CU of
    size 64/32/16 splits into four with probability p_split[depth]; a CU
    that is not fully inside the picture always splits (8x8 CUs outside are
    dropped), as the encoder's quadtree does at picture borders."""
    rng = np.random.default_rng(seed)
    out = []

    def visit(x, y, n, depth):
        inside = x + n <= width and y + n <= height
        if x >= width or y >= height:
            return
        if n == 8:
            if inside:
                out.append((x, y, 8))
            return
        if not inside or rng.random() < p_split[depth]:
            h = n // 2
            for dy in (0, h):
                for dx in (0, h):
                    visit(x + dx, y + dy, h, depth + 1)
        else:
            out.append((x, y, n))

    for y0 in range(0, height, 64):
        for x0 in range(0, width, 64):
            visit(x0, y0, 64, 0)
    return out


def cu_pus(cus, width, height, num_refs, mvp=(0, 0), with_4x4=False):
    """The PUs an encoder searches for the leaf CUs `cus` (every partition
    mode of the CU: 2Nx2N, 2NxN, Nx2N and the four AMP modes for 16..64;
    8x8, 8x4, 4x8 for 8x8 CUs, plus 4x4 when `with_4x4`), for each
    reference, and the CU records (CU_DTYPE) with the index of each CU's
    2Nx2N PU per reference and packed residual / level offsets."""
    rows = []
    for (x, y, n) in cus:
        if n == 8:
            modes = [(x, y, 8, 8), (x, y, 8, 4), (x, y + 4, 8, 4), (x, y, 4, 8), (x + 4, y, 4, 8)]
            if with_4x4:
                modes += [(x, y, 4, 4), (x + 4, y, 4, 4), (x, y + 4, 4, 4), (x + 4, y + 4, 4, 4)]
        else:
            modes = _cu_modes(n, x, y)
        rows.append(modes)
    per_ref = sum(len(m) for m in rows)
    pus = np.zeros(per_ref * num_refs, PU_DTYPE)
    cu = np.zeros(len(cus), CU_DTYPE)
    cu["pu"] = -1
    flat = [t for m in rows for t in m]
    xs = np.array([t[0] for t in flat], np.int16)
    ys = np.array([t[1] for t in flat], np.int16)
    parts = np.array([_part(t[2], t[3]) for t in flat], np.uint8)
    first = np.cumsum([0] + [len(m) for m in rows])[:-1]
    for r in range(num_refs):
        sl = slice(r * per_ref, (r + 1) * per_ref)
        pus["x"][sl], pus["y"][sl], pus["part"][sl], pus["ref"][sl] = xs, ys, parts, r
        cu["pu"][:, r] = r * per_ref + first
    pus["mvp_x"], pus["mvp_y"] = mvp
    size = np.array([n for (_, _, n) in cus], np.int64)
    cu["x"] = [c[0] for c in cus]
    cu["y"] = [c[1] for c in cus]
    cu["size"] = size
    area = size * size
    ncoef = np.where(size == 64, area // 4, area)
    cu["offset"] = np.cumsum(area) - area
    cu["coef_offset"] = np.cumsum(ncoef) - ncoef
    return set_limits(pus, width, height), cu
