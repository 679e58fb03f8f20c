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
LIB_PATH = os.path.join(HERE, "libxavs2gpu.so")

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
    "xavs2gpu_kernel_launches": (ctypes.c_uint64, []),
    "xavs2gpu_version": (ctypes.c_char_p, []),
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
    "xavs2gpu_me_stream": (_P, [_P]),
    "xavs2gpu_me_plan_stats": (None, [_P, _P, _P, _P]),
    "xavs2gpu_me_get_plane": (_I, [_P, _I, _I, _P, _S]),
    "xavs2gpu_me_set_profiling": (None, [_P, _I]),
    "xavs2gpu_me_phase_ms": (_I, [_P, _P]),
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

    def results(self):
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

    def set_profiling(self, on=True):
        self.lib.xavs2gpu_me_set_profiling(self.h, 1 if on else 0)

    def phase_ms(self):
        out = (ctypes.c_float * 4)()
        self._check(self.lib.xavs2gpu_me_phase_ms(self.h, out), "phase_ms")
        return list(out)

    def plan_stats(self):
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self.lib.xavs2gpu_me_plan_stats(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
        return a.value, b.value, c.value


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
