"""CPU checkers for the xavs2 hot path -- TEST INFRASTRUCTURE ONLY.

``liboracle.so`` is this project's C restatement of the reference algorithms
(``xavs2_oracle.c``); ``_ref/libxavs2ref.so`` is the reference's own C
primitives compiled from its source files (only where the reference tree is
present).  Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s
CPU-baseline leg may import this package; the GPU product never does.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libxavs2ref.so")


def _recipe_ref_src():
    """The reference source directory the build recipe (Makefile, REF_SRC)
    names; XAVS2_REF_SRC overrides it."""
    with open(os.path.join(HERE, "Makefile")) as f:
        for line in f:
            if line.startswith("REF_SRC") and "?=" in line:
                return line.split("?=", 1)[1].strip()
    return ""


REF_SRC = os.environ.get("XAVS2_REF_SRC") or _recipe_ref_src()

# LumaPU order (pixel.h:50-65)
PU_W = [4, 8, 16, 32, 64, 8, 4, 16, 8, 32, 16, 64, 32, 16, 12, 16, 4, 32, 24, 32, 8, 64, 48, 64, 16]
PU_H = [4, 8, 16, 32, 64, 4, 8, 8, 16, 16, 32, 32, 64, 12, 16, 4, 16, 24, 32, 8, 32, 48, 64, 16, 64]
TU_PARTS = [0, 1, 2, 3, 4, 15, 16, 19, 20, 23, 24]


class MeParams(ctypes.Structure):
    _fields_ = [("search_range", ctypes.c_int32), ("lambda_factor", ctypes.c_int32),
                ("use_hadamard", ctypes.c_int32), ("fractional_me", ctypes.c_int32),
                ("fast_sub_me", ctypes.c_int32), ("enable_pmvr", ctypes.c_int32)]


class Pu(ctypes.Structure):
    _fields_ = [("x", ctypes.c_int16), ("y", ctypes.c_int16), ("part", ctypes.c_uint8),
                ("ref", ctypes.c_uint8), ("mvp_x", ctypes.c_int16), ("mvp_y", ctypes.c_int16),
                ("min_x", ctypes.c_int16), ("min_y", ctypes.c_int16),
                ("max_x", ctypes.c_int16), ("max_y", ctypes.c_int16)]


class MeResult(ctypes.Structure):
    _fields_ = [("bmv_x", ctypes.c_int16), ("bmv_y", ctypes.c_int16), ("bcost", ctypes.c_int32),
                ("mvcost", ctypes.c_int32), ("imv_x", ctypes.c_int16), ("imv_y", ctypes.c_int16),
                ("icost", ctypes.c_int32)]


PU_DTYPE = np.dtype([("x", "<i2"), ("y", "<i2"), ("part", "u1"), ("ref", "u1"),
                     ("mvp_x", "<i2"), ("mvp_y", "<i2"), ("min_x", "<i2"), ("min_y", "<i2"),
                     ("max_x", "<i2"), ("max_y", "<i2")])
RESULT_DTYPE = np.dtype([("bmv_x", "<i2"), ("bmv_y", "<i2"), ("bcost", "<i4"), ("mvcost", "<i4"),
                         ("imv_x", "<i2"), ("imv_y", "<i2"), ("icost", "<i4")])
assert PU_DTYPE.itemsize == ctypes.sizeof(Pu) == 18
assert RESULT_DTYPE.itemsize == ctypes.sizeof(MeResult) == 20


def build(with_ref=None):
    """Compile liboracle.so (and the reference build when its sources exist)."""
    targets = ["all"]
    if with_ref is None:
        with_ref = os.path.isdir(REF_SRC)
    if with_ref:
        targets.append("ref")
    subprocess.run(["make", "-s", "-j4", "-C", HERE, "REF_SRC=" + REF_SRC] + targets, check=True)


_oracle = None
_ref = None

_P = ctypes.c_void_p
_I = ctypes.c_int
_S = ctypes.c_ssize_t

# argument types of the C entry points (pointers are passed as c_void_p)
_ORACLE_SIGS = {
    "xo_sad": (_I, [_I, _P, _S, _P, _S]), "xo_satd": (_I, [_I, _P, _S, _P, _S]),
    "xo_sa8d": (_I, [_I, _P, _S, _P, _S]), "xo_ssd": (_I, [_I, _P, _S, _P, _S]),
    "xo_sad_x3": (None, [_I, _P, _P, _P, _P, _S, _P]),
    "xo_sad_x4": (None, [_I, _P, _P, _P, _P, _P, _S, _P]),
    "xo_avg": (None, [_I, _P, _S, _P, _S, _P, _S]),
    "xo_sub_ps": (None, [_I, _P, _S, _P, _P, _S, _S]),
    "xo_add_ps": (None, [_I, _P, _S, _P, _P, _S, _S]),
    "xo_copy_pp": (None, [_I, _P, _S, _P, _S]), "xo_copy_ps": (None, [_I, _P, _S, _P, _S]),
    "xo_copy_sp": (None, [_I, _P, _S, _P, _S]), "xo_copy_ss": (None, [_I, _P, _S, _P, _S]),
    "xo_ssd_block": (_I, [_P, _S, _P, _S, _I, _I]),
    "xo_average": (None, [_P, _I, _P, _I, _P, _I, _I, _I]),
    "xo_mad": (_I, [_P, _I, _I]),
    "xo_intpl_luma_hor": (None, [_P, _I, _P, _I, _P, _I, _I, _I, _P]),
    "xo_intpl_luma_ver": (None, [_P, _I, _P, _I, _I, _I, _P]),
    "xo_intpl_luma_ext": (None, [_P, _I, _P, _I, _I, _I, _P]),
    "xo_intpl_luma_block_hor": (None, [_P, _I, _P, _I, _I, _I, _P]),
    "xo_intpl_luma_block_ver": (None, [_P, _I, _P, _I, _I, _I, _P]),
    "xo_intpl_luma_block_ext": (None, [_P, _I, _P, _I, _I, _I, _P, _P]),
    "xo_intpl_chroma_block_hor": (None, [_P, _I, _P, _I, _I, _I, _P]),
    "xo_intpl_chroma_block_ver": (None, [_P, _I, _P, _I, _I, _I, _P]),
    "xo_intpl_chroma_block_ext": (None, [_P, _I, _P, _I, _I, _I, _P, _P]),
    "xo_interpolate_frame": (None, [_P, _P, _I, _I, _I, _I, _I]),
    "xo_expand_border": (None, [_P, _I, _I, _I, _I]),
    "xo_dct": (None, [_I, _P, _P, _I]), "xo_idct": (None, [_I, _P, _P, _I]),
    "xo_dct_half": (None, [_I, _P, _P, _I]),
    "xo_transform_4x4_2nd": (None, [_P, _I]), "xo_inv_transform_4x4_2nd": (None, [_P, _I]),
    "xo_transform_2nd": (None, [_P, _I, _I, _I, _I]),
    "xo_inv_transform_2nd": (None, [_P, _I, _I, _I, _I]),
    "xo_quant": (_I, [_P, _I, _I, _I, _I]), "xo_wquant": (_I, [_P, _I, _I, _I, _I, _P]),
    "xo_dequant": (None, [_P, _I, _I, _I]), "xo_abs_coeff": (None, [_P, _P, _I]),
    "xo_add_sign": (_I, [_P, _P, _I]),
    "xo_tq_chain": (_I, [_I, _P, _P, _I, _I, _I]),
    "xo_tq_batch": (None, [_P, _I, _P, _P, _P, _P, _I]),
    "xo_me_search": (_I, [_P, _P, _P, _S, _P, _S, _P]),
    "xo_me_search_list": (None, [_P, _P, _I, _P, _S, _P, _S, _P, _I]),
    "xo_pu_set_limits": (None, [_P, _I, _I, _I, _I]),
    "xo_intra_pred": (None, [_I, _P, _P, _I, _I, _I, _I]),
    "xo_intra_fill_edge": (None, [_P, _I, _I, _I, _I, _I, _I, _P]),
    "xo_intra_fill_edges": (None, [_P, _I, _P, _I, _I, _I, _P, ctypes.c_int64]),
    "xo_intra_mode_costs": (None, [_P, _P, _I, _I, _I, _I, _P, ctypes.c_double, _I, _P]),
    "xo_intra_candidates": (_I, [_P, _I, _I, _I, _I, _P, _P, _P]),
    "xo_intra_rmd_batch": (None, [_P, _I, _P, _P, _I, ctypes.c_double, _I, _I, _I, _I, _P, _I]),
    "xo_deblock_luma": (None, [_I, _P, _I, _I, _I, _P]),
    "xo_deblock_chroma": (None, [_I, _P, _P, _I, _I, _I, _P]),
    "xo_deblock_picture": (None, [_P, _I, _P, _P, _I, _I, _I, _P, _I, _I]),
    "xo_sao_block": (None, [_P, _I, _P, _I, _I, _I, _P, _P]),
    "xo_sao_picture": (None, [_P, _P, _I, _I, _I, _I, _I, _P]),
    "xo_lowres_filter": (None, [_P, _I, _P, _I, _I, _I]),
    "xo_lookahead_picture": (None, [_P, _I, _I, _I, _P, _I, _P, _P, _P]),
    "xo_skip_costs": (None, [_P, _I, _P, _I, _I, _I, _I, _P, _I, ctypes.c_double, _I, _P, _P, _P]),
}
_REF_SIGS = {
    "xr_cmp": (_I, [_I, _I, _P, _S, _P, _S]),
    "xr_sad_x3": (None, [_I, _P, _P, _P, _P, _S, _P]),
    "xr_sad_x4": (None, [_I, _P, _P, _P, _P, _P, _S, _P]),
    "xr_avg": (None, [_I, _P, _S, _P, _S, _P, _S]),
    "xr_sub_ps": (None, [_I, _P, _S, _P, _P, _S, _S]),
    "xr_add_ps": (None, [_I, _P, _S, _P, _P, _S, _S]),
    "xr_copy": (None, [_I, _I, _P, _S, _P, _S]),
    "xr_ssd_block": (_I, [_P, _S, _P, _S, _I, _I]),
    "xr_average": (None, [_P, _I, _P, _I, _P, _I, _I, _I]),
    "xr_mad": (_I, [_P, _I, _I]),
    "xr_intpl_luma_hor": (None, [_P, _I, _P, _I, _P, _I, _I, _I, _P]),
    "xr_intpl_luma_ver": (None, [_P, _I, _P, _I, _I, _I, _P]),
    "xr_intpl_luma_ext": (None, [_P, _I, _P, _I, _I, _I, _P]),
    "xr_intpl_block": (None, [_I, _P, _I, _P, _I, _I, _I, _P, _P]),
    "xr_interpolate_frame": (None, [_P, _I, _I, _I, _I, _I]),
    "xr_dct": (None, [_I, _I, _P, _P, _I]), "xr_2nd": (None, [_I, _P, _I, _I, _I, _I]),
    "xr_quant": (_I, [_P, _I, _I, _I, _I]), "xr_wquant": (_I, [_P, _I, _I, _I, _I, _P]),
    "xr_dequant": (None, [_P, _I, _I, _I]), "xr_abs_coeff": (None, [_P, _P, _I]),
    "xr_add_sign": (_I, [_P, _P, _I]),
    "xr_me_search": (_I, [_P, _P, _P, _S, _P, _I, _P]),
    "xr_me_search_list": (None, [_P, _P, _I, _P, _S, _P, _I, _P, _I]),
    "xr_intra_pred": (None, [_I, _P, _P, _I, _I, _I, _I]),
    "xr_intra_fill_edge": (None, [_I, _P, _I, _P, _P, ctypes.c_uint32, _I, _I]),
    "xr_deblock_luma": (None, [_I, _P, _I, _I, _I, _P]),
    "xr_deblock_chroma": (None, [_I, _P, _P, _I, _I, _I, _P]),
    "xr_sao_block": (None, [_P, _I, _P, _I, _I, _I, _P, _P]),
    "xr_lowres_filter": (None, [_P, _I, _P, _I, _I, _I]),
}


def _apply_sigs(l, sigs):
    for name, (res, args) in sigs.items():
        f = getattr(l, name)
        f.restype = res
        f.argtypes = args


def lib():
    global _oracle
    if _oracle is None:
        if not os.path.exists(ORACLE_SO):
            build(with_ref=False)
        _oracle = ctypes.CDLL(ORACLE_SO)
        _apply_sigs(_oracle, _ORACLE_SIGS)
        _oracle.xo_luma_filter.restype = ctypes.POINTER(ctypes.c_int8)
        _oracle.xo_chroma_filter.restype = ctypes.POINTER(ctypes.c_int8)
    return _oracle


def ref_lib():
    """The reference build, or None where it cannot be built."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_SO):
            if not os.path.isdir(REF_SRC):
                return None
            build(with_ref=True)
        _ref = ctypes.CDLL(REF_SO)
        _apply_sigs(_ref, _REF_SIGS)
        _ref.xr_init()
    return _ref


def ptr(a, off=0):
    """Pointer to element `off` (flat index) of a contiguous numpy array."""
    return ctypes.c_void_p(a.ctypes.data + off * a.itemsize)


def lambda_factor(qp, factor=0.68):
    """i_lambda_factor for a P frame without GOP factors (encoder.c:232-341):
    lambda = 2^((qp-11)/4) * 0.85 * 0.8, factor = round(65536 * sqrt(lambda))."""
    lam = 2.0 ** ((qp - 11) / 4.0) * factor
    return int(65536.0 * np.sqrt(lam) + 0.5)


def padded_plane(img, pad):
    """Copy an HxW uint8 image into a buffer with `pad` replicated pixels on
    each side; returns (buffer, offset of pixel (0,0), stride)."""
    h, w = img.shape
    buf = np.pad(img, pad, mode="edge").astype(np.uint8)
    stride = w + 2 * pad
    return np.ascontiguousarray(buf).reshape(-1), pad * stride + pad, stride


def interpolate_frame(lib_, img, pad=80, mode=2, ref=False, lcu_level=6):
    """Frame sub-pel planes via the oracle (ref=False) or the reference's own
    row-wise interpolation (ref=True).  Returns a (16, H+2p, W+2p) array."""
    h, w = img.shape
    src, off, stride = padded_plane(img, pad)
    planes = np.zeros((16, src.size), np.uint8)
    planes[0] = src
    arr = (ctypes.c_void_p * 16)()
    for k in range(16):
        arr[k] = ptr(planes[k], off).value
    if ref:
        lib_.xr_interpolate_frame(arr, stride, w, h, lcu_level, mode)
    else:
        lib_.xo_interpolate_frame(arr, ptr(planes[0], off), stride, w, h, pad, mode)
    return planes.reshape(16, h + 2 * pad, w + 2 * pad)


# ---- the full-picture chain's inter candidates (rdo.c:1333-1477) -----------
CAND_DTYPE = np.dtype([("cu", "<i4"), ("mode", "i1"), ("split_type", "i1"), ("pad_", "<i2"),
                       ("res_offset", "<i8"), ("coef_offset", "<i8")])
# partition PUs of a CU after its 2Nx2N PU, in quarters of the CU side:
# (dx, dy, w, h); mode m >= 1 owns PUs 2m - 1 and 2m
_CU_PARTS = [(0, 0, 4, 4), (0, 0, 4, 2), (0, 2, 4, 2), (0, 0, 2, 4), (2, 0, 2, 4), (0, 0, 4, 1), (0, 1, 4, 3),
             (0, 0, 4, 3), (0, 3, 4, 1), (0, 0, 1, 4), (1, 0, 3, 4), (0, 0, 3, 4), (3, 0, 1, 4)]


def _split_tus(S, split_type):
    """(x, y, w, h) of the four split TUs of an S x S CU: quarters (1),
    horizontal strips (2), vertical strips (3) (rdo.c:1419-1463)."""
    if split_type == 2:
        return [(0, t * S // 4, S, S // 4) for t in range(4)]
    if split_type == 3:
        return [(t * S // 4, 0, S // 4, S) for t in range(4)]
    h = S // 2
    return [((t & 1) * h, (t >> 1) * h, h, h) for t in range(4)]


def chain_candidate(olib, cur, planes, res, cu, mode, split_type, qp):
    """One inter candidate of a CU as the chain computes it: each PU of the
    mode predicted from the reference with its smallest search cost (first
    on ties) at that search's MV from the sub-pel planes (planes[r] =
    interpolate_frame(...) of reference r, margin 80), the residual, the TU
    chain (xo_tq_chain: dct -> quant -> dequant -> idct, i_level from the TU
    shape) of the one CU-sized TU and of the four split TUs.  Returns a dict:
    cost (sum of the PUs' search costs), levels / nnz / rres (reconstructed
    residual, S x S) / dist (SSD of clip(pred + rres)) per variant (0 one TU,
    1 split)."""
    x, y, S = int(cu["x"]), int(cu["y"]), int(cu["size"])
    ks = [0] if mode == 0 else [2 * mode - 1, 2 * mode]
    pred = np.zeros((S, S), np.int32)
    cost = 0
    for k in ks:
        best = None
        for r in range(len(planes)):
            q = res[int(cu["pu"][r]) + k]
            if best is None or q["bcost"] < best[0]:
                best = (int(q["bcost"]), r, int(q["bmv_x"]), int(q["bmv_y"]))
        cost += best[0]
        _, r, mvx, mvy = best
        dx, dy, w, h = (v * S // 4 for v in _CU_PARTS[k])
        pl = planes[r][((mvy & 3) << 2) + (mvx & 3)]
        oy, ox = 80 + y + dy + (mvy >> 2), 80 + x + dx + (mvx >> 2)
        pred[dy:dy + h, dx:dx + w] = pl[oy:oy + h, ox:ox + w]
    src = cur[y:y + S, x:x + S].astype(np.int32)
    resid = (src - pred).astype(np.int16)
    out = {"cost": cost, "levels": [], "nnz": [], "rres": [], "dist": []}
    for variant in (0, 1):
        tus = [(0, 0, S, S)] if variant == 0 else _split_tus(S, split_type)
        rres = np.zeros((S, S), np.int16)
        levels, nnzs = [], []
        for (tx, ty, tw, th) in tus:
            blk = np.ascontiguousarray(resid[ty:ty + th, tx:tx + tw]).reshape(-1).copy()
            coef = np.zeros(tw * th, np.int16)
            part = PU_W.index(tw) if tw == th else [k for k in range(25) if PU_W[k] == tw and PU_H[k] == th][0]
            nnzs.append(olib.xo_tq_chain(part, ptr(blk), ptr(coef), qp, 0, 0))
            nc = tw * th // 4 if (tw == 64 or th == 64) else tw * th
            levels.append(coef[:nc])
            rres[ty:ty + th, tx:tx + tw] = blk.reshape(th, tw)
        rec = np.clip(pred + rres, 0, 255)
        out["levels"].append(np.concatenate(levels))
        out["nnz"].append(nnzs)
        out["rres"].append(rres)
        out["dist"].append(int(((src - rec) ** 2).sum()))
    out["pred"] = pred
    return out


def chain_sample_check(olib, out, cur, refs, pus, cus, res_gpu, prm_tuple, qp, cu_idx, threads=1):
    """Checks a chain's (or a served picture's) outputs for the CUs cu_idx
    against the oracle: the search of every PU of those CUs (oracle's
    xo_me_search_list on the same pictures), every candidate of those CUs
    (chain_candidate with the oracle's search results) and each CU's choice
    and reconstructed block.  `out` holds the downloaded outputs (cands,
    nnz, coef, rres, cost, dist, choice, recon).  Returns (PU searches
    checked, candidates checked, list of mismatch descriptions)."""
    h, w = cur.shape
    stride = w + 160
    cands = out["cands"]
    first = np.searchsorted(cands["cu"], cu_idx)
    last = np.searchsorted(cands["cu"], cu_idx, side="right")
    sel = []
    for c, a, b in zip(cu_idx, first, last):
        nk = 1 if b - a == 1 else (5 if int(cus[c]["size"]) == 8 else 13)
        for r in range(len(refs)):
            sel.extend(range(int(cus[c]["pu"][r]), int(cus[c]["pu"][r]) + nk))
    sel = np.array(sorted(set(sel)), np.int64)
    flats = [np.ascontiguousarray(interpolate_frame(olib, r, mode=2).reshape(16, -1)) for r in refs]
    frefs = (ctypes.c_void_p * (16 * len(refs)))(*[ptr(f[k], 80 * stride + 80).value for f in flats
                                                   for k in range(16)])
    sub = np.ascontiguousarray(pus[sel])
    got = np.zeros(len(sel), RESULT_DTYPE)
    olib.xo_me_search_list(ctypes.byref(MeParams(*prm_tuple)), ptr(sub), len(sub), ptr(cur), w, frefs, stride,
                           ptr(got), threads)
    bad = []
    res = np.zeros(len(pus), RESULT_DTYPE)
    res[sel] = got
    diff = np.flatnonzero((got.view(np.uint8).reshape(len(sel), -1) !=
                           np.ascontiguousarray(res_gpu[sel]).view(np.uint8).reshape(len(sel), -1)).any(axis=1))
    bad += ["search of PU %d" % sel[i] for i in diff[:5]]
    planes = [f.reshape(16, h + 160, w + 160) for f in flats]
    n_cands = 0
    for c, a, b in zip(cu_idx, first, last):
        exp = {}
        for i in range(a, b):
            cd = cands[i]
            e = chain_candidate(olib, cur, planes, res, cus[c], int(cd["mode"]), int(cd["split_type"]), qp)
            exp[i] = e
            n_cands += 1
            S = int(cus[c]["size"])
            ro, co = int(cd["res_offset"]), int(cd["coef_offset"])
            n0, n1 = len(e["levels"][0]), len(e["levels"][1])
            ok = (int(out["cost"][i]) == e["cost"] and list(out["dist"][i]) == e["dist"] and
                  list(out["nnz"][5 * i:5 * i + 5]) == [e["nnz"][0][0]] + e["nnz"][1] and
                  np.array_equal(out["rres"][ro:ro + S * S].reshape(S, S), e["rres"][0]) and
                  np.array_equal(out["coef"][co:co + n0], e["levels"][0]) and
                  np.array_equal(out["coef"][co + n0:co + n0 + n1], e["levels"][1]))
            if not ok:
                bad.append("candidate %d (CU %d mode %d)" % (i, c, int(cd["mode"])))
        best = min(range(a, b), key=lambda k: (exp[k]["cost"], k))
        split = int(exp[best]["dist"][1] < exp[best]["dist"][0])
        ch = out["choice"][c]
        x, y, S = int(cus[c]["x"]), int(cus[c]["y"]), int(cus[c]["size"])
        rec = np.clip(exp[best]["pred"] + exp[best]["rres"][split], 0, 255)
        if (int(ch["cand"]), int(ch["split"])) != (best, split) or not np.array_equal(out["recon"][y:y + S, x:x + S], rec):
            bad.append("choice of CU %d" % c)
    return len(sel), n_cands, bad
