"""Recorded primitive calls of a real xavs2 encode (the config-0 oracle):
parsing and replay.  TEST INFRASTRUCTURE ONLY.

The records come from oracle/enc_record.c (format in oracle/enc_calls.h):
every sampled call of an entry of the reference's primitive table with its
scalar arguments, snapshots of the memory regions it reads (before the call)
and writes (after it), and its return value.  `replay` rebuilds each call's
buffers with the recorded strides, offsets and aliasing, calls a backend's
function for the same table entry, and compares every written region and the
return value with the recording.
"""
import ctypes
import struct

import numpy as np

KINDS = ["sad", "satd", "sa8d", "ssd", "sad_x3", "sad_x4", "sub_ps", "add_ps", "copy_sp", "copy_ps", "copy_ss",
         "copy_pp", "avg", "mad", "ssd_block", "average", "luma_hor", "luma_ver", "luma_ext", "luma_ver_x3",
         "luma_hor_x3", "luma_ext_x3", "luma_block_hor", "luma_block_ver", "luma_block_ext", "chroma_block_hor",
         "chroma_block_ver", "chroma_block_ext", "intra", "dct", "idct", "dct_half", "t4_2nd", "inv_t4_2nd",
         "t_2nd", "inv_t_2nd", "abs_coeff", "add_sign", "quant", "dequant", "wquant", "deblock_luma",
         "deblock_chroma", "sao", "lowres"]
MAX_SLOTS = 33
MAGIC = 0x43455258
COUNT_MAGIC = 0x544E4358
# entries whose C type returns a value (int32)
RETURNS = {"sad", "satd", "sa8d", "ssd", "mad", "ssd_block", "add_sign", "quant", "wquant"}


class Buf:
    __slots__ = ("esize", "flags", "alias", "stride", "inr", "outr", "data_in", "data_out")


def parse(blob):
    """Records (kind, slot, call index, return value, arguments, byte span)
    and the per-entry call counts of a recording."""
    mv = memoryview(blob)
    pos = 0
    records = []
    counts = None
    while pos < len(mv):
        magic, = struct.unpack_from("<I", mv, pos)
        if magic == COUNT_MAGIC:
            nk, ns = struct.unpack_from("<II", mv, pos + 4)
            counts = np.frombuffer(mv[pos + 12:pos + 12 + 8 * nk * ns], "<i8").reshape(nk, ns).copy()
            pos += 12 + 8 * nk * ns
            continue
        if magic != MAGIC:
            raise ValueError("bad record at %d" % pos)
        start = pos
        kind, slot, idx, nargs, _, ret = struct.unpack_from("<HHIHHq", mv, pos + 4)
        pos += 24
        args = []
        for _ in range(nargs):
            t = chr(mv[pos])
            pos += 1
            if t != "b":
                v, = struct.unpack_from("<q", mv, pos)
                pos += 8
                args.append((t, v))
                continue
            b = Buf()
            b.esize, b.flags, b.alias, b.stride = struct.unpack_from("<BBhq", mv, pos)
            pos += 12
            reg = struct.unpack_from("<8i", mv, pos)
            pos += 32
            b.inr, b.outr = reg[:4], reg[4:]
            dt = {1: np.uint8, 2: np.int16, 4: np.int32}[b.esize]
            b.data_in = b.data_out = None
            for flag, r, name in ((1, b.inr, "data_in"), (2, b.outr, "data_out")):
                if b.flags & flag:
                    rows, cols = r[1] - r[0], r[3] - r[2]
                    n = rows * cols * b.esize
                    setattr(b, name, np.frombuffer(mv[pos:pos + n], dt).reshape(rows, cols))
                    pos += n
            args.append(("b", b))
        records.append((KINDS[kind], slot, idx, ret, args, (start, pos)))
    return records, counts


def _span(b):
    """Element offsets (lo, hi) relative to the pointer that the regions cover."""
    lo, hi = None, None
    for flag, r in ((1, b.inr), (2, b.outr)):
        if r[1] > r[0] and r[3] > r[2]:
            a = r[0] * b.stride + r[2]
            z = (r[1] - 1) * b.stride + r[3]
            lo = a if lo is None else min(lo, a)
            hi = z if hi is None else max(hi, z)
    return lo, hi


def _place(arr, base, b, r, data):
    for y in range(r[1] - r[0]):
        o = base + (r[0] + y) * b.stride + r[2]
        arr[o:o + (r[3] - r[2])] = data[y]


def _read(arr, base, b, r):
    rows = [arr[base + (r[0] + y) * b.stride + r[2]:base + (r[0] + y) * b.stride + r[3]] for y in range(r[1] - r[0])]
    return np.stack(rows) if rows else np.zeros((0, r[3] - r[2]), arr.dtype)


def replay_call(fn_addr, kind, ret, args, fill=0):
    """Calls fn_addr with the recorded arguments; returns a list of
    mismatch descriptions (empty when every output and the return value
    equal the recording)."""
    # one host buffer per distinct address, covering the regions of every
    # argument that shares it (in-place transforms, recon written over its
    # prediction), with 32 spare elements on either side
    spans = {}
    for i, (t, v) in enumerate(args):
        if t == "b":
            root = i if v.alias < 0 else v.alias
            lo, hi = _span(v)
            if lo is None:
                lo, hi = 0, 1
            a, z = spans.get(root, (lo, hi))
            spans[root] = (min(a, lo), max(z, hi))
    bufs = {}       # arg index -> (array, base element, Buf)
    for i, (t, v) in enumerate(args):
        if t != "b":
            continue
        b = v
        dt = {1: np.uint8, 2: np.int16, 4: np.int32}[b.esize]
        if b.alias >= 0:
            arr, base, _ = bufs[b.alias]
        else:
            lo, hi = spans[i]
            arr = np.full(hi - lo + 64, fill, dt)
            base = -lo + 32
        if b.data_in is not None:
            _place(arr, base, b, b.inr, b.data_in)
        bufs[i] = (arr, base, b)
    cargs, ctypes_list, keep = [], [], []
    i = 0
    while i < len(args):
        t, v = args[i]
        if t == "i":
            cargs.append(ctypes.c_int32(v)); ctypes_list.append(ctypes.c_int32)
        elif t == "p":
            cargs.append(ctypes.c_int64(v)); ctypes_list.append(ctypes.c_int64)
        elif t == "a":
            ptrs = (ctypes.c_void_p * v)()
            for k in range(v):
                arr, base, b = bufs[i + 1 + k]
                ptrs[k] = arr.ctypes.data + base * arr.itemsize
            keep.append(ptrs)
            cargs.append(ctypes.cast(ptrs, ctypes.c_void_p)); ctypes_list.append(ctypes.c_void_p)
            i += 1 + v
            continue
        else:
            arr, base, b = bufs[i]
            cargs.append(ctypes.c_void_p(arr.ctypes.data + base * arr.itemsize)); ctypes_list.append(ctypes.c_void_p)
        i += 1
    restype = ctypes.c_int32 if kind in RETURNS else None
    f = ctypes.CFUNCTYPE(restype, *ctypes_list)(fn_addr)
    got = f(*cargs)
    bad = []
    if restype is not None and int(got) != int(np.int32(ret)):
        bad.append("return %d, recorded %d" % (got, ret))
    for i, (arr, base, b) in bufs.items():
        if b.data_out is None:
            continue
        out = _read(arr, base, b, b.outr)
        if not np.array_equal(out, b.data_out):
            d = np.argwhere(out != b.data_out)[0]
            bad.append("arg %d at %s: %d, recorded %d" % (i, tuple(d), out[tuple(d)], b.data_out[tuple(d)]))
    return bad


def replay(records, entry, fill=0):
    """Replays every record through entry(kind, slot) -> function address
    (None: no such entry in the backend, counted as skipped).  Returns
    (replayed per kind, skipped per kind, mismatch list)."""
    done, skipped, bad = {}, {}, []
    for kind, slot, idx, ret, args, _ in records:
        addr = entry(kind, slot)
        if not addr:
            skipped[kind] = skipped.get(kind, 0) + 1
            continue
        for msg in replay_call(addr, kind, ret, args, fill):
            bad.append("%s[%d] call %d: %s" % (kind, slot, idx, msg))
        done[kind] = done.get(kind, 0) + 1
    return done, skipped, bad


def oracle_entry(olib):
    """Backend: the oracle's table (xo_tab_entry)."""
    olib.xo_tab_entry.restype = ctypes.c_void_p
    olib.xo_tab_entry.argtypes = [ctypes.c_int, ctypes.c_int]
    return lambda kind, slot: olib.xo_tab_entry(KINDS.index(kind), slot)


def gpu_entry(lib):
    """Backend: the GPU library's drop-in tables, filled by its table
    initialisers exactly as an encoder installs them."""
    n_pix = 13 * 25 + 2 + 4 + 2
    pixf = (ctypes.c_void_p * n_pix)()
    lib.xavs2gpu_pixel_init(0, pixf)
    lib.xavs2gpu_mad_init(0, ctypes.byref(pixf, (13 * 25 + 2) * ctypes.sizeof(ctypes.c_void_p)))
    dctf = (ctypes.c_void_p * (3 * 25 + 9))()
    lib.xavs2gpu_dct_init(0, dctf)
    lib.xavs2gpu_quant_init(0, dctf)
    intraf = (ctypes.c_void_p * 33)()
    lib.xavs2gpu_intra_pred_init(0, intraf)
    dbk = (ctypes.c_void_p * 4)()
    lib.xavs2gpu_deblock_init(0, dbk)
    sao = (ctypes.c_void_p * 1)()
    lib.xavs2gpu_sao_init(0, sao)

    def sym(name):
        return ctypes.cast(getattr(lib, name), ctypes.c_void_p).value

    singles = {"luma_hor": "xavs2gpu_intpl_luma_hor", "luma_ver": "xavs2gpu_intpl_luma_ver",
               "luma_ext": "xavs2gpu_intpl_luma_ext", "luma_ver_x3": "xavs2gpu_intpl_luma_ver_x3",
               "luma_hor_x3": "xavs2gpu_intpl_luma_hor_x3", "luma_ext_x3": "xavs2gpu_intpl_luma_ext_x3",
               "luma_block_hor": "xavs2gpu_intpl_luma_block_hor", "luma_block_ver": "xavs2gpu_intpl_luma_block_ver",
               "luma_block_ext": "xavs2gpu_intpl_luma_block_ext",
               "chroma_block_hor": "xavs2gpu_intpl_chroma_block_hor",
               "chroma_block_ver": "xavs2gpu_intpl_chroma_block_ver",
               "chroma_block_ext": "xavs2gpu_intpl_chroma_block_ext", "lowres": "xavs2gpu_lowres_filter"}
    dct_single = ["t4_2nd", "inv_t4_2nd", "t_2nd", "inv_t_2nd", "abs_coeff", "add_sign", "quant", "dequant",
                  "wquant"]

    def entry(kind, slot):
        k = KINDS.index(kind)
        if k <= KINDS.index("avg"):
            return pixf[k * 25 + slot]
        if kind == "mad":
            return pixf[13 * 25 + 2 + slot]
        if kind == "ssd_block":
            return pixf[13 * 25 + 6]
        if kind == "average":
            return pixf[13 * 25 + 7]
        if kind in singles:
            return sym(singles[kind])
        if kind == "intra":
            return intraf[slot]
        if kind in ("dct", "idct", "dct_half"):
            return dctf[("dct", "idct", "dct_half").index(kind) * 25 + slot]
        if kind in dct_single:
            return dctf[75 + dct_single.index(kind)]
        if kind == "deblock_luma":
            return dbk[slot]
        if kind == "deblock_chroma":
            return dbk[2 + slot]
        if kind == "sao":
            return sao[0]
        return None

    return entry


def select(blob, keep_per_entry=None):
    """A recording reduced to at most keep_per_entry records per entry (the
    first half and the last half of its sampled calls), with its call-count
    trailer; all records when keep_per_entry is None."""
    records, counts = parse(blob)
    by_entry = {}
    for r in records:
        by_entry.setdefault((r[0], r[1]), []).append(r)
    keep = set()
    for rs in by_entry.values():
        if keep_per_entry is None or len(rs) <= keep_per_entry:
            keep.update(r[5] for r in rs)
        else:
            half = keep_per_entry // 2
            keep.update(r[5] for r in rs[:half] + rs[len(rs) - (keep_per_entry - half):])
    out = b"".join(bytes(blob[a:b]) for r in records for (a, b) in [r[5]] if r[5] in keep)
    nk, ns = counts.shape
    return out + struct.pack("<III", COUNT_MAGIC, nk, ns) + counts.astype("<i8").tobytes()
