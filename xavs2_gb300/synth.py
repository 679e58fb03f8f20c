"""Seeded synthetic video content for the benchmarks and tests.

The reference's sample configurations name an external test sequence that
is not available; these generators stand in for it:

* base picture: uniform noise blurred with a Gaussian (sigma 3) and rescaled
  to [16, 235];
* next picture: the previous one displaced by quarter-pel motion (AVS2
  8-tap luma filter for the fractional part), plus Gaussian noise (sigma 2),
  clipped to [0, 255].  Motion is either one global translation or one of
  several motions chosen per 8x8 block by a seeded label map.
"""
import numpy as np

_TAPS = np.array([[0, 0, 0, 64, 0, 0, 0, 0],
                  [-1, 4, -10, 57, 19, -7, 3, -1],
                  [-1, 4, -11, 40, 40, -11, 4, -1],
                  [-1, 3, -7, 19, 57, -10, 4, -1]], np.float64)


def base_picture(rng, width, height, sigma=3.0):
    from scipy.ndimage import gaussian_filter
    noise = rng.integers(0, 256, (height, width)).astype(np.float64)
    blur = gaussian_filter(noise, sigma, mode="reflect")
    lo, hi = blur.min(), blur.max()
    return np.round(16 + (blur - lo) * (219.0 / max(hi - lo, 1e-9))).astype(np.uint8)


def shift_qpel(img, mvx, mvy):
    """img displaced by (mvx, mvy) quarter-pels: out(x, y) = img(x + mv/4)."""
    h, w = img.shape
    ix, fx = mvx >> 2, mvx & 3
    iy, fy = mvy >> 2, mvy & 3
    pad = 4 + max(abs(ix), abs(iy))
    p = np.pad(img.astype(np.float64), pad, mode="edge")
    ys = np.arange(h) + pad + iy
    xs = np.arange(w) + pad + ix
    rows = p[ys[0] - 3:ys[-1] + 5]
    # horizontal
    hor = sum(_TAPS[fx][k] * rows[:, xs[0] - 3 + k:xs[-1] - 3 + k + 1] for k in range(8)) / 64.0
    out = sum(_TAPS[fy][k] * hor[k:k + h] for k in range(8)) / 64.0
    return np.clip(np.round(out), 0, 255)


def next_picture(rng, prev, n_motions=1, max_px=8, block=8, noise=2.0):
    h, w = prev.shape
    mvs = rng.integers(-max_px * 4, max_px * 4 + 1, (n_motions, 2))
    if n_motions == 1:
        out = shift_qpel(prev, int(mvs[0, 0]), int(mvs[0, 1]))
    else:
        labels = rng.integers(0, n_motions, ((h + block - 1) // block, (w + block - 1) // block))
        lab = np.kron(labels, np.ones((block, block), np.int64))[:h, :w]
        out = np.zeros((h, w))
        for m in range(n_motions):
            sel = lab == m
            if sel.any():
                out[sel] = shift_qpel(prev, int(mvs[m, 0]), int(mvs[m, 1]))[sel]
    out = out + rng.normal(0.0, noise, (h, w))
    return np.clip(np.round(out), 0, 255).astype(np.uint8)


_CTAPS = np.array([[0, 64, 0, 0], [-4, 62, 6, 0], [-6, 56, 15, -1], [-5, 47, 25, -3],
                   [-4, 36, 36, -4], [-3, 25, 47, -5], [-1, 15, 56, -6], [0, 6, 62, -4]], np.float64)


def shift_eighth_chroma(img, mvx, mvy):
    """A chroma plane displaced by (mvx, mvy) eighth-pels with the AVS2
    4-tap chroma filter (the luma motion in quarter-pels at half size)."""
    h, w = img.shape
    ix, fx = mvx >> 3, mvx & 7
    iy, fy = mvy >> 3, mvy & 7
    pad = 2 + max(abs(ix), abs(iy))
    p = np.pad(img.astype(np.float64), pad, mode="edge")
    ys = np.arange(h) + pad + iy
    xs = np.arange(w) + pad + ix
    rows = p[ys[0] - 1:ys[-1] + 3]
    hor = sum(_CTAPS[fx][k] * rows[:, xs[0] - 1 + k:xs[-1] - 1 + k + 1] for k in range(4)) / 64.0
    out = sum(_CTAPS[fy][k] * hor[k:k + h] for k in range(4)) / 64.0
    return np.clip(np.round(out), 0, 255)


def config0_sequence(n=8, width=416, height=240, seed=0, max_px=8, noise=2.0):
    """The plain-encoder sequence: n 4:2:0 pictures (Y, U, V).  Picture 0 is
    blurred noise rescaled to [16, 235] (chroma likewise at half size); each
    later picture is the previous one moved by one translation U[-8, 8] px
    per axis in quarter-pel steps (AVS2 8-tap luma, 4-tap chroma at the same
    displacement), plus Gaussian noise, clipped."""
    rng = np.random.default_rng(seed)
    y = base_picture(rng, width, height)
    u = base_picture(rng, width // 2, height // 2)
    v = base_picture(rng, width // 2, height // 2)
    seq = [(y, u, v)]
    for _ in range(n - 1):
        mvx, mvy = (int(m) for m in rng.integers(-max_px * 4, max_px * 4 + 1, 2))
        y = np.clip(np.round(shift_qpel(y, mvx, mvy) + rng.normal(0.0, noise, y.shape)), 0, 255).astype(np.uint8)
        u, v = (np.clip(np.round(shift_eighth_chroma(c, mvx, mvy) + rng.normal(0.0, noise, c.shape)), 0, 255)
                .astype(np.uint8) for c in (u, v))
        seq.append((y, u, v))
    return seq


def me_workload(seed=1, width=1920, height=1080, n_motions=16, max_px=32):
    """Current picture and two references (k-1, k-2) for the batched
    motion-search benchmark: 16 block-local motions U[-32, 32] px in
    quarter-pel steps."""
    rng = np.random.default_rng(seed)
    f0 = base_picture(rng, width, height)
    f1 = next_picture(rng, f0, n_motions, max_px)
    f2 = next_picture(rng, f1, n_motions, max_px)
    return f2, [f1, f0]


TQ_BLOCK_DTYPE = np.dtype([("offset", "<i8"), ("coef_offset", "<i8"), ("part", "<i4"), ("qp", "<i4"),
                           ("flags", "<i4"), ("pad_", "<i4")])


def tq_blocks(n, seed=3, parts=(0, 1, 2, 3, 4)):
    """Descriptors of the batched transform+quant workload: TU shape uniform
    over `parts` (LumaPU indices; default the squares 4..64), QP uniform in
    [22, 51], half of the 4x4 blocks through the intra 4x4 secondary
    transform (b_intra set with it), blocks packed back to back.  Returns
    (blocks, residual elements, level elements, per-block zero mask: 10 % of
    the blocks are all-zero)."""
    from . import PU_W, PU_H
    rng = np.random.default_rng(seed)
    part = rng.choice(np.asarray(parts), n)
    w, h = np.asarray(PU_W)[part], np.asarray(PU_H)[part]
    size = (w * h).astype(np.int64)
    ncoef = np.where((w == 64) | (h == 64), size // 4, size)
    blocks = np.zeros(n, TQ_BLOCK_DTYPE)
    blocks["part"] = part
    blocks["qp"] = rng.integers(22, 52, n)
    sec = (part == 0) & (rng.random(n) < 0.5)
    blocks["flags"] = np.where(sec, 3, 0)
    blocks["offset"] = np.cumsum(size) - size
    blocks["coef_offset"] = np.cumsum(ncoef) - ncoef
    zero = rng.random(n) < 0.1
    return blocks, int(size.sum()), int(ncoef.sum()), zero


def tq_residual(blocks, zero, total, seed=4, device="cpu"):
    """int16 residuals for `blocks` as a torch tensor on `device`: Laplacian
    (scale 12) by inverse CDF of a seeded uniform, rounded, clipped to
    [-255, 255]; blocks flagged in `zero` are all zero."""
    import torch
    from . import PU_W, PU_H
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    u = torch.rand(total, generator=g, device=device, dtype=torch.float32) - 0.5
    x = -12.0 * torch.sign(u) * torch.log1p(-2.0 * u.abs().clamp(max=0.4999999))
    res = x.round().clamp(-255, 255).to(torch.int16)
    part = blocks["part"]
    size = (np.asarray(PU_W)[part] * np.asarray(PU_H)[part]).astype(np.int64)
    keep = torch.from_numpy((~zero).astype(np.int16)).to(device)
    res *= torch.repeat_interleave(keep, torch.from_numpy(size).to(device), output_size=total)
    return res


def chain_pictures(n, width, height, seed=21, pan_px=12, n_motions=2, max_px=4):
    """Pictures for the full-picture chain: a base picture, then each picture
    = the previous one panned by `pan_px` pixels to the left plus
    `n_motions` block-local quarter-pel motions U[-max_px, max_px] and noise."""
    rng = np.random.default_rng(seed)
    frames = [base_picture(rng, width, height)]
    for _ in range(n - 1):
        panned = shift_qpel(frames[-1], 4 * pan_px, 0)
        frames.append(next_picture(rng, panned, n_motions, max_px))
    return frames


# ---- intra blocks --------------------------------------------------------------
INTRA_ENC_SHAPES = [(4, 4), (8, 8), (16, 16), (32, 32), (64, 64), (4, 16), (16, 4), (8, 32), (32, 8)]
INTRA_ALL_SHAPES = INTRA_ENC_SHAPES + [(16, 64), (64, 16)]
# modes for RDO per block level (a preset-5 row of the encoder's table:
# 4x4 .. 64x64) and the rough search's neighbour counts of that preset
INTRA_RDO_NUM = {2: 6, 3: 6, 4: 6, 5: 4, 6: 3}
INTRA_DIST2, INTRA_DIST1 = 4, 2


def _intra_partition(rng, x0, y0, size, out, all_shapes):
    """Quad-tree split of a CTU into CUs (64 .. 8), each predicted as one
    block, as four SDIP strips (32 / 16 CUs) or four 4x4 blocks (8x8 CUs)."""
    if size > 8 and rng.random() < 0.55:
        h = size // 2
        for dy in (0, h):
            for dx in (0, h):
                _intra_partition(rng, x0 + dx, y0 + dy, h, out, all_shapes)
        return
    r = rng.random()
    if size in (16, 32) and r < 0.3:
        q = size // 4
        if rng.random() < 0.5:
            out.extend((x0, y0 + i * q, size, q) for i in range(4))
        else:
            out.extend((x0 + i * q, y0, q, size) for i in range(4))
    elif size == 64 and all_shapes and r < 0.3:
        if rng.random() < 0.5:
            out.extend((x0, y0 + i * 16, 64, 16) for i in range(4))
        else:
            out.extend((x0 + i * 16, y0, 16, 64) for i in range(4))
    elif size == 8 and r < 0.3:
        out.extend((x0 + dx, y0 + dy, 4, 4) for dy in (0, 4) for dx in (0, 4))
    else:
        out.append((x0, y0, size, size))


def intra_edge_window(bw, bh):
    """Samples below / above the top-left edge sample that the predictors of
    a bw x bh block read (fill_reference_samples pads this far)."""
    return bh + (11 * bw) // 4 + 6, bw + (11 * bh) // 4 + 6


def intra_pack(rects, recon, rng, block_dtype):
    """Descriptors and packed edge samples for blocks (x0, y0, w, h) of a
    picture: top row / top-right from the reconstruction row above, left
    column / left-down from the column to the left, coordinates clamped into
    the picture; a missing side repeats the other one (128 when neither
    exists).  Each block's window is 16-byte aligned in `edges`."""
    height, width = recon.shape
    rects = np.asarray(rects, np.int64).reshape(-1, 4)
    n = len(rects)
    lo = np.array([intra_edge_window(int(w), int(h))[0] for _, _, w, h in rects], np.int64)
    hi = np.array([intra_edge_window(int(w), int(h))[1] for _, _, w, h in rects], np.int64)
    size = (lo + hi + 1 + 15) // 16 * 16
    start = np.cumsum(size) - size
    edges = np.full(int(size.sum()) if n else 0, 128, np.uint8)
    blocks = np.zeros(n, block_dtype)
    for (bw, bh) in sorted(set(map(tuple, rects[:, 2:].tolist()))):
        sel = np.nonzero((rects[:, 2] == bw) & (rects[:, 3] == bh))[0]
        if not len(sel):
            continue
        x0, y0 = rects[sel, 0][:, None], rects[sel, 1][:, None]
        L, H = intra_edge_window(bw, bh)
        top_ok, left_ok = y0 > 0, x0 > 0
        k = np.arange(1, H + 1)[None, :]
        j = np.arange(1, L + 1)[None, :]
        top = recon[np.maximum(y0 - 1, 0), np.clip(x0 + k - 1, 0, width - 1)]
        left = recon[np.clip(y0 + j - 1, 0, height - 1), np.maximum(x0 - 1, 0)]
        rep_l = recon[y0[:, 0], np.maximum(x0[:, 0] - 1, 0)][:, None]
        rep_t = recon[np.maximum(y0[:, 0] - 1, 0), x0[:, 0]][:, None]
        top = np.where(top_ok, top, np.where(left_ok, rep_l, 128))
        left = np.where(left_ok, left, np.where(top_ok, rep_t, 128))
        corner = np.where(top_ok[:, 0] & left_ok[:, 0], recon[np.maximum(y0[:, 0] - 1, 0), np.maximum(x0[:, 0] - 1, 0)],
                          np.where(top_ok[:, 0], rep_t[:, 0], np.where(left_ok[:, 0], rep_l[:, 0], 128)))
        ep = start[sel] + L
        edges[ep] = corner
        edges[ep[:, None] + k] = top
        edges[ep[:, None] - j] = left
        blocks["edge_offset"][sel] = ep
    blocks["fenc_offset"] = rects[:, 1] * width + rects[:, 0]
    blocks["width"], blocks["height"] = rects[:, 2], rects[:, 3]
    blocks["dc_avail"] = ((rects[:, 1] > 0).astype(np.int16) << 8) | (rects[:, 0] > 0)
    m0 = rng.integers(0, 33, n)
    m1 = rng.integers(0, 32, n)
    blocks["mpm"][:, 0] = m0
    blocks["mpm"][:, 1] = m1 + (m1 >= m0)
    level = np.log2(np.maximum(rects[:, 2], rects[:, 3])).astype(int)
    blocks["num_for_rdo"] = np.array([INTRA_RDO_NUM.get(v, 6) for v in range(7)])[level]
    return blocks, edges


def intra_blocks(rng, src, recon, all_shapes=False, block_dtype=None):
    """One partition of the picture (width, height multiples of 64) into
    intra blocks of every shape, with packed edges (see intra_pack)."""
    height, width = src.shape
    rects = []
    for y0 in range(0, height, 64):
        for x0 in range(0, width, 64):
            _intra_partition(rng, x0, y0, 64, rects, all_shapes)
    return intra_pack(rects, recon, rng, block_dtype)


def _zorder(ux, uy):
    r = np.zeros_like(ux)
    for b in range(5):
        r |= ((ux >> b) & 1) << (2 * b) | ((uy >> b) & 1) << (2 * b + 1)
    return r


def intra_neighbors(rects, width, height, lcu_size=64):
    """MD_I_* availability of blocks (x0, y0, w, h) of a one-slice picture as
    get_intra_neighbors derives it (md_intra.c:60-83): a side is available
    when its last 4x4 unit lies inside the picture and, for the top-right and
    left-down runs, when it precedes the block in the z-scan of 4x4 units
    within the LCU (the rule the tab_TR_Avail / tab_DL_Avail tables of
    block_info.c:50-160 hold; the row above the LCU counts as coded, the LCU
    to the right and the row below it as not)."""
    rects = np.asarray(rects, np.int64).reshape(-1, 4)
    x, y, w, h = rects.T
    n = lcu_size // 4
    left = x >= 4
    top = y >= 4
    tl = left & top
    # the top-right run's last unit, the left-down run's last unit
    tr = top & (x + 2 * w - 4 < width)
    ld = left & (y + 2 * h - 4 < height)
    ux, uy = ((x + w) // 4 - 1) % n, (y // 4) % n                    # the block's top-right 4x4 unit
    tr_z = np.where(uy == 0, True, np.where(ux == n - 1, False, _zorder(ux + 1, uy - 1) < _zorder(ux, uy)))
    vx, vy = (x // 4) % n, ((y + h) // 4 - 1) % n                    # the block's bottom-left 4x4 unit
    ld_z = np.where(vy == n - 1, False, np.where(vx == 0, True, _zorder(vx - 1, vy + 1) < _zorder(vx, vy)))
    return (left.astype(np.int32) | top << 1 | (ld & ld_z) << 2 | (tr & tr_z) << 3 | tl << 4).astype(np.int32)


def intra_fill_jobs(rects, width, height, rng, block_dtype, job_dtype, lcu_size=64):
    """Descriptors for building every block's edge on the device from a
    reconstructed picture (xavs2gpu_intra_fill_edges) and for the RMD batch
    that reads them: each window 16-byte aligned in an edge buffer of
    `size` bytes, availability from intra_neighbors, the DC availability
    word from its top / left bits, random MPMs.  Returns (blocks, jobs, size)."""
    rects = np.asarray(rects, np.int64).reshape(-1, 4)
    n = len(rects)
    win = np.array([intra_edge_window(int(w), int(h)) for _, _, w, h in rects], np.int64).reshape(-1, 2)
    size = (win[:, 0] + win[:, 1] + 1 + 15) // 16 * 16
    start = np.cumsum(size) - size
    avail = intra_neighbors(rects, width, height, lcu_size)
    jobs = np.zeros(n, job_dtype)
    jobs["edge_offset"] = start + win[:, 0]
    jobs["x"], jobs["y"] = rects[:, 0], rects[:, 1]
    jobs["width"], jobs["height"] = rects[:, 2], rects[:, 3]
    jobs["avail"] = avail
    blocks = np.zeros(n, block_dtype)
    blocks["edge_offset"] = jobs["edge_offset"]
    blocks["fenc_offset"] = rects[:, 1] * width + rects[:, 0]
    blocks["width"], blocks["height"] = rects[:, 2], rects[:, 3]
    blocks["dc_avail"] = (((avail >> 1) & 1) << 8) | (avail & 1)
    m0 = rng.integers(0, 33, n)
    m1 = rng.integers(0, 32, n)
    blocks["mpm"][:, 0] = m0
    blocks["mpm"][:, 1] = m1 + (m1 >= m0)
    level = np.log2(np.maximum(rects[:, 2], rects[:, 3])).astype(int)
    blocks["num_for_rdo"] = np.array([INTRA_RDO_NUM.get(v, 6) for v in range(7)])[level]
    return blocks, jobs, int(size.sum())


def intra_level_blocks(width, height, shapes=None):
    """Every block an encoder's intra mode decision visits on a picture: the
    CUs of each level (64 .. 8) that lie inside it, the 4x4 blocks, and the
    SDIP strips of the 32 / 16 CUs, each set tiling the picture."""
    shapes = shapes or INTRA_ENC_SHAPES
    rects = []
    for bw, bh in shapes:
        ys, xs = np.meshgrid(np.arange(0, height - bh + 1, bh), np.arange(0, width - bw + 1, bw), indexing="ij")
        rects.append(np.stack([xs.ravel(), ys.ravel(), np.full(xs.size, bw), np.full(xs.size, bh)], 1))
    return np.concatenate(rects)


# ---- in-loop filters --------------------------------------------------------------
def _blocky(rng, w, h, amp):
    from scipy.ndimage import gaussian_filter
    img = gaussian_filter(rng.integers(0, 256, (h, w)).astype(np.float64), 2.0)
    img = 40 + (img - img.min()) * (170.0 / max(np.ptp(img), 1e-9))
    off = rng.integers(-amp, amp + 1, ((h + 7) // 8, (w + 7) // 8))
    img += np.kron(off, np.ones((8, 8)))[:h, :w]
    return np.clip(np.round(img), 0, 255).astype(np.uint8)


def deblock_picture(rng, w, h, p_edge=0.8):
    """A 4:2:0 picture with 8x8 blocking artefacts (blurred noise plus a
    random offset per 8x8 block) and per-8x8-block edge parameters: edge type
    (none / luma only / both) per direction with none on the picture border,
    half-edge flags, and alpha / beta in the ranges of the AVS2 tables."""
    from . import DEBLOCK_SCU_DTYPE
    y = _blocky(rng, w, h, 6)
    u = _blocky(rng, w // 2, h // 2, 4)
    v = _blocky(rng, w // 2, h // 2, 4)
    n = (w // 8) * (h // 8)
    scus = np.zeros(n, DEBLOCK_SCU_DTYPE)
    t = rng.random((n, 2))
    scus["type"] = np.where(t < p_edge * 0.75, 2, np.where(t < p_edge, 1, 0))
    sx = np.arange(n) % (w // 8)
    sy = np.arange(n) // (w // 8)
    scus["type"][sx == 0, 0] = 0
    scus["type"][sy == 0, 1] = 0
    scus["flag"] = (rng.random((n, 2, 2)) < 0.9).astype(np.uint8)
    scus["alpha"] = rng.integers(4, 65, (n, 2))
    scus["beta"] = rng.integers(1, 28, (n, 2))
    scus["alpha_c"] = rng.integers(4, 65, (n, 2))
    scus["beta_c"] = rng.integers(1, 28, (n, 2))
    return y, u, v, scus


def sao_params(rng, w, h, lcu_level, p_off=0.1):
    """Per-LCU SAO parameters: per component a type (off with probability
    p_off, else EO_0 / EO_90 / EO_135 / EO_45 / BO uniformly), EO offsets in
    the AVS2 ranges (class 0, 1 >= 0; class 3, 4 <= 0; class 2 zero), BO
    offsets on four bands from a random start band, and the side
    availabilities of a single-slice picture."""
    from . import SAO_LCU_DTYPE
    S = 1 << lcu_level
    wl, hl = (w + S - 1) // S, (h + S - 1) // S
    lcus = np.zeros(wl * hl, SAO_LCU_DTYPE)
    lx = np.arange(wl * hl) % wl
    ly = np.arange(wl * hl) // wl
    lcus["avail"] = (ly > 0) | ((ly < hl - 1) << 1) | ((lx > 0) << 2) | ((lx < wl - 1) << 3)
    for i in range(wl * hl):
        for c in range(3):
            if rng.random() < p_off:
                lcus["type"][i, c] = -1
                continue
            t = int(rng.integers(0, 5))
            lcus["type"][i, c] = t
            if t < 4:
                lcus["offset"][i, c, :5] = (rng.integers(0, 7), rng.integers(0, 2), 0, -rng.integers(0, 2),
                                            -rng.integers(0, 7))
            else:
                b = int(rng.integers(0, 29))
                lcus["offset"][i, c, b:b + 4] = rng.integers(-7, 8, 4)
    return lcus


# ---- skip / direct candidates -----------------------------------------------------
def skip_candidates(rng, width, height, nrefs, per_cu=5, motion=(0, 0), levels=(3, 4, 5, 6), cand_dtype=None):
    """Candidates for every aligned CU of the given levels inside the
    picture: first a temporal-style candidate with four quadrant PUs, then
    single-PU candidates around `motion` (quarter-pel), a third of them
    bi-predicted from two references, some repeating an earlier candidate's
    motion (the encoder skips those); header bits 1..12.  Returns
    (candidates, number of CUs)."""
    rects = []
    for lv in levels:
        S = 1 << lv
        for y in range(0, height - S + 1, S):
            for x in range(0, width - S + 1, S):
                rects.append((x, y, lv))
    n_cu = len(rects)
    cands = np.zeros(n_cu * per_cu, cand_dtype)
    cands["ref"] = -1
    mx0, my0 = motion
    k = 0
    for cu, (x, y, lv) in enumerate(rects):
        for j in range(per_cu):
            c = cands[k]
            c["x"], c["y"], c["size_log2"], c["cu"] = x, y, lv, cu
            c["rate"] = int(rng.integers(1, 13))
            if j == 0:
                c["n_pu"] = 4
                for q in range(4):
                    c["ref"][q, 0] = int(rng.integers(0, nrefs))
                    c["mv"][q, 0] = (mx0 + int(rng.integers(-6, 7)), my0 + int(rng.integers(-6, 7)))
            elif j >= 3 and rng.random() < 0.3:
                c["n_pu"] = cands[k - 1]["n_pu"]
                c["ref"] = cands[k - 1]["ref"]
                c["mv"] = cands[k - 1]["mv"]
            else:
                c["n_pu"] = 1
                c["ref"][0, 0] = int(rng.integers(0, nrefs))
                c["mv"][0, 0] = (mx0 + int(rng.integers(-12, 13)), my0 + int(rng.integers(-12, 13)))
                if nrefs > 1 and rng.random() < 0.35:
                    c["ref"][0, 1] = int(rng.integers(0, nrefs))
                    c["mv"][0, 1] = (mx0 + int(rng.integers(-12, 13)), my0 + int(rng.integers(-12, 13)))
            cands[k] = c
            k += 1
    return cands, n_cu
