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
