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
