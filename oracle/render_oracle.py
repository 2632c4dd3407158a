"""CPU restatement of the headless point rasteriser (test infrastructure only).

The reference's draw pass (assets/shaders/draw.wgsl:18-40): one quad of
half-size 0.4 world units per particle, white on black, MSAA 4
(runners/bevy/src/render/pipeline.rs:52-56).  Pixel coordinates
X = x * sx, Y = height_px - y * sy (sx = width_px / W, sy = height_px / H);
a particle covers [X - hx, X + hx) x [Y - hy, Y + hy), hx = 0.4 sx,
hy = 0.4 sy; the four standard sample positions per pixel.  A multisampled
target turns a sample white once any quad covers it, so a pixel resolves to
255 * (samples covered by the union of the quads) // 4.
"""
import numpy as np

SX = np.array([0.375, 0.875, 0.125, 0.625], np.float32)
SY = np.array([0.125, 0.375, 0.625, 0.875], np.float32)


def render(pos, world_w, world_h, width_px, height_px):
    f = np.float32
    pos = np.asarray(pos, np.float32).reshape(-1, 2)
    sx, sy = f(f(width_px) / f(world_w)), f(f(height_px) / f(world_h))
    cover = np.zeros((height_px, width_px), np.uint32)
    hx, hy = f(f(0.4) * sx), f(f(0.4) * sy)
    for x, y in pos:
        X = f(x * sx)
        Y = f(f(height_px) - f(y * sy))
        x0, x1, y0, y1 = f(X - hx), f(X + hx), f(Y - hy), f(Y + hy)
        if not (x1 > 0 and y1 > 0 and x0 < width_px and y0 < height_px):
            continue
        for py in range(max(int(np.floor(y0)), 0), min(int(np.floor(y1)), height_px - 1) + 1):
            for px in range(max(int(np.floor(x0)), 0), min(int(np.floor(x1)), width_px - 1) + 1):
                s_x = (f(px) + SX).astype(np.float32)
                s_y = (f(py) + SY).astype(np.float32)
                hit = (s_x >= x0) & (s_x < x1) & (s_y >= y0) & (s_y < y1)
                cover[py, px] |= int(np.sum(hit.astype(np.uint32) << np.arange(4, dtype=np.uint32)))
    samples = sum((cover >> k) & 1 for k in range(4))
    return (255 * samples // 4).astype(np.uint8)
