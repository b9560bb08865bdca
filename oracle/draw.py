"""CPU restatement of the renderer's particle fields (src/render.rs:886-1075: the splat, tint,
down and blur passes of Renderer::render; shaders/splat.vert, splat.frag, tint.frag,
down.frag, blur.frag) and of the wet map (render.rs:640-668, shaders/wet.frag).

Test infrastructure: the checker of the engine's draw (sprout_sim_draw). numpy float32 for
the arithmetic, each operation in the order the engine's kernels take it, so the two agree bit
for bit. Where the reference leaves the order or the precision to the graphics hardware, the
engine fixes them and this restatement follows the engine:
- a texel's uv is the affine map the triangle interpolates, evaluated at the texel's centre
  (by reciprocals of the zoom, the kernel's radius and its length along the path);
- the particles' contributions are summed as 64-bit fixed point (2^-32, round to nearest
  even) and rounded to half once (the hardware blends each one into a half-float target);
- bilinear taps weigh the texels by the exact fraction (the hardware by a few bits of it).
Parity with the reference's own images is unpinned: its passes run under Vulkan, which is
unavailable here. render.rs's own test (wide_field_fits_its_image_at_every_zoom) is restated on
`layout` in tests/test_draw.py.
"""
from __future__ import annotations

import numpy as np

f32 = np.float32

# render.rs constants
SPLAT_RADIUS = f32(1.5)
ACCUM_KERNEL_TEXELS = f32(2.8)
ACCUM_MAX_DIV = f32(2.0)
SPLAT_MIN_TEXELS = f32(1.5)
EXPOSURE = f32(1.0) / f32(160.0)
WIDE_SIGMA = f32(2.0)
WIDE_SIGMA_TEXELS = f32(3.0)
WIDE_MIN_FACTOR = f32(2.0)
WIDE_MAX_FACTOR = f32(64.0)
TINT_DIV = 2
LOOK_RADIUS = f32(1.0)
ROW_STEAM = 57         # common.glsl
STREAK_MAX = f32(1.5)  # splat.vert
REACH = f32(1.75)      # wet.frag
WETTING = f32(0.3)
G = [f32(v) for v in (1.0, 0.8825, 0.6065, 0.3247, 0.1353, 0.0439, 0.0111)]   # blur.frag
FIX = 2.0 ** 32


def _clampf(v, lo, hi):
    return f32(min(max(f32(v), f32(lo)), f32(hi)))


def layout(center, zoom, extent, tint_live=True):
    """The passes' parameters for a view (render.rs:889-930, WideLayout::new 245-251, the
    images of ensure_targets 715, 742-745): per pass its map, kernel and used texels."""
    zoom = f32(zoom)
    ew, eh = int(extent[0]), int(extent[1])
    half_w, half_h = f32(ew) * f32(0.5), f32(eh) * f32(0.5)
    div = _clampf(SPLAT_RADIUS * zoom / ACCUM_KERNEL_TEXELS, 1.0, ACCUM_MAX_DIV)
    aw = min(max(int(np.ceil(f32(ew) / div)), 1), ew)
    ah = min(max(int(np.ceil(f32(eh) / div)), 1), eh)
    radius = max(SPLAT_RADIUS, f32(SPLAT_MIN_TEXELS * div / zoom))
    weight = f32(f32(SPLAT_RADIUS / radius) * f32(SPLAT_RADIUS / radius))
    base = dict(cx=f32(center[0]), cy=f32(center[1]), zoom=zoom, half_w=half_w, half_h=half_h, exposure=EXPOSURE)
    sharp = dict(base, div=div, radius=radius, weight=weight, w=aw, h=ah, tint=False, izoom=f32(f32(1.0) / zoom),
                 iradius=f32(f32(1.0) / radius))
    dt = f32(div * f32(TINT_DIV))
    tw = min(max(-(-aw // TINT_DIV), 1), -(-ew // TINT_DIV))
    th = min(max(-(-ah // TINT_DIV), 1), -(-eh // TINT_DIV))
    rt = max(SPLAT_RADIUS, f32(SPLAT_MIN_TEXELS * dt / zoom))
    tint = dict(base, div=dt, radius=rt, weight=f32(f32(SPLAT_RADIUS / rt) * f32(SPLAT_RADIUS / rt)), w=tw, h=th, tint=True,
                izoom=f32(f32(1.0) / zoom), iradius=f32(f32(1.0) / rt))
    factor = _clampf(WIDE_SIGMA * zoom / WIDE_SIGMA_TEXELS, WIDE_MIN_FACTOR, WIDE_MAX_FACTOR)
    image = [max(1, int(np.ceil(f32(ew) / WIDE_MIN_FACTOR))), max(1, int(np.ceil(f32(eh) / WIDE_MIN_FACTOR)))]
    ww = min(max(int(np.ceil(f32(ew) / factor)), 1), image[0])
    wh = min(max(int(np.ceil(f32(eh) / factor)), 1), image[1])
    wide = dict(w=ww, h=wh, taps=int(np.ceil(f32(f32(factor / div) * f32(0.5)))), factor=f32(factor / div),
                wide_factor=factor, step=f32(f32(f32(f32(0.5) * WIDE_SIGMA) * zoom) / factor), image=image)
    rl = max(LOOK_RADIUS, f32(SPLAT_MIN_TEXELS * div / zoom))
    h0, h1, h2 = f32(-0.3375), f32(0.67), f32(f32(0.66) + f32(1.0))   # composite.frag's key light + the view
    hn = np.sqrt(f32(f32(f32(h0 * h0) + f32(h1 * h1)) + f32(h2 * h2)))
    look = dict(base, div=div, radius=rl, weight=f32(f32(LOOK_RADIUS / rl) * f32(LOOK_RADIUS / rl)), w=aw, h=ah, look=True,
                tint=False, izoom=f32(f32(1.0) / zoom), iradius=f32(f32(1.0) / rl), H=(f32(h0 / hn), f32(h1 / hn), f32(h2 / hn)))
    return dict(sharp=sharp, tint=tint if tint_live else None, wide=wide, look=look)


def shares_a_group(rows, groups):
    """FluidSim::shares_a_group (mod.rs:1872-1878)."""
    seen = [0] * 8
    for r in rows:
        if r == ROW_STEAM:
            continue
        seen[min(int(groups[r]), 7)] += 1
    return any(n >= 2 for n in seen)


def _payload(p, row, groups, optics, v, st=None):
    """What particle p lays down per unit kernel: (first channel, values) (splat.vert; look.vert
    with its look.comp state st)."""
    if v.get("look"):
        z, w = int(st[2]), v["weight"]
        ax, ay = f32(f32(z & 1023) / f32(1023.0)), f32(f32((z >> 10) & 1023) / f32(1023.0))
        az = f32(f32(f32((z >> 20) & 1023) / f32(1023.0)) - f32(0.5))
        hx, hy, hz = v["H"]
        sheen = f32(f32(f32(f32(f32(hx * hx) * ax) + f32(f32(hy * hy) * ay)) + f32(f32(f32(f32(2.0) * hx) * hy) * az))
                    + f32(f32(hz * hz) * f32(f32(f32(1.0) - ax) - ay)))
        phi = f32(f32(int(st[3]) & 0xFFFF) / f32(65535.0))
        lie = _clampf(f32(0.5) + f32(ax - ay), 0.0, 1.0)
        return 0, [f32(sheen * w), f32(phi * w), f32(lie * w), f32(f32(1.0) * w)]
    if not v["tint"]:
        return min(max(int(groups[row]), 0), 3), [v["weight"]]
    o = optics[row]
    idx = o["idx"]
    s = _clampf(p["s"], 0.0, 1.0) if idx[0] >= 0 else f32(0.0)
    kc = o["absorb"].astype(f32)
    kp = optics[idx[0]]["absorb"].astype(f32) if idx[0] >= 0 else kc
    w = f32(0.0) if row == ROW_STEAM else v["weight"]
    if idx[1] == 0:
        c = [f32(s * kc[0]) * w, f32(s * kc[1]) * w, f32(s * kc[2]) * w,
             f32(f32(s * kc[3]) + f32(f32(f32(1.0) - s) * kp[3])) * w, s * w, f32(1.0) * w, f32(0.0) * w]
    else:
        c = [kc[0] * w, kc[1] * w, kc[2] * w, kc[3] * w, f32(0.0) * w, f32(0.0) * w, w]
    return 0, [f32(x) for x in c]


def splat(parts, groups, optics, v, look_state=None, look_list=None):
    """The fixed-point texel sums of one splat pass (splat.vert + splat.frag, tint.frag with
    v["tint"], or look.vert + look.frag over the listed slots with their look.comp state):
    int64 (h, w, 4 or 8), 2^-32 units."""
    h, w = v["h"], v["w"]
    nch = 8 if v["tint"] else 4
    acc = np.zeros((h, w, nch), np.int64)
    cx, cy, zoom, div = v["cx"], v["cy"], v["zoom"], v["div"]
    half_w, half_h, radius = v["half_w"], v["half_h"], v["radius"]
    look = bool(v.get("look"))
    slots = look_list if look else range(len(parts))
    for slot in slots:
        p = parts[int(slot)]
        low = int(p["kind"]) & 255
        if not look and (low == 0 or (v["tint"] and low - 1 == ROW_STEAM)):
            continue
        row = low - 1
        vx, vy = (f32(0.0), f32(0.0)) if look else (f32(p["vel"][0]), f32(p["vel"][1]))
        speed = np.sqrt(f32(f32(vx * vx) + f32(vy * vy)))
        dx, dy = (f32(vx / speed), f32(vy / speed)) if speed > f32(1e-3) else (f32(1.0), f32(0.0))
        streak = min(f32(speed * v["exposure"]), f32(STREAK_MAX * radius))
        along = f32(radius + f32(f32(0.5) * streak))
        ialong = f32(f32(1.0) / along)
        ex = f32(f32(p["pos"][0]) - f32(dx * f32(f32(0.5) * streak)))
        ey = f32(f32(p["pos"][1]) - f32(dy * f32(f32(0.5) * streak)))
        tx0 = f32(f32(f32(f32(f32(ex - along) - cx) * zoom) + half_w) / div)
        tx1 = f32(f32(f32(f32(f32(ex + along) - cx) * zoom) + half_w) / div)
        ty0 = f32(f32(f32(-f32(f32(ey + along) - cy) * zoom) + half_h) / div)
        ty1 = f32(f32(f32(-f32(f32(ey - along) - cy) * zoom) + half_h) / div)
        if not (tx1 >= -1.0 and ty1 >= -1.0 and tx0 <= f32(w) + f32(1.0) and ty0 <= f32(h) + f32(1.0)):
            continue
        i0 = int(max(f32(np.floor(tx0)) - f32(1.0), f32(0.0)))
        i1 = int(min(f32(np.ceil(tx1)) + f32(1.0), f32(w - 1)))
        j0 = int(max(f32(np.floor(ty0)) - f32(1.0), f32(0.0)))
        j1 = int(min(f32(np.ceil(ty1)) + f32(1.0), f32(h - 1)))
        if i1 < i0 or j1 < j0:
            continue
        ii = np.arange(i0, i1 + 1).astype(f32)
        jj = np.arange(j0, j1 + 1).astype(f32)
        px = cx + ((ii + f32(0.5)) * div - half_w) * v["izoom"]
        py = cy - ((jj + f32(0.5)) * div - half_h) * v["izoom"]
        rx = (px[None, :] - ex).astype(f32)
        ry = (py[:, None] - ey).astype(f32)
        u = (rx * dx + ry * dy) * ialong
        w2 = (ry * dx - rx * dy) * v["iradius"]
        r2 = u * u + w2 * w2
        inside = r2 < f32(1.0)
        k = (f32(1.0) - r2) * (f32(1.0) - r2)
        ch0, c = _payload(p, row, groups, optics, v, look_state[int(slot)] if look else None)
        for q, cq in enumerate(c):
            val = (cq * k).astype(f32)
            fix = np.rint(val * f32(FIX)).astype(np.int64)
            acc[j0:j1 + 1, i0:i1 + 1, ch0 + q] += np.where(inside, fix, 0)
    return acc


def unfix(acc):
    """The fixed-point sums as half floats (through FP64 and FP32, as the engine rounds them)."""
    return (acc.astype(np.float64) * (1.0 / FIX)).astype(np.float32).astype(np.float16)


def look_field(parts, look_state, look_list, lay):
    """The look field (h, w, 4) float16 of the listed slots."""
    return unfix(splat(parts, None, None, lay["look"], look_state, look_list))


def fields(parts, groups, optics, lay):
    """The sharp field (h, w, 4) and, when the tint pass runs, the tint field's two images, all
    float16."""
    sharp = unfix(splat(parts, groups, optics, lay["sharp"]))
    if lay["tint"] is None:
        return sharp, None, None
    t = unfix(splat(parts, groups, optics, lay["tint"]))
    share = t[..., 4:8].copy()
    share[..., 3] = 0
    return sharp, t[..., 0:4].copy(), share


def bilinear(img, x, y):
    """Bilinear samples of a float16 (h, w, 4) image at texel coordinates (arrays), clamped to
    its edge: (1 - fy) ((1 - fx) t00 + fx t10) + fy ((1 - fx) t01 + fx t11)."""
    h, w = img.shape[:2]
    src = img.astype(np.float32)
    xs, ys = (x - f32(0.5)).astype(f32), (y - f32(0.5)).astype(f32)
    xf, yf = np.floor(xs), np.floor(ys)
    fx, fy = (xs - xf)[..., None], (ys - yf)[..., None]
    xi, yi = xf.astype(np.int64), yf.astype(np.int64)
    x0, x1 = np.clip(xi, 0, w - 1), np.clip(xi + 1, 0, w - 1)
    y0, y1 = np.clip(yi, 0, h - 1), np.clip(yi + 1, 0, h - 1)
    a, b, c, e = src[y0, x0], src[y0, x1], src[y1, x0], src[y1, x1]
    gx, gy = f32(1.0) - fx, f32(1.0) - fy
    return (gy * (gx * a + fx * b) + fy * (gx * c + fx * e)).astype(f32)


def down(sharp, wide):
    """down.frag: the wide field's first image (h, w, 4) float16."""
    sh, sw = sharp.shape[:2]
    factor, taps = wide["factor"], wide["taps"]
    yy, xx = np.meshgrid(np.arange(wide["h"]).astype(f32), np.arange(wide["w"]).astype(f32), indexing="ij")
    cx, cy = (xx + f32(0.5)) * factor, (yy + f32(0.5)) * factor
    mx, my = f32(sw) - f32(0.5), f32(sh) - f32(0.5)
    total = np.zeros(cx.shape + (4,), f32)
    for tj in range(taps):
        for ti in range(taps):
            ox = f32(f32(f32(f32(ti) + f32(0.5)) / f32(taps)) - f32(0.5)) * factor
            oy = f32(f32(f32(f32(tj) + f32(0.5)) / f32(taps)) - f32(0.5)) * factor
            total = (total + bilinear(sharp, np.minimum(cx + ox, mx), np.minimum(cy + oy, my))).astype(f32)
    return (total / f32(taps * taps)).astype(f32).astype(np.float16)


def blur(img, step, vert):
    """blur.frag, one direction: float16 (h, w, 4) in and out."""
    h, w = img.shape[:2]
    yy, xx = np.meshgrid(np.arange(h).astype(f32), np.arange(w).astype(f32), indexing="ij")
    px, py = xx + f32(0.5), yy + f32(0.5)
    hx, hy = f32(w) - f32(0.5), f32(h) - f32(0.5)
    total = (G[0] * bilinear(img, px, py)).astype(f32)
    norm = G[0]
    for k in range(1, 7):
        o = f32(f32(k) * step)
        if vert:
            a = bilinear(img, px, np.minimum(np.maximum(py + o, f32(0.5)), hy))
            b = bilinear(img, px, np.minimum(np.maximum(py - o, f32(0.5)), hy))
        else:
            a = bilinear(img, np.minimum(np.maximum(px + o, f32(0.5)), hx), py)
            b = bilinear(img, np.minimum(np.maximum(px - o, f32(0.5)), hx), py)
        total = (total + G[k] * (a + b)).astype(f32)
        norm = f32(norm + f32(f32(2.0) * G[k]))
    return (total / norm).astype(f32).astype(np.float16)


def wide_field(sharp, wide):
    """Passes 2-4: down, blur across, blur down."""
    w0 = down(sharp, wide)
    w1 = blur(w0, wide["step"], vert=False)
    return blur(w1, wide["step"], vert=True)


def wet(prev, cell, comp, sdf, sprop, now):
    """wet.frag over the grid: prev (H, W, 4) float32, updated where a cell is wet now. cell,
    comp, sprop: (H, W, 4); sdf: (H + 1, W + 1) node distances; now: float32 seconds."""
    out = prev.copy()
    d = (f32(0.25) * (((sdf[:-1, :-1] + sdf[:-1, 1:]) + sdf[1:, :-1]) + sdf[1:, 1:])).astype(f32)
    sw = sprop[..., 3].astype(f32)
    code = np.floor((sw - np.floor(sw)) * f32(128.0) + f32(0.5)).astype(f32)
    hit = ~((d > REACH) | (cell[..., 0] < WETTING)) & (code >= f32(1.0))
    out[hit, 0] = code[hit]
    out[hit, 1] = comp[..., 2][hit]
    out[hit, 2] = f32(now)
    out[hit, 3] = f32(1.0)
    return out
