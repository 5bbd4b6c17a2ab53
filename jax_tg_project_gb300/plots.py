"""Headless PNG output of field slices and diagnostic series (no matplotlib).

The reference writes two figures at the end of a run with matplotlib
(jax/taylor_green_jax.py:282-306, cuda/taylor_green_cuda/plotting.py:7-31,
cuda/taylor_green_mhd/plotting.py:9-48): the velocity (and magnetic) components
on a mid plane, and the energy / enstrophy (MHD: kinetic, magnetic, total energy,
cross helicity) series.  Here the same two images are rasterised with
NumPy and written by a small PNG encoder (zlib + CRC-32 chunks, the PNG
specification's filter type 0 rows): one panel per field component with a
colour bar, and one line plot per series with grid lines and square markers.
Panels carry no text; ``save_plots`` returns the value range of every panel so
that callers can print it.  File names follow the reference.
"""
from __future__ import annotations

import struct
import zlib

import numpy as np

# anchor colours of the viridis and plasma palettes (van der Walt & Smith), interpolated
_VIRIDIS = ["#440154", "#482878", "#3e4989", "#31688e", "#26828e", "#1f9e89", "#35b779",
            "#6ece58", "#b5de2b", "#fde725"]
_PLASMA = ["#0d0887", "#46039f", "#7201a8", "#9c179e", "#bd3786", "#d8576b", "#ed7953",
           "#fb9f3a", "#fdca26", "#f0f921"]
_PALETTES = {"viridis": _VIRIDIS, "plasma": _PLASMA}

FILES = {  # (slice, diagnostics) file names of the reference entry points
    "jax": ("taylor_green_slice.png", "taylor_green_diagnostics.png"),
    "hydro": ("taylor_green_cuda_slice.png", "taylor_green_cuda_diagnostics.png"),
    "mhd": ("taylor_green_mhd_slice.png", "taylor_green_mhd_diagnostics.png"),
}


def write_png(path, img):
    """Write an (H, W, 3) uint8 RGB image as a PNG file."""
    img = np.ascontiguousarray(img, dtype=np.uint8)
    if img.ndim != 3 or img.shape[2] != 3:
        raise ValueError("write_png expects an (H, W, 3) uint8 array")
    h, w, _ = img.shape

    def chunk(kind, data):
        return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data))

    raw = b"".join(b"\x00" + img[r].tobytes() for r in range(h))  # filter type 0 per row
    png = (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0))
           + chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b""))
    with open(path, "wb") as f:
        f.write(png)


def read_png(path):
    """Read an RGB PNG written by ``write_png`` (8-bit, filter type 0) back into an array."""
    with open(path, "rb") as f:
        data = f.read()
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG file")
    pos, idat, w = 8, b"", None
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        kind = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        if struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0] != zlib.crc32(kind + body):
            raise ValueError(f"bad CRC in chunk {kind!r}")
        if kind == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
            if (depth, ctype) != (8, 2):
                raise ValueError("only 8-bit RGB")
        elif kind == b"IDAT":
            idat += body
        pos += 12 + n
    rows = np.frombuffer(zlib.decompress(idat), dtype=np.uint8).reshape(h, 1 + 3 * w)
    if np.any(rows[:, 0] != 0):
        raise ValueError("only filter type 0")
    return rows[:, 1:].reshape(h, w, 3).copy()


def colormap(values, name="viridis", lo=None, hi=None):
    """Map values to RGB (uint8) by linear interpolation between the palette anchors."""
    anchors = np.array([[int(c[i:i + 2], 16) for i in (1, 3, 5)] for c in _PALETTES[name]], float)
    v = np.asarray(values, dtype=np.float64)
    lo = np.nanmin(v) if lo is None else lo
    hi = np.nanmax(v) if hi is None else hi
    s = np.zeros_like(v) if hi <= lo else np.clip((v - lo) / (hi - lo), 0.0, 1.0)
    pos = s * (len(anchors) - 1)
    i0 = np.minimum(pos.astype(int), len(anchors) - 2)
    f = (pos - i0)[..., None]
    return np.round(anchors[i0] * (1 - f) + anchors[i0 + 1] * f).astype(np.uint8)


def _upscale(img, scale):
    return np.repeat(np.repeat(img, scale, axis=0), scale, axis=1)


def slice_panels(fields, cmaps, scale=None, pad=12, bar=14):
    """Panels of 2-D fields (row-major list of rows, each a list of (nx, ny) arrays) drawn
    like imshow(field.T, origin="lower") with a colour bar to the right of each; returns
    the image and the (min, max) of every panel."""
    rows = len(fields)
    cols = max(len(r) for r in fields)
    n = max(f.shape[0] for r in fields for f in r)
    scale = scale or max(1, 256 // n)
    ph = pw = n * scale
    cw = pw + pad + bar + 2 * pad
    ch = ph + 2 * pad
    img = np.full((rows * ch, cols * cw, 3), 255, np.uint8)
    ranges = []
    for r, row in enumerate(fields):
        for c, fld in enumerate(row):
            fld = np.asarray(fld, dtype=np.float64)
            lo, hi = float(fld.min()), float(fld.max())
            ranges.append((lo, hi))
            tile = colormap(fld.T[::-1], cmaps[r], lo, hi)  # transpose, origin at the bottom
            tile = _upscale(tile, scale)
            y0, x0 = r * ch + pad, c * cw + pad
            img[y0:y0 + tile.shape[0], x0:x0 + tile.shape[1]] = tile
            ramp = colormap(np.linspace(hi, lo, tile.shape[0])[:, None].repeat(bar, 1), cmaps[r], lo, hi)
            bx = x0 + pw + pad
            img[y0:y0 + tile.shape[0], bx:bx + bar] = ramp
    return img, ranges


def _line(img, x0, y0, x1, y1, color):
    n = int(max(abs(x1 - x0), abs(y1 - y0))) + 1
    xs = np.round(np.linspace(x0, x1, n)).astype(int)
    ys = np.round(np.linspace(y0, y1, n)).astype(int)
    ok = (xs >= 0) & (xs < img.shape[1]) & (ys >= 0) & (ys < img.shape[0])
    img[ys[ok], xs[ok]] = color


def series_panels(t, series, colors, ncols=1, width=900, height=320, pad=30):
    """Line plots (one panel per series, ncols per row) with a light grid and square markers;
    returns the image and the (min, max) of every series."""
    t = np.asarray(t, dtype=np.float64)
    nrow = (len(series) + ncols - 1) // ncols
    img = np.full((nrow * height, ncols * width, 3), 255, np.uint8)
    ranges = []
    for k, (y, col) in enumerate(zip(series, colors)):
        y = np.asarray(y, dtype=np.float64)
        r, c = divmod(k, ncols)
        X0, Y0 = c * width + pad, r * height + pad
        W, H = width - 2 * pad, height - 2 * pad
        lo, hi = float(y.min()), float(y.max())
        ranges.append((lo, hi))
        span = (hi - lo) or max(abs(hi), 1.0)
        tl, th = float(t.min()), float(t.max())
        tspan = (th - tl) or 1.0
        for g in range(1, 5):  # grid
            gx = X0 + W * g // 5
            gy = Y0 + H * g // 5
            img[Y0:Y0 + H, gx] = (225, 225, 225)
            img[gy, X0:X0 + W] = (225, 225, 225)
        img[Y0, X0:X0 + W] = img[Y0 + H - 1, X0:X0 + W] = 0  # frame
        img[Y0:Y0 + H, X0] = img[Y0:Y0 + H, X0 + W - 1] = 0
        px = X0 + 4 + (W - 9) * (t - tl) / tspan
        py = Y0 + H - 5 - (H - 9) * (y - lo) / span
        rgb = tuple(int(col[i:i + 2], 16) for i in (1, 3, 5))
        for i in range(len(t) - 1):
            _line(img, px[i], py[i], px[i + 1], py[i + 1], rgb)
        for xi, yi in zip(np.round(px).astype(int), np.round(py).astype(int)):
            img[max(yi - 2, 0):yi + 3, max(xi - 2, 0):xi + 3] = rgb
    return img, ranges


def save_plots(plan, state, times, series, kind="hydro", directory="."):
    """Write the slice and diagnostics PNGs of a run; returns the file paths and the value
    ranges of the panels.  ``series`` is the (records, batch, 8) diagnostics array of
    ``Plan.run`` (run 0 is drawn); ``kind`` is "jax", "hydro" or "mhd" (file names)."""
    import os
    phys = plan.inverse(state)[0].float().cpu().numpy()  # (F, n, n, n)
    n = phys.shape[-1]
    # the JAX script slices u[:, :, N // 2] (the y = N/2 plane: x, z panels); the CuPy
    # packages slice [:, :, :, n // 2] (z = N/2: x, y)
    sl = phys[:, :, n // 2, :] if kind == "jax" else phys[:, :, :, n // 2]
    h = np.asarray(series)[:, 0]
    if plan.F == 6:
        img, r1 = slice_panels([[sl[0], sl[1], sl[2]], [sl[3], sl[4], sl[5]]], ["viridis", "plasma"])
        ser = [h[:, 0], h[:, 3], h[:, 5], h[:, 4]]  # E_k, E_m, total, H_c
        img2, r2 = series_panels(times, ser, ["#1f3fbf", "#d62728", "#2ca02c", "#bf3fbf"], ncols=2)
    else:
        img, r1 = slice_panels([[sl[0], sl[1], sl[2]]], ["viridis"])
        img2, r2 = series_panels(times, [h[:, 0], h[:, 1]], ["#1f3fbf", "#d62728"])
    f_slice, f_diag = (os.path.join(directory, f) for f in FILES[kind])
    write_png(f_slice, img)
    write_png(f_diag, img2)
    return {"slice": f_slice, "diagnostics": f_diag, "slice_ranges": r1, "series_ranges": r2}
