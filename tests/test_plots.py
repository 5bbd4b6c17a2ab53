"""Headless PNG output (plots.py): encoder round trip, palettes and panel layout (CPU)."""
import numpy as np
import pytest

from jax_tg_project_gb300 import plots


def test_png_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    img = rng.integers(0, 256, size=(37, 53, 3), dtype=np.uint8)
    path = str(tmp_path / "a.png")
    plots.write_png(path, img)
    back = plots.read_png(path)
    assert back.dtype == np.uint8 and np.array_equal(back, img)
    with open(path, "rb") as f:
        data = bytearray(f.read())
    data[40] ^= 0xFF  # corrupt a byte inside a chunk: the CRC check catches it
    bad = str(tmp_path / "b.png")
    with open(bad, "wb") as f:
        f.write(bytes(data))
    with pytest.raises(ValueError):
        plots.read_png(bad)


def test_palette_endpoints_and_order():
    v = plots.colormap(np.array([0.0, 1.0]), "viridis")
    assert tuple(v[0]) == (0x44, 0x01, 0x54) and tuple(v[1]) == (0xfd, 0xe7, 0x25)
    p = plots.colormap(np.linspace(0, 1, 50), "plasma")
    assert tuple(p[0]) == (0x0d, 0x08, 0x87) and tuple(p[-1]) == (0xf0, 0xf9, 0x21)
    flat = plots.colormap(np.full(4, 3.0))  # constant field: no division by zero
    assert (flat == flat[0]).all()


def test_slice_panels_layout():
    x = np.linspace(0, 2 * np.pi, 16, endpoint=False)
    f = np.sin(x)[:, None] * np.cos(x)[None, :]
    img, ranges = plots.slice_panels([[f, -f, 0 * f]], ["viridis"])
    assert img.shape[0] == 16 * 16 + 24 and img.shape[1] == 3 * (256 + 12 + 14 + 24)
    assert ranges[0] == pytest.approx((f.min(), f.max())) and ranges[2] == (0.0, 0.0)
    # origin at the bottom: field row x=0 is the left column, y grows upwards
    tile = img[12:12 + 256, 12:12 + 256]
    assert np.array_equal(tile[-1, 0], plots.colormap(np.array([f[0, 0]]), "viridis", f.min(), f.max())[0])


def test_series_panels_draw_lines():
    t = np.linspace(0, 1, 11)
    img, ranges = plots.series_panels(t, [np.exp(-t), t ** 2], ["#1f3fbf", "#d62728"])
    assert img.shape == (640, 900, 3)
    blue = np.all(img == (0x1f, 0x3f, 0xbf), axis=-1)
    red = np.all(img == (0xd6, 0x27, 0x28), axis=-1)
    assert blue[:320].sum() > 100 and red[320:].sum() > 100 and not red[:320].any()
    assert ranges[0] == pytest.approx((np.exp(-1.0), 1.0))
