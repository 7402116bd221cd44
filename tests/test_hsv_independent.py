"""A second, independent statement of the colour adjustment against the oracle's.

color_adjustment.rs:53-87 adjust_pixel converts the brightness/contrast-adjusted
pixel to HSV with palette 0.7.6, shifts the hue, scales the saturation and
converts back.  The oracle (and the CUDA path, bit for bit) restates palette's
hexcone conversion in palette's own case split.  Here the same adjustment is
written again from the textbook hexcone model (A. R. Smith, "Color gamut
transform pairs", SIGGRAPH 1978: V = max, C = max - min, H' = ((G-B)/C) mod 6,
(B-R)/C + 2 or (R-G)/C + 4 by the maximal channel, S = C/V; back through
X = C (1 - |H' mod 2 - 1|) and the six sectors), vectorised in float32 numpy
with one rounding per operation, and compared with the oracle over every third
sRGB8 colour for several adjustments.  The two formulations may round
differently (the textbook hue is taken mod 6, palette's may be negative before
the shift), so the bar is the path's pixel tolerance of +-1 LSB, and the share
of bit-identical channels is checked too: a misread hexcone (a wrong sector, a
reversed hue direction) would differ by far more, on many colours.
"""
import ctypes as C

import numpy as np
import pytest

F = np.float32


def _colours():
    """Every third sRGB8 colour (5.6 million): the colours whose R + G + B is a
    multiple of 3, so every pair of values of any two channels occurs."""
    i = np.arange(0, 1 << 24, 3, dtype=np.uint32)
    return np.stack([(i >> 16) & 0xFF, (i >> 8) & 0xFF, i & 0xFF], -1).astype(np.uint8)


def adjust_textbook(rgb: np.ndarray, brightness: float, contrast: float, hue: float, sat: float) -> np.ndarray:
    """color_adjustment.rs:53-87 from the textbook hexcone model, float32 per op."""
    b, c, h_shift, s_mul = F(brightness), F(contrast), F(hue), F(sat)
    v = rgb.astype(F) / F(255.0)
    x = np.clip((v - F(0.5)) * c + F(0.5), F(0.0), F(1.0))  # contrast about 0.5
    x = np.clip(x + b, F(0.0), F(1.0))                          # then brightness
    if h_shift != 0.0 or s_mul != 1.0:
        r, g, bl = x[:, 0], x[:, 1], x[:, 2]
        V = np.maximum(np.maximum(r, g), bl)
        m = np.minimum(np.minimum(r, g), bl)
        Cc = V - m
        safe = np.where(Cc > 0, Cc, F(1.0))
        hp = np.where(V == r, np.mod((g - bl) / safe, F(6.0)),
                      np.where(V == g, (bl - r) / safe + F(2.0), (r - g) / safe + F(4.0)))
        H = np.where(Cc > 0, hp * F(60.0), F(0.0)).astype(F)
        S = np.where(V > 0, Cc / np.where(V > 0, V, F(1.0)), F(0.0)).astype(F)
        H2 = np.mod(H + h_shift, F(360.0)).astype(F)
        S2 = np.clip(S * s_mul, F(0.0), F(1.0))
        C2 = V * S2
        Hp = H2 / F(60.0)
        X = C2 * (F(1.0) - np.abs(np.mod(Hp, F(2.0)) - F(1.0)))
        sector = np.floor(Hp).astype(np.int32)
        zero = np.zeros_like(C2)
        r1 = np.select([sector == 0, sector == 1, sector == 2, sector == 3, sector == 4], [C2, X, zero, zero, X], C2)
        g1 = np.select([sector == 0, sector == 1, sector == 2, sector == 3, sector == 4], [X, C2, C2, X, zero], zero)
        b1 = np.select([sector == 0, sector == 1, sector == 2, sector == 3, sector == 4], [zero, zero, X, C2, C2], X)
        mm = V - C2
        x = np.clip(np.stack([r1 + mm, g1 + mm, b1 + mm], -1).astype(F), F(0.0), F(1.0))
    return np.clip(x * F(255.0), F(0.0), F(255.0)).astype(np.uint8)  # `as u8` truncates


# (brightness, contrast, hue shift, saturation): the ranges calculate_optimal_adjustment
# produces at strength <= 1 (contrast 1, hue within +-90, saturation around 1), plus a
# contrast change and the clamps' ends
SETTINGS = [(0.0, 1.0, 37.5, 1.0), (0.1, 1.0, -64.0, 0.8), (-0.2, 1.0, 12.25, 1.35), (0.0, 1.0, 0.0, 0.4),
            (0.05, 1.3, -90.0, 1.6), (0.0, 1.0, 179.0, 1.0), (-1.0, 1.0, 5.0, 2.0)]


@pytest.mark.parametrize("setting", SETTINGS)
def test_textbook_hexcone_agrees_with_the_oracle(orc, setting):
    rgb = _colours()
    want = adjust_textbook(rgb, *setting)
    got = np.empty_like(rgb)
    adj = np.array(setting, np.float32)
    orc.lib().orc_adjust_pixels(adj.ctypes.data_as(C.POINTER(C.c_float)), rgb.ctypes.data_as(C.POINTER(C.c_uint8)),
                                rgb.shape[0], got.ctypes.data_as(C.POINTER(C.c_uint8)))
    diff = np.abs(got.astype(np.int16) - want.astype(np.int16))
    same = float((diff == 0).mean())
    print(f"setting {setting}: max diff {int(diff.max())}, identical channels {100 * same:.5f}%")
    assert diff.max() <= 1, setting
    assert same > 0.995, setting  # observed 99.80-100% over all 2^24 colours
