"""Headless image output: the RGBA32F texels crt_render_frame / crt_shade
write, saved as a binary PPM (the reference shows its oImage texture on a
full-screen quad, srcOpenGL/application.cpp:248-260; with no display here the
texture goes to a file)."""
from __future__ import annotations

import numpy as np


def to_rgb8(texels, width: int, height: int) -> np.ndarray:
    """(height, width, 3) uint8, top row first: texture row 0 is the bottom of
    the displayed image (GL texture origin), colour channels clamped to [0, 1]
    and rounded to 8 bits, alpha dropped."""
    t = np.asarray(texels, np.float32).reshape(height, width, 4)
    rgb = np.clip(np.nan_to_num(t[::-1, :, :3], nan=0.0), 0.0, 1.0)
    return np.floor(rgb * 255.0 + 0.5).astype(np.uint8)


def write_ppm(path: str, texels, width: int, height: int) -> None:
    rgb = to_rgb8(texels, width, height)
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (width, height))
        f.write(rgb.tobytes())
