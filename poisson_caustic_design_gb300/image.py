"""Image ingest (main.cpp:13-109): the reference's PNG loader and resize.

    gray = image_to_grid("target.png")                  # main.cpp:29-109
    pixels = resize_image(gray, 4 * res, 4 * res)       # main.cpp:13-27 (GPU)

``image_to_grid`` decodes the PNG in the library (host code; libpng's
transforms as the reference sets them) and returns the gray grid
0.299 r + 0.587 g + 0.114 b of samples / 255 as a height x width float64 array.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check


def image_to_grid(filename: str) -> np.ndarray:
    L = _lib.load()
    w, h = C.c_int(0), C.c_int(0)
    check(L.pcd_image_to_grid(filename.encode(), C.byref(w), C.byref(h), None), "pcd_image_to_grid")
    out = np.empty((h.value, w.value))
    check(L.pcd_image_to_grid(filename.encode(), C.byref(w), C.byref(h),
                              out.ctypes.data_as(C.POINTER(C.c_double))), "pcd_image_to_grid")
    return out


def png_decode(data: bytes) -> np.ndarray:
    """8-bit RGBA (height x width x 4) of a PNG byte string."""
    L = _lib.load()
    w, h = C.c_int(0), C.c_int(0)
    check(L.pcd_png_decode(data, len(data), C.byref(w), C.byref(h), None), "pcd_png_decode")
    out = np.empty((h.value, w.value, 4), dtype=np.uint8)
    check(L.pcd_png_decode(data, len(data), C.byref(w), C.byref(h), out.ctypes.data_as(C.c_char_p)),
          "pcd_png_decode")
    return out


def resize_image(image, new_width: int, new_height: int) -> np.ndarray:
    """resize_image (main.cpp:13-27) on the GPU: nearest sample at integer
    source indices x * old_width / new_width, y * old_height / new_height."""
    img = np.ascontiguousarray(image, dtype=np.float64)
    out = np.empty((int(new_height), int(new_width)))
    L = _lib.load()
    check(L.pcd_resize_image(img.ctypes.data_as(C.POINTER(C.c_double)), img.shape[1], img.shape[0],
                             out.ctypes.data_as(C.POINTER(C.c_double)), int(new_width), int(new_height)),
          "pcd_resize_image")
    return out
