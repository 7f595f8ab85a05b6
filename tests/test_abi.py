"""The C-ABI library loads and exports every function include/pcd.h declares
(no device calls: runs without a GPU)."""
import os
import re

from conftest import ROOT


def declared_functions():
    src = open(os.path.join(ROOT, "include", "pcd.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pcd_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    from poisson_caustic_design_gb300 import _lib

    L = _lib.load()
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    # the ctypes table covers the same set
    assert set(names) <= set(_lib.SIGNATURES), set(names) - set(_lib.SIGNATURES)



def test_tensor_core_entry_points_refuse_unsupported_arguments():
    """The tcgen05 GEMM and convolution entry points check their arguments on
    the host before any device call (so this runs without a GPU): images that
    do not tile into the TMA boxes, fewer than 32 channels, a box of more
    images than the batch, MN-major extents below the 64-wide box, an unknown
    kernel path or default."""
    from poisson_caustic_design_gb300 import _lib

    L = _lib.load()
    bad = 2  # PCD_BAD_ARG
    x, w, out = 1 << 20, 2 << 20, 3 << 20  # placeholders, 16-byte aligned; never dereferenced
    assert L.pcd_conv3x3_bf16(x, 2, 24, 24, 64, 64, w, 576, 32, out, 32, None) == bad    # 24 x 24 does not tile
    assert L.pcd_conv3x3_bf16(x, 2, 16, 16, 16, 16, w, 144, 32, out, 32, None) == bad    # 16 channels
    assert L.pcd_conv3x3_bf16(x, 1, 8, 8, 64, 64, w, 576, 32, out, 32, None) == bad      # box of 2 images, batch 1
    assert L.pcd_conv3x3_bf16(x + 8, 2, 16, 16, 64, 64, w, 576, 32, out, 32, None) == bad  # x not 16-byte aligned
    assert L.pcd_conv3x3_wgrad_bf16(x, 2, 16, 16, 64, 64, w, 16, out, 576, 1, None, None) == bad  # N below 32
    assert L.pcd_gemm_bf16_layout(x, 40, 1, w, 64, 1, out, 40, 1, 32, 64, 256, 1, None, None) == bad  # M 32 < 64
    assert L.pcd_gemm_bf16_path(x, 64, w, 64, out, 64, 64, 64, 64, 1, None, 5, None) == bad
    assert L.pcd_gemm_set_default_path(3) == bad
    assert b"tcgen05" in L.pcd_last_error() or b"default path" in L.pcd_last_error()
