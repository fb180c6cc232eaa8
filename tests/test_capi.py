"""CPU checks of the C ABI: the library loads, exports every declared symbol,
and its host-only entry points (planning, errors) behave like zimg's."""
import ctypes as C
import math
import os
import re
import threading

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "zimg_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^ZG_API\s+[\w\s\*]*?\b(zg_\w+)\s*\(", text, flags=re.M)))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("zg_compute_filter", "zg_resize_pass_create", "zg_resize_pass_process", "zg_resize_create",
                 "zg_resize_process", "zg_batch_create", "zg_batch_process", "zg_graph_build", "zg_graph_process",
                 "zg_get_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_ctypes_binding_covers_header(lib):
    from zimg_gb300 import capi
    bound = {n for n, _, _ in capi.SIGNATURES}
    assert bound == set(declared_functions())


def test_struct_layouts_match_header(lib):
    """The ctypes mirrors have the C layout (compiled check against the header)."""
    import subprocess
    import tempfile
    from zimg_gb300 import capi
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "zimg_gb300.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(zg_pass_params), sizeof(zg_resize_params), sizeof(zg_batch_io),
         sizeof(zg_image_format), sizeof(zg_graph_builder_params), sizeof(zg_image_buffer),
         offsetof(zg_image_format, active_region), sizeof(zg_colorspace_params));
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "t")
        subprocess.check_call(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), c, "-o", exe])
        got = [int(x) for x in subprocess.check_output([exe]).split()]
    want = [C.sizeof(capi.PassParams), C.sizeof(capi.ResizeParams), C.sizeof(capi.BatchIO),
            C.sizeof(capi.ImageFormat), C.sizeof(capi.GraphBuilderParams), C.sizeof(capi.ImageBuffer),
            capi.ImageFormat.active_region.offset, C.sizeof(capi.ColorspaceParams)]
    assert got == want


def test_errors_match_zimg_codes(lib):
    import zimg_gb300 as zg
    with pytest.raises(zg.ZimgError) as e:
        zg.compute_filter("lanczos", 100, 50, a=16)  # filter.cpp:232-238
    assert e.value.code == 2048  # ILLEGAL_ARGUMENT
    with pytest.raises(zg.ZimgError) as e:
        zg.compute_filter(99, 100, 50)
    assert e.value.code == 2049  # ENUM_OUT_OF_RANGE
    with pytest.raises(zg.ZimgError) as e:
        zg.compute_filter("bilinear", 0, 50)
    assert e.value.code == 2050  # INVALID_IMAGE_SIZE


def test_last_error_is_thread_local(lib):
    import zimg_gb300 as zg
    from zimg_gb300 import capi
    lib.zg_clear_last_error()
    with pytest.raises(zg.ZimgError):
        zg.compute_filter("lanczos", 100, 50, a=16)
    seen = {}

    def other():
        seen["code"] = capi.last_error()[0]

    t = threading.Thread(target=other)
    t.start()
    t.join()
    assert seen["code"] == 0
    assert capi.last_error()[0] == 2048
    lib.zg_clear_last_error()
    assert capi.last_error() == (0, "")


def test_version(lib):
    a, b, c = C.c_uint(), C.c_uint(), C.c_uint()
    lib.zg_get_version_info(C.byref(a), C.byref(b), C.byref(c))
    assert (a.value, b.value) == (1, 0)


def test_depth_create_errors(lib):
    """zg_depth_create rejects what zimg's DepthConversion rejects, with zimg's
    codes, before touching a device."""
    import ctypes as C
    from zimg_gb300 import capi

    def create(tin, din, tout, dout, dither=0, fin=0, fout=0, w=64, h=32):
        p = capi.DepthParams(w, h, capi.PixelFormat(tin, din, fin, 0, 0), capi.PixelFormat(tout, dout, fout, 0, 0),
                             dither, 0)
        out = C.c_void_p()
        return lib.zg_depth_create(C.byref(p), C.byref(out))

    assert create(2, 17, 0, 8) == 1028            # HALF deeper than 16 bits: BIT_DEPTH_OVERFLOW
    # ERROR_DIFFUSION on a plane whose wavefront fits no shared-memory budget:
    # UNSUPPORTED_OPERATION
    assert create(3, 32, 0, 8, dither=3, w=70000, h=2000) == 3072
    assert create(1, 7, 1, 10) == 1028            # limited range below 8 bits: BIT_DEPTH_OVERFLOW
    assert create(0, 9, 1, 10) == 1028            # depth beyond the type
    assert create(1, 10, 0, 8, dither=9) == 2049  # ENUM_OUT_OF_RANGE
    assert create(5, 10, 0, 8) == 2049
    p = capi.DepthParams(0, 32, capi.PixelFormat(1, 10, 0, 0, 0), capi.PixelFormat(0, 8, 0, 0, 0), 0, 0)
    h = C.c_void_p()
    assert lib.zg_depth_create(C.byref(p), C.byref(h)) == 2050  # INVALID_IMAGE_SIZE


def test_colorspace_create_errors(lib):
    """zg_colorspace_create maps zimg's API codes as zimg.cpp:114-123,238-305
    does and finds zimg's paths, failing with zimg's codes before touching a
    device."""
    import ctypes as C
    from zimg_gb300 import capi

    def create(cin, cout):
        p = capi.ColorspaceParams(16, 16, *cin, *cout, math.nan, 0, 0, 0)
        h = C.c_void_p()
        return lib.zg_colorspace_create(C.byref(p), C.byref(h))

    assert create((1, 1, 1), (0, 300, 1)) == 2049   # outside 0..255: ENUM_OUT_OF_RANGE
    assert create((11, 1, 1), (0, 1, 1)) == 3074    # ST 2085 YDZDX: not mapped, NO_COLORSPACE_CONVERSION
    assert create((1, 1, 1), (2, 2, 2)) == 3074     # no path to an unspecified colorspace
    assert create((10, 16, 9), (0, 1, 1)) == 3074   # BT.2020 CL needs BT.709 transfer (invalid)
    assert create((14, 1, 9), (0, 1, 1)) == 3074    # ICtCp needs PQ or HLG


def test_unresize_create_errors(lib):
    """zg_unresize_create refuses an upscale, as zimg's context builder does
    (bilinear.cpp:109-110), before touching a device."""
    import ctypes as C
    from zimg_gb300 import capi
    h = C.c_void_p()
    p = capi.UnresizeParams(64, 48, 96, 24, 0.0, 0.0)
    assert lib.zg_unresize_create(C.byref(p), C.byref(h)) == 3076  # RESAMPLING_NOT_AVAILABLE
    p = capi.UnresizeParams(64, 48, 0, 24, 0.0, 0.0)
    assert lib.zg_unresize_create(C.byref(p), C.byref(h)) == 2050  # INVALID_IMAGE_SIZE


def test_wide_forms_used_starts_empty(lib):
    """zg_wide_forms_used is per host thread: a thread that enqueued no wide
    pass reads 0, with or without reset."""
    import threading
    out = []
    t = threading.Thread(target=lambda: out.extend([lib.zg_wide_forms_used(0), lib.zg_wide_forms_used(1)]))
    t.start()
    t.join()
    assert out == [0, 0]
