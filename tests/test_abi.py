"""CPU checks of the C ABI: the library loads (no GPU needed) and exports
every function include/xavs2_gb300.h declares; the drop-in tables have the
reference's layout."""
import ctypes
import os
import re
import subprocess
import tempfile

import pytest

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "xavs2_gb300.h")
REF_SRC = oracle.REF_SRC


@pytest.fixture(scope="module")
def libpath():
    from xavs2_gb300 import build
    try:
        return build.build()
    except (RuntimeError, FileNotFoundError) as e:   # no nvcc on this machine
        pytest.skip("cannot build the CUDA library here: %s" % e)


def declared_functions():
    out = subprocess.run(["gcc", "-E", "-P", "-x", "c", HEADER], capture_output=True, text=True, check=True).stdout
    names = set(re.findall(r"\b(xavs2gpu_\w+)\s*\(", out))
    # typedef'd function pointer types are not exported symbols
    types = set(re.findall(r"\(\s*\*\s*(xavs2gpu_\w+)\s*\)", out))
    return sorted(names - types)


def test_header_compiles_as_c():
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "t.c")
        with open(src, "w") as f:
            f.write('#include "xavs2_gb300.h"\nint main(void){return XAVS2GPU_NUM_PU_SIZES == 25 ? 0 : 1;}\n')
        subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I" + os.path.dirname(HEADER), src, "-o",
                        os.path.join(d, "t")], check=True)
        assert subprocess.run([os.path.join(d, "t")]).returncode == 0


def test_library_exports_all_declared(libpath):
    names = declared_functions()
    assert len(names) > 400
    lib = ctypes.CDLL(libpath)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing[:10]


def test_no_fallback_without_gpu(libpath):
    """Without a GPU the library reports an error instead of computing on the CPU."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    lib = ctypes.CDLL(libpath)
    lib.xavs2gpu_set_abort_on_error(0)
    lib.xavs2gpu_init.restype = ctypes.c_int
    assert lib.xavs2gpu_init(0) != 0
    lib.xavs2gpu_get_error.restype = ctypes.c_char_p
    assert lib.xavs2gpu_get_error()


@pytest.mark.skipif(not os.path.isdir(REF_SRC), reason="reference sources not present")
def test_table_layout_matches_reference():
    """xavs2gpu_pixel_funcs_t / xavs2gpu_dct_funcs_t have the member offsets of
    the reference's pixel_funcs_t / dct_funcs_t (pixel.h:141-166,
    primitives.h:101-119), so xavs2gpu_*_init can fill the encoder's tables."""
    members_pix = ["sad", "satd", "sa8d", "ssd", "sad_x3", "sad_x4", "sub_ps", "add_ps", "copy_sp", "copy_ps",
                   "copy_ss", "copy_pp", "avg", "intra_cmp", "fpel_cmp", "madf", "ssd_block", "average"]
    members_dct = ["dct", "idct", "dct_half", "transform_4x4_2nd", "inv_transform_4x4_2nd", "transform_2nd",
                   "inv_transform_2nd", "abs_coeff", "add_sign", "quant", "dequant", "wquant"]
    checks = ["sizeof(pixel_funcs_t) == sizeof(xavs2gpu_pixel_funcs_t)",
              "sizeof(dct_funcs_t) == sizeof(xavs2gpu_dct_funcs_t)"]
    checks += ["offsetof(pixel_funcs_t, %s) == offsetof(xavs2gpu_pixel_funcs_t, %s)" % (m, m) for m in members_pix]
    checks += ["offsetof(dct_funcs_t, %s) == offsetof(xavs2gpu_dct_funcs_t, %s)" % (m, m) for m in members_dct]
    body = "\n".join('    if (!(%s)) { printf("%%s\\n", "%s"); bad++; }' % (c, c) for c in checks)
    code = ('#include <stdio.h>\n#include <stddef.h>\n#include "common.h"\n#include "primitives.h"\n'
            '#include "xavs2_gb300.h"\nint main(void){int bad=0;\n%s\nreturn bad;}\n' % body)
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "layout.c")
        with open(src, "w") as f:
            f.write(code)
        exe = os.path.join(d, "layout")
        subprocess.run(["gcc", "-w", "-I" + os.path.join(ROOT, "oracle", "ref_shim"), "-I" + REF_SRC,
                        "-I" + os.path.join(REF_SRC, "common"), "-I" + os.path.dirname(HEADER), src, "-o", exe],
                       check=True)
        r = subprocess.run([exe], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout
