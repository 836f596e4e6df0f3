"""The C-ABI library: it loads, exports every function include/malevich.h declares, and rejects
bad arguments with status codes (no GPU needed for these calls)."""
import ctypes
import os
import re

import pytest

from malevich_gb300 import api, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return api.load_library()


def declared_functions():
    src = open(os.path.join(ROOT, "include", "malevich.h")).read()
    return sorted(set(re.findall(r"MLV_API\s+[\w\s\*]+?\b(mlv_\w+)\s*\(", src)))


def test_header_and_python_agree():
    assert sorted(api.EXPORTS) == declared_functions()


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_abi_version(lib):
    # 2: mlv_rasterizer_desc gained fill_rule and sample_position
    assert lib.mlv_get_abi_version() == 5


def test_null_handles_are_rejected(lib):
    assert lib.mlv_create_device(0, None) == 1
    assert lib.mlv_destroy_device(None) == 1
    assert lib.mlv_create_buffer(None, None, None, None) == 1
    assert lib.mlv_draw_indexed(None, 3, 0, 0) == 1
    assert lib.mlv_finish(None) == 1
    assert b"NULL" in lib.mlv_get_last_error_string() or len(lib.mlv_get_last_error_string()) > 0


def test_no_device_reports_device_error(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    assert lib.mlv_create_device(0, ctypes.byref(h)) == 4


def _struct_fields(name):
    """Field names of a `typedef struct name {...} name;` in the header, in order."""
    src = open(os.path.join(ROOT, "include", "malevich.h")).read()
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), src, re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    names = []
    for decl in body.split(";"):
        decl = decl.strip()
        if decl:
            names += [n.strip().split("[")[0] for n in decl.split(None, 1)[1].split(",")]
    return names


@pytest.mark.parametrize("cname,pytype", [("mlv_tuning", "Tuning"), ("mlv_stats", "Stats"),
                                          ("mlv_rasterizer_desc", "RasterizerDesc")])
def test_python_structs_mirror_the_header(cname, pytype):
    cls = getattr(api, pytype, None)
    if cls is None:
        pytest.skip("%s has no ctypes mirror" % cname)
    assert [n for n, _ in cls._fields_] == _struct_fields(cname)
