"""A C caller, as the reference's own code would be one: include/malevich.h compiles as plain C99
with warnings as errors, a program links libmalevich_gb300.so and calls the ABI (only calls that
need no GPU: version, argument checks, error strings)."""
import os
import shutil
import subprocess

import pytest

from malevich_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <stdio.h>
#include <string.h>
#include "malevich.h"

int main(void) {
    mlv_device dev = NULL;
    mlv_tuning tuning;
    mlv_viewport vp = {0.0f, 0.0f, 64.0f, 64.0f, 0.0f, 1.0f};
    (void)vp;
    memset(&tuning, 0, sizeof(tuning));
    if (mlv_get_abi_version() != MLV_ABI_VERSION) return 10;
    if (mlv_create_device(0, NULL) != MLV_ERROR_INVALID_ARG) return 11;
    if (mlv_draw_indexed(NULL, 3, 0, 0) != MLV_ERROR_INVALID_ARG) return 12;
    if (mlv_set_tuning(NULL, &tuning) != MLV_ERROR_INVALID_ARG) return 13;
    if (strlen(mlv_get_last_error_string()) == 0) return 14;
    (void)dev;
    printf("abi %d ok\n", mlv_get_abi_version());
    return 0;
}
"""


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_header_compiles_as_c99_and_the_library_links(tmp_path):
    so = build.build()
    libdir = os.path.dirname(so) if isinstance(so, str) and so.endswith(".so") else os.path.join(ROOT, "malevich_gb300")
    src = tmp_path / "caller.c"
    src.write_text(PROGRAM)
    exe = tmp_path / "caller"
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", os.path.join(ROOT, "include"),
                    str(src), "-o", str(exe), "-L", libdir, "-lmalevich_gb300", "-Wl,-rpath," + libdir],
                   check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, (out.returncode, out.stdout, out.stderr)
    assert "ok" in out.stdout
