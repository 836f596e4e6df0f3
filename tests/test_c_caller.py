"""A C caller, as the reference's own code would be one: include/malevich.h compiles as plain C99
with warnings as errors, a program links libmalevich_gb300.so and calls the ABI (on the CPU only
the calls that need no GPU: version, argument checks, error strings), and on the GPU a C program
replays the reference's render() on its Suprematism input and matches the reference's output."""
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


RENDER = r"""
/* The reference's render() (main.c:1265-1299) for one object, written against the C ABI: create a
   device, upload the inputs, clear, set the pipeline state, draw, read back. Inputs and outputs go
   through two binary files so that the test can compare the result with the reference's own. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "malevich.h"

#define CHECK(call) do { mlv_status s_ = (call); if (s_ != MLV_OK) { \
    fprintf(stderr, "%s: %d %s\n", #call, (int)s_, mlv_get_last_error_string()); return 20; } } while (0)

int main(int argc, char **argv) {
    uint32_t head[4];        /* width, height, vertex count, index count */
    float clear[5], vpf[6];  /* clear colour + depth, viewport */
    float *vb; uint32_t *ib, *color; float *depth;
    FILE *f;
    mlv_device dev; mlv_context ctx;
    mlv_buffer vbuf, ibuf;
    mlv_texture2d rt, ds;
    mlv_buffer_desc bd;
    mlv_texture2d_desc td;
    mlv_viewport vp;
    mlv_stats st;
    uint32_t stride = 32, offset = 0;
    if (argc != 3) return 2;
    f = fopen(argv[1], "rb");
    if (!f || fread(head, 4, 4, f) != 4 || fread(clear, 4, 5, f) != 5 || fread(vpf, 4, 6, f) != 6) return 3;
    vb = (float *)malloc((size_t)head[2] * 32);
    ib = (uint32_t *)malloc((size_t)head[3] * 4);
    color = (uint32_t *)malloc((size_t)head[0] * head[1] * 4);
    depth = (float *)malloc((size_t)head[0] * head[1] * 4);
    if (fread(vb, 32, head[2], f) != head[2] || fread(ib, 4, head[3], f) != head[3]) return 4;
    fclose(f);

    CHECK(mlv_create_device(0, &dev));
    CHECK(mlv_get_immediate_context(dev, &ctx));
    bd.byte_width = (uint64_t)head[2] * 32; bd.bind_flags = MLV_BIND_VERTEX_BUFFER; bd.reserved = 0;
    CHECK(mlv_create_buffer(dev, &bd, vb, &vbuf));
    bd.byte_width = (uint64_t)head[3] * 4; bd.bind_flags = MLV_BIND_INDEX_BUFFER;
    CHECK(mlv_create_buffer(dev, &bd, ib, &ibuf));
    td.width = head[0]; td.height = head[1]; td.format = MLV_FORMAT_R8G8B8A8_UNORM; td.bind_flags = MLV_BIND_RENDER_TARGET;
    CHECK(mlv_create_texture2d(dev, &td, NULL, 0, &rt));
    td.format = MLV_FORMAT_D32_FLOAT; td.bind_flags = MLV_BIND_DEPTH_STENCIL;
    CHECK(mlv_create_texture2d(dev, &td, NULL, 0, &ds));
    {
        /* the same inputs once more as one grouped upload (no reference counterpart): one block,
           the index buffer at a 16-byte aligned offset; the image must not change */
        const uint64_t vb_bytes = (uint64_t)head[2] * 32, ib_at = (vb_bytes + 15) / 16 * 16;
        const uint64_t ib_bytes = (uint64_t)head[3] * 4;
        unsigned char *block = (unsigned char *)calloc(1, (size_t)(ib_at + ib_bytes));
        mlv_upload ups[2];
        memcpy(block, vb, (size_t)vb_bytes);
        memcpy(block + ib_at, ib, (size_t)ib_bytes);
        memset(ups, 0, sizeof(ups));
        ups[0].kind = MLV_UPLOAD_BUFFER; ups[0].resource = vbuf; ups[0].src_offset = 0; ups[0].size = vb_bytes;
        ups[1].kind = MLV_UPLOAD_BUFFER; ups[1].resource = ibuf; ups[1].src_offset = ib_at; ups[1].size = ib_bytes;
        CHECK(mlv_update_resources_async(ctx, block, ib_at + ib_bytes, ups, 2));
        CHECK(mlv_finish(ctx));
        free(block);
    }

    /* render(): clear, viewport, targets, shaders, buffers, draw_indexed (main.c:1268-1296) */
    CHECK(mlv_reset_stats(ctx));
    CHECK(mlv_clear_render_target_view(ctx, rt, clear));
    CHECK(mlv_clear_depth_stencil_view(ctx, ds, clear[4]));
    vp.top_left_x = vpf[0]; vp.top_left_y = vpf[1]; vp.width = vpf[2]; vp.height = vpf[3];
    vp.min_depth = vpf[4]; vp.max_depth = vpf[5];
    CHECK(mlv_rs_set_viewports(ctx, 1, &vp));
    CHECK(mlv_om_set_render_targets(ctx, rt, ds));
    CHECK(mlv_ia_set_primitive_topology(ctx, MLV_PRIMITIVE_TOPOLOGY_TRIANGLELIST));
    CHECK(mlv_ia_set_vertex_buffers(ctx, 0, 1, &vbuf, &stride, &offset));
    CHECK(mlv_ia_set_index_buffer(ctx, ibuf, MLV_FORMAT_R32_UINT, 0));
    CHECK(mlv_vs_set_shader(ctx, MLV_VS_PASSTHROUGH));
    CHECK(mlv_ps_set_shader(ctx, MLV_PS_PASSTHROUGH));
    CHECK(mlv_draw_indexed(ctx, head[3], 0, 0));
    CHECK(mlv_read_texture2d(ctx, rt, color, 0));
    CHECK(mlv_read_texture2d(ctx, ds, depth, 0));
    CHECK(mlv_get_stats(ctx, &st));

    f = fopen(argv[2], "wb");
    if (!f) return 5;
    fwrite(color, 4, (size_t)head[0] * head[1], f);
    fwrite(depth, 4, (size_t)head[0] * head[1], f);
    fwrite(&st, sizeof(st), 1, f);
    fclose(f);
    CHECK(mlv_destroy_texture2d(rt));
    CHECK(mlv_destroy_texture2d(ds));
    CHECK(mlv_destroy_buffer(vbuf));
    CHECK(mlv_destroy_buffer(ibuf));
    CHECK(mlv_destroy_device(dev));
    free(vb); free(ib); free(color); free(depth);
    printf("render ok\n");
    return 0;
}
"""


@pytest.mark.gpu
@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_c_program_renders_the_suprematism_frame_like_the_reference(tmp_path):
    """A C program replays the reference's render() on its own fixed Suprematism input
    (main.c:232-254) through the C ABI on the GPU; colour, depth and Stats must equal the
    reference's outputs in the golden fixture bit for bit."""
    import numpy as np
    so = build.build()
    libdir = os.path.dirname(so) if isinstance(so, str) and so.endswith(".so") else os.path.join(ROOT, "malevich_gb300")
    z = np.load(os.path.join(ROOT, "tests", "golden", "suprematism.npz"))
    w, h = (int(v) for v in z["frame/size"])
    vb = np.ascontiguousarray(z["frame/draw0/vb"], np.float32)
    ib = np.ascontiguousarray(z["frame/draw0/ib"], np.uint32)
    n = int(z["frame/draw0/ints"][2])
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        f.write(np.array([w, h, len(vb), n], np.uint32).tobytes())
        f.write(np.concatenate([z["frame/clear_color"], z["frame/clear_depth"]]).astype(np.float32).tobytes())
        f.write(np.asarray(z["frame/draw0/viewport"], np.float32).tobytes())
        f.write(vb.tobytes())
        f.write(ib[:n].tobytes())
    src = tmp_path / "render.c"
    src.write_text(RENDER)
    exe = tmp_path / "render"
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", os.path.join(ROOT, "include"),
                    str(src), "-o", str(exe), "-L", libdir, "-lmalevich_gb300", "-Wl,-rpath," + libdir],
                   check=True, capture_output=True, text=True)
    out_path = tmp_path / "out.bin"
    out = subprocess.run([str(exe), str(inp), str(out_path)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, (out.returncode, out.stdout, out.stderr)
    raw = out_path.read_bytes()
    color = np.frombuffer(raw[:w * h * 4], np.uint32).reshape(h, w)
    depth = np.frombuffer(raw[w * h * 4:w * h * 8], np.float32).reshape(h, w)
    stats = np.frombuffer(raw[w * h * 8:w * h * 8 + 64], np.uint64)
    assert np.array_equal(color, z["out/color"]), "colour differs from the reference's"
    assert np.array_equal(depth.view(np.uint32), z["out/depth"].view(np.uint32)), "depth differs from the reference's"
    assert list(stats[:5]) == list(z["out/stats"]), (stats[:5], z["out/stats"])
