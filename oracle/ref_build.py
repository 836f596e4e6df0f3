"""Build the reference's own draw path as a headless shared library (test infrastructure only).

The reference (OzgurCerlet/Malevich) is a Win32 program; its pipeline core is plain C with AVX2 and
OpenMP: `source/main.c:1-282` (types, globals) and `source/main.c:561-1261` (the stages and
`draw_indexed`), plus `source/math.h`, `source/common_shader_core.h` and the seven shader files.
This recipe copies exactly those sources from the reference tree into `oracle/_ref/src/`, applies
the mechanical patches listed below, and compiles one `libmalevich_ref_<W>x<H>.so` per render-target
size (the reference fixes WIDTH/HEIGHT at compile time, `source/main.c:21-22`).

Mechanical patches (none changes a computed value):
  1. Drop the Win32, Remotery and octarine includes and `#pragma comment(lib, ...)` lines
     (`main.c:3-4,12-19`); a generated shim header supplies HWND/UINT and no-op Remotery macros.
  2. WIDTH/HEIGHT become overridable (`main.c:21-22`).
  3. MSVC vector members `.m256_f32[i]` (`main.c:715-726`) and `.m256i_i32[i]`
     (`common_shader_core.h:174`) become pointer casts.
  4. The PS function-pointer prototype (`main.c:99`) gains the fourth `i256 mask` argument that
     its call site passes (`main.c:1172`) and every pixel shader takes.
     The implicit-int declarations `const fragment_linear_coordinate` (`main.c:582,596`) get `i32`.
  5. The per-bin tile arrays (`main.c:1055-1056`) get 32-byte alignment: `_mm256_load_ps` at
     `main.c:1165` requires it, and gcc does not align a plain stack array that way (the
     unaligned load faults). For the same reason the shim routes the core's `malloc` to a
     32-byte aligned allocator: the stage buffers are read and written through `f256` pointers
     (`main.c:676-691,709-712`), which gcc accesses with aligned vector moves.
  6. `inline` becomes `static inline` after the system includes of `math.h` (C99 inline semantics
     would otherwise leave undefined symbols); `__cdecl` is defined away; `max`/`min` macros added.
  7. SVML `_mm256_acos_ps/_exp_ps/_pow_ps` (`math.h:21-23`) are linked from `ref_svml_shim.c`,
     which applies libm `acosf/expf/powf` per lane (SVML itself is closed and absent).
  8. Additive instrumentation hooks (macros defined by `ref_harness.c`): capture the assembled
     triangles and the per-(bin, triangle) TileInfo masks before they are freed
     (`main.c:1255-1258`), and record the triangle id next to every masked colour store
     (`main.c:1180`) so the harness can return a triangle-ID buffer.
Built with `-O3 -mavx2 -mfma -fopenmp -ffp-contract=off -fwrapv`. x86-64 only: the core is AVX2.

Usage: python oracle/ref_build.py [--reference DIR] [--sizes 1280x720,1920x1080]
"""
import argparse
import os
import re
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
# Where this recipe looks for the reference's sources: $MALEVICH_REFERENCE, else the checkout this
# build container mounts. The only place the product's files name that location.
DEFAULT_REFERENCE = "/root/reference"


def reference_dir():
    """The reference checkout this recipe builds from, or None when its sources are absent (as on
    a host that only runs the prebuilt files)."""
    d = os.environ.get("MALEVICH_REFERENCE", DEFAULT_REFERENCE)
    return d if os.path.isdir(os.path.join(d, "source")) else None
DEFAULT_SIZES = ["1280x720", "1920x1080", "1200x720", "480x272", "256x256", "512x512", "64x64", "32x32"]
SHADERS = ["basic_vs.c", "vertex_lighting_vs.c", "passthrough_vs.c", "fullscreen_vs.c",
           "basic_ps.c", "passthrough_ps.c", "env_lighting_ps.c"]

SHIM = r"""#pragma once
/* Generated by oracle/ref_build.py: stand-ins for the Win32 and Remotery names that the kept part
   of the reference's main.c still mentions. */
#include <stdlib.h>
#include <string.h>
typedef void *HWND;
typedef unsigned int UINT;
/* 32-byte aligned heap blocks: the stage buffers are accessed through __m256 pointers */
static inline void *ref_malloc32(size_t n) {
    void *p = NULL;
    if (posix_memalign(&p, 64, n ? n : 64)) return NULL;
    return p;
}
#define malloc(n) ref_malloc32(n)
#define rmt_BeginCPUSample(name, flags)
#define rmt_EndCPUSample()
#ifndef REF_HOOK_TRIANGLES
#define REF_HOOK_TRIANGLES(tris, n, attrs)
#define REF_HOOK_TILE_INFOS(infos, n, bins, nbins, ids)
#define REF_HOOK_READ_IDS(bin_index, ids)
#define REF_HOOK_STORE_ID(ids_row, mask, tri_id)
#define REF_HOOK_WRITE_IDS(bin_index, ids)
#endif
"""


def _sub_once(text, old, new, what):
    if old not in text:
        raise RuntimeError("reference source changed: cannot find " + what)
    return text.replace(old, new, 1)


def patch_main(src):
    lines = src.splitlines(keepends=True)
    head = "".join(lines[0:282])          # main.c:1-282  types and globals
    core = "".join(lines[560:1261])       # main.c:561-1261 pipeline stages
    head = _sub_once(head, "#include <windows.h>", '#include "win_shim.h"', "windows.h include")
    head = _sub_once(head, '#include "external/Remotery/Remotery.h"', "", "Remotery include")
    head = _sub_once(head, '#include "external/octarine/octarine_mesh.h"', "", "octarine mesh include")
    head = _sub_once(head, '#include "external/octarine/octarine_image.h"', "", "octarine image include")
    head = re.sub(r'#pragma comment\(lib, "[^"]*"\)', "", head)
    head = re.sub(r"#define WIDTH\s+1200[^\n]*", "#ifndef WIDTH\n#define WIDTH 1200\n#endif", head)
    head = re.sub(r"#define HEIGHT\s+720[^\n]*", "#ifndef HEIGHT\n#define HEIGHT 720\n#endif", head)
    head = _sub_once(head, "void *p_pixel_output_data, const void *p_shader_resource_views);",
                     "void *p_pixel_output_data, const void *p_shader_resource_views, i256 mask);",
                     "PS shader prototype")
    core = re.sub(r"(vertex_output\[\d+\])\.m256_f32\[i\]", r"((f32*)&\1)[i]", core)
    core = core.replace("const fragment_linear_coordinate", "const i32 fragment_linear_coordinate")
    core = _sub_once(core, "u32 a_tile_colors[64];\n\t\tf32 a_tile_depths[64];",
                     "__attribute__((aligned(32))) u32 a_tile_colors[64];\n"
                     "\t\t__attribute__((aligned(32))) f32 a_tile_depths[64];", "tile arrays")
    # instrumentation hooks (additive)
    core = _sub_once(core, "read_tile(min_bounds, a_tile_colors, a_tile_depths);",
                     "read_tile(min_bounds, a_tile_colors, a_tile_depths);\n"
                     "\t\tu64 a_tile_ids[64]; REF_HOOK_READ_IDS(bin.bin_index, a_tile_ids);",
                     "read_tile call")
    core = _sub_once(core, "_mm256_maskstore_epi32(a_tile_colors + fragment_y_index * 8, mask, encoded_color);",
                     "_mm256_maskstore_epi32(a_tile_colors + fragment_y_index * 8, mask, encoded_color);\n"
                     "\t\t\t\tREF_HOOK_STORE_ID(a_tile_ids + fragment_y_index * 8, mask, tile_info.triangle_id);",
                     "colour mask store")
    core = _sub_once(core, "write_tile(bin.bin_index, a_tile_colors, a_tile_depths);",
                     "REF_HOOK_WRITE_IDS(bin.bin_index, a_tile_ids);\n"
                     "\t\twrite_tile(bin.bin_index, a_tile_colors, a_tile_depths);",
                     "write_tile call")
    core = _sub_once(core, "\tfree(p_vertex_input_data);",
                     "\tREF_HOOK_TRIANGLES(p_triangles, assembled_triangle_count, p_attributes);\n"
                     "\tREF_HOOK_TILE_INFOS(p_tile_infos, total_triangle_count_in_bins, p_compacted_bins, "
                     "num_compacted_bins, p_triangle_ids);\n"
                     "\tfree(p_vertex_input_data);",
                     "draw_indexed frees")
    return head + "\n" + core


def patch_math(src):
    src = _sub_once(src, "#include <immintrin.h>",
                    "#include <immintrin.h>\n#include <stdlib.h>\n#include <string.h>\n#include <assert.h>\n"
                    "#define inline static inline\n#define __cdecl\n"
                    "#ifndef max\n#define max(a,b) (((a)>(b))?(a):(b))\n#endif\n"
                    "#ifndef min\n#define min(a,b) (((a)<(b))?(a):(b))\n#endif\n",
                    "immintrin include")
    return src


def patch_core_header(src):
    return src.replace("mask.m256i_i32[i]", "((i32*)&mask)[i]")


def prepare_sources(reference):
    srcdir = os.path.join(reference, "source")
    dst = os.path.join(OUT, "src")
    os.makedirs(dst, exist_ok=True)

    def rd(name):
        with open(os.path.join(srcdir, name), "r", encoding="utf-8", errors="replace") as f:
            return f.read()

    def wr(name, text):
        with open(os.path.join(dst, name), "w") as f:
            f.write(text)

    wr("win_shim.h", SHIM)
    wr("main_core.c", patch_main(rd("main.c")))
    wr("math.h", patch_math(rd("math.h")))
    wr("common_shader_core.h", patch_core_header(rd("common_shader_core.h")))
    for s in SHADERS:
        wr(s, rd(s))
    return dst


CFLAGS = ["-O3", "-mavx2", "-mfma", "-fopenmp", "-ffp-contract=off", "-fwrapv", "-std=gnu2x", "-fPIC",
          "-DNDEBUG", "-w", "-Wno-incompatible-pointer-types"]


def compile_size(srcdir, size):
    w, h = size.split("x")
    objdir = os.path.join(OUT, "obj_" + size)
    os.makedirs(objdir, exist_ok=True)
    out = os.path.join(OUT, "libmalevich_ref_%s.so" % size)
    srcs = [os.path.join(srcdir, s) for s in SHADERS]
    srcs += [os.path.join(HERE, "ref_svml_shim.c"), os.path.join(HERE, "ref_harness.c")]
    cmd = ["gcc"] + CFLAGS + ["-DWIDTH=%s" % w, "-DHEIGHT=%s" % h, "-I", srcdir, "-shared", "-o", out] + srcs + ["-lm"]
    subprocess.run(cmd, check=True)
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=reference_dir() or os.environ.get("MALEVICH_REFERENCE", DEFAULT_REFERENCE))
    ap.add_argument("--sizes", default=",".join(DEFAULT_SIZES))
    args = ap.parse_args(argv)
    if not os.path.isdir(os.path.join(args.reference, "source")):
        print("reference sources not found at %s; nothing built" % args.reference, file=sys.stderr)
        return 1
    import platform
    if platform.machine() not in ("x86_64", "AMD64"):
        print("the reference core is AVX2 code: x86-64 only; nothing built", file=sys.stderr)
        return 1
    srcdir = prepare_sources(args.reference)
    sizes = [s for s in args.sizes.split(",") if s]
    with ThreadPoolExecutor(max_workers=min(8, len(sizes))) as ex:
        for out in ex.map(lambda s: compile_size(srcdir, s), sizes):
            print("built", out)
    return 0


if __name__ == "__main__":
    sys.exit(main())
