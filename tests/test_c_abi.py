"""The C ABI from C: a program compiled against include/rusterize_gb300.h and
linked to librusterize_gb300.so (as a Rust, Go or C caller would bind it)
parses WKT, builds the raster grid, and creates a context.  Without a GPU
the context call must fail with RZ_NO_DEVICE and a message (CPU test); with
one, the program burns the geometry with rz_rasterize and with
rz_rasterize_rows from host buffers and prints both rasters, which must
equal the oracle's (GPU test)."""

import shutil
import subprocess

import pytest

from rusterize_gb300 import _lib

PROGRAM = r"""
#include <stdio.h>
#include <string.h>
#include "rusterize_gb300.h"

int main(void) {
  char err[512];
  if (rz_abi_version() != RZ_ABI_VERSION) return 10;
  if (rz_dtype_size(RZ_F64) != 8 || rz_dtype_size(RZ_U8) != 1) return 11;
  rz_pixel_fn fn;
  if (rz_pixel_fn_from_str("count", &fn, err, sizeof err) != RZ_OK || fn != RZ_COUNT) return 12;
  if (rz_pixel_fn_from_str("median", &fn, err, sizeof err) != RZ_VALUE_ERROR) return 13;

  const char* wkt[2] = {"POLYGON ((0 0, 10 0, 10 5, 0 5, 0 0))", "POINT (2.5 7.5)"};
  size_t lens[2] = {strlen(wkt[0]), strlen(wkt[1])};
  rz_geom_buffer* buf = NULL;
  if (rz_parse_wkt(wkt, lens, 2, &buf, err, sizeof err) != RZ_OK) return 14;
  rz_geoms g;
  if (rz_geom_buffer_view(buf, &g) != RZ_OK) return 15;
  if (g.n_geoms != 2 || g.n_parts != 2 || g.n_vertices != 6) return 16;

  double res[2] = {1.0, 1.0};
  rz_raster_info info;
  if (rz_raster_info_build(&g, RZ_RI_RES, NULL, res, NULL, -1, &info, err, sizeof err) != RZ_OK) return 17;
  printf("grid %llu %llu %.3f %.3f %.3f %.3f\n", (unsigned long long)info.nrows, (unsigned long long)info.ncols,
         info.xmin, info.ymin, info.xmax, info.ymax);

  rz_context* ctx = NULL;
  rz_status st = rz_context_create(0, &ctx, err, sizeof err);
  if (st == RZ_OK) {
    printf("context ok\n");
    /* sum of per-geometry values (u8) with background 0 */
    unsigned char vals[2] = {3, 5}, bg = 0;
    unsigned char out[9 * 11], rows[4 * 11];
    rz_stats stats;
    if (info.nrows != 9 || info.ncols != 11) return 18;
    if (rz_rasterize(ctx, &g, vals, &bg, NULL, 1, &info, RZ_SUM, RZ_U8, 0, out, &stats, err, sizeof err) != RZ_OK) {
      printf("rasterize failed: %s\n", err);
      return 19;
    }
    if (rz_rasterize_rows(ctx, &g, vals, &bg, NULL, 1, &info, 3, 7, RZ_SUM, RZ_U8, 0, rows, &stats, err,
                          sizeof err) != RZ_OK) {
      printf("rasterize_rows failed: %s\n", err);
      return 20;
    }
    printf("raster");
    for (int i = 0; i < 9 * 11; ++i) printf(" %d", out[i]);
    printf("\nrows");
    for (int i = 0; i < 4 * 11; ++i) printf(" %d", rows[i]);
    printf("\n");
    rz_context_destroy(ctx);
  } else {
    printf("context %d %s\n", (int)st, err);
  }
  rz_geom_buffer_free(buf);
  return 0;
}
"""


def _run_program(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    from rusterize_gb300 import _build

    _lib.load()  # builds the library if needed
    so = _build.lib_path()
    src = tmp_path / "use_abi.c"
    exe = tmp_path / "use_abi"
    src.write_text(PROGRAM)
    subprocess.run([cc, "-std=c11", "-I", str(so.parents[2] / "include"), str(src), "-o", str(exe), str(so),
                    f"-Wl,-rpath,{so.parent}"], check=True)
    res = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, (res.returncode, res.stdout, res.stderr)
    return res.stdout.splitlines()


def test_c_program_uses_the_abi(tmp_path):
    import rusterize_gb300 as rz
    from rusterize_gb300 import geometry as G

    lines = _run_program(tmp_path)
    # the grid the builder infers from C equals the one the Python front end gets
    t = G.from_wkt(["POLYGON ((0 0, 10 0, 10 5, 0 5, 0 0))", "POINT (2.5 7.5)"])
    i = rz.raster_info(t, res=(1.0, 1.0))
    assert lines[0] == f"grid {i.nrows} {i.ncols} {i.xmin:.3f} {i.ymin:.3f} {i.xmax:.3f} {i.ymax:.3f}"
    assert lines[0] == "grid 9 11 -0.500 -0.500 10.500 8.000"
    if lines[1] != "context ok":  # no GPU here: the engine refuses, with its message
        assert lines[1].startswith(f"context {_lib.RZ_NO_DEVICE} ")
        assert "no CPU fallback" in lines[1]


@pytest.mark.gpu
def test_c_program_burns_through_the_abi(tmp_path):
    import numpy as np

    import rusterize_gb300 as rz
    from rusterize_gb300 import geometry as G

    from _util import oracle_burn

    lines = _run_program(tmp_path)
    assert lines[1] == "context ok", lines
    t = G.from_wkt(["POLYGON ((0 0, 10 0, 10 5, 0 5, 0 0))", "POINT (2.5 7.5)"])
    info = rz.raster_info(t, res=(1.0, 1.0))
    ref = oracle_burn(t, info, fn="sum", values=np.array([3, 5], np.uint8), background=0, dtype="uint8")[0]
    got = np.array([int(v) for v in lines[2].split()[1:]], np.uint8).reshape(9, 11)
    rows = np.array([int(v) for v in lines[3].split()[1:]], np.uint8).reshape(4, 11)
    assert np.array_equal(got, ref)
    assert np.array_equal(rows, ref[3:7])
    assert got.sum() > 0
