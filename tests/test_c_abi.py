"""The C ABI from plain C: a C99 program includes include/cctgpu.h, links libcctgpu.so and calls
its host-side entry points (no device needed).  Checks that the header is valid C, that the
exported symbols resolve at link time, and that sizes and argument checks behave as from
Python."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "cctpy_gb300", "lib")

PROGRAM = r"""
#include <stdio.h>
#include <string.h>
#include "cctgpu.h"

int main(void) {
    char msg[256];
    int64_t off[3] = {0, 46080, 46080 + 300};          /* two designs: 360 tiles and 3 tiles */
    int64_t unit_off[3], chunks[2], chunk_tiles[2], bad[3] = {0, 10, 5};
    int32_t group = 0;
    double layer[CCT_LAYER_DOUBLES];
    int64_t units, packed, scratch;
    int rc;

    printf("version %d tile %d\n", cct_version(), cct_f32c_tile());
    packed = cct_f32c_packed_bytes(off, 2);
    printf("packed %lld\n", (long long)packed);
    scratch = cct_track_scratch_bytes(2, 4096);
    printf("scratch_positive %d\n", scratch > 0);
    units = cct_test_plan_units(off, 2, 4096, 1, 456, 0, unit_off, chunks, chunk_tiles, &group);
    printf("plan %lld group %d units_ok %d\n", (long long)units, (int)group, unit_off[2] == units);
    units = cct_test_plan_units(bad, 2, 10, 1, 456, 0, unit_off, chunks, chunk_tiles, &group);
    rc = cct_last_error(msg, sizeof msg);
    printf("bad_offsets %lld status %d decrease %d\n", (long long)units, rc, strstr(msg, "decrease") != NULL);
    memset(layer, 0, sizeof layer);
    layer[19] = 4.0;                                     /* winding number */
    layer[20] = 36.0;                                    /* segments per winding */
    layer[12] = 0.95; layer[13] = 0.083;                 /* big_r, small_r */
    layer[3] = 1.0; layer[7] = 1.0; layer[11] = 1.0;     /* XI, YI, ZI */
    layer[17] = 8.0 * 3.141592653589793;                 /* xi end */
    layer[21] = 0.0;                                     /* no tilt angles */
    printf("layer_segments %lld\n", (long long)cct_layer_segments(layer, 1));
    rc = cct_track_set_units_per_cta(65);
    printf("units_per_cta_65 %d default %d\n", rc, (int)cct_track_units_per_cta());
    return 0;
}
"""


@pytest.fixture(scope="module")
def program(tmp_path_factory):
    if not os.path.exists(os.path.join(LIBDIR, "libcctgpu.so")):
        pytest.skip("libcctgpu.so not built")
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    d = tmp_path_factory.mktemp("cabi")
    src, exe = d / "prog.c", d / "prog"
    src.write_text(PROGRAM)
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), str(src),
                        "-o", str(exe), "-L", LIBDIR, "-lcctgpu", f"-Wl,-rpath,{LIBDIR}"],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_program_calls_host_entry_points(program):
    r = subprocess.run([str(program)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    out = dict(line.split(" ", 1) for line in r.stdout.strip().splitlines())
    assert out["version"].split() == ["100", "tile", "128"]
    assert int(out["packed"]) > 363 * 4704
    assert out["scratch_positive"] == "1"
    plan = out["plan"].split()
    assert int(plan[0]) > 0 and plan[1:] == ["group", "256", "units_ok", "1"]
    assert out["bad_offsets"].split() == ["-2", "status", "1", "decrease", "1"]
    assert int(out["layer_segments"]) == 4 * 36
    assert out["units_per_cta_65"].split() == ["1", "default", "8"]
