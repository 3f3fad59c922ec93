"""A C host program against the C ABI: it must compile as C99 against
include/gbh.h and link against libgbh.so.  Run without a GPU, gbh_create
fails and gbh_last_error(NULL) says why; with a GPU it steps and exits 0."""
import os
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_DIR = os.path.join(ROOT, "gravity_gb300")

PROGRAM = r"""
#include <stdio.h>
#include <stdlib.h>
#include "gbh.h"
int main(void) {
    const uint32_t n = 1024;
    gbh_body* bodies = calloc(n, sizeof(gbh_body));
    for (uint32_t i = 0; i < n; ++i) {
        bodies[i].pos_mass[0] = (float)i / n - 0.5f;
        bodies[i].pos_mass[1] = (float)((i * 37u) % n) / n - 0.5f;
        bodies[i].pos_mass[3] = 1.0f / n;
        bodies[i].vel_density[3] = 1.0f;
    }
    gbh_ctx* ctx;
    gbh_units u = {1, 1, 1, 1, 10, 1.0f};
    float bounds[6] = {-1, -1, -1, 1, 1, 1};
    if (gbh_create(&ctx, n, bounds, &u, 0) != GBH_OK) {
        printf("create failed: %s\n", gbh_last_error(NULL));
        free(bodies);
        return 1;
    }
    int rc = gbh_upload_bodies(ctx, bodies, n, 0);
    if (!rc) rc = gbh_init(ctx);
    gbh_step_params p = {.dt = 1e-3f, .theta = 0.5f, .softening = 1e-4f, .restitution = 0.2f,
                         .static_or_dynamic = GBH_BOUNDS_DYNAMIC};
    for (int s = 0; s < 10 && !rc; ++s) rc = gbh_step(ctx, &p);
    if (!rc) rc = gbh_read_bodies(ctx, GBH_BODIES_IN, bodies, n, 0);
    if (rc) printf("failed: %s\n", gbh_last_error(ctx));
    gbh_destroy(ctx);
    free(bodies);
    return rc ? 2 : 0;
}
"""


def test_c_host_compiles_links_and_reports_errors(gbh_lib):
    lib = os.path.join(LIB_DIR, "libgbh.so")
    if not os.path.exists(lib):
        pytest.skip("libgbh.so not built")
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "host.c"), os.path.join(d, "host")
        open(src, "w").write(PROGRAM)
        subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), src, "-L", LIB_DIR,
                        "-lgbh", f"-Wl,-rpath,{LIB_DIR}", "-o", exe], check=True)
        r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    if r.returncode == 1:
        # no usable GPU: the failure is reported through gbh_last_error(NULL)
        assert r.stdout.startswith("create failed: ") and len(r.stdout.strip()) > len("create failed:")
    else:
        assert r.returncode == 0, r.stdout
