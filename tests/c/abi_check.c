/* A plain C99 host of include/vct.h: compiled with -std=c99 -pedantic
 * -Werror and linked against libvct.so by tests/test_c_abi.py.  It uses
 * only the calls that need no GPU, and exits non-zero on any mismatch. */
#include <stdio.h>
#include <string.h>

#include "vct.h"

static int failures = 0;
#define CHECK(cond)                                             \
    do {                                                        \
        if (!(cond)) {                                          \
            fprintf(stderr, "check failed: %s\n", #cond);       \
            ++failures;                                         \
        }                                                       \
    } while (0)

int main(void) {
    vct_params p;
    vct_tuning t;
    vct_config cfg;
    vct_ctx* ctx = NULL;
    vct_triangles tris;
    float mvp[48];

    CHECK(vct_abi_version() == VCT_ABI_VERSION);
    CHECK(strcmp(vct_status_string(VCT_OK), "ok") == 0);

    /* the struct layouts a C compiler sees are the library's */
    CHECK(vct_struct_layout("vct_params") == (int64_t)sizeof(vct_params));
    CHECK(vct_struct_layout("vct_light") == (int64_t)sizeof(vct_light));
    CHECK(sizeof(vct_light) == 80); /* the reference's std140 light record */
    CHECK(vct_struct_layout("vct_config") == (int64_t)sizeof(vct_config));
    CHECK(vct_struct_layout("vct_tuning") == (int64_t)sizeof(vct_tuning));
    CHECK(vct_struct_layout("vct_scene_desc") == (int64_t)sizeof(vct_scene_desc));
    CHECK(vct_struct_layout("vct_params.pv") == (int64_t)offsetof(vct_params, pv));
    CHECK(vct_struct_layout("no_such_struct") == -1);

    /* reference defaults (src/Application.h:36-103) */
    vct_default_params(&p);
    CHECK(p.voxelize_lighting == 1 && p.axis_override == -1);
    CHECK(p.voxel_set_opacity == 0.5f && p.temporal_decay == 0.8f);
    CHECK(p.diffuse_cone.steps == 16 && p.specular_cone.steps == 32);
    CHECK(p.warp_mode == VCT_WARP_NONE && p.trace_filter == VCT_FILTER_SOFTWARE);
    CHECK(p.max_tess_level == (float)VCT_MAX_TESS_LEVEL && p.pv[0] == 1.0f && p.pv[1] == 0.0f);
    vct_default_tuning(&t);
    CHECK(t.voxel_unit_pixels == 512 && t.voxel_blocks_per_sm == 3);

    /* arguments are validated before any device work */
    memset(&cfg, 0, sizeof cfg);
    cfg.voxel_dim = 48; /* not a power of two */
    cfg.voxel_min[0] = cfg.voxel_min[1] = cfg.voxel_min[2] = -1.0f;
    cfg.voxel_max[0] = cfg.voxel_max[1] = cfg.voxel_max[2] = 1.0f;
    CHECK(vct_create(&cfg, &ctx) == VCT_ERR_INVALID_ARGUMENT && ctx == NULL);
    CHECK(strstr(vct_last_error(), "power of two") != NULL);
    CHECK(vct_create(NULL, &ctx) == VCT_ERR_INVALID_ARGUMENT);
    CHECK(vct_destroy(NULL) == VCT_OK);
    cfg.voxel_dim = 64;
    CHECK(vct_voxel_mvp(&cfg, mvp) == VCT_OK);
    CHECK(mvp[15] == 1.0f);
    memset(&tris, 0, sizeof tris);
    tris.count = 3; /* non-zero count with NULL arrays */
    CHECK(vct_voxelize_static(&cfg, &p, &tris, NULL, 0, NULL, NULL, NULL, NULL, NULL, NULL) ==
          VCT_ERR_INVALID_ARGUMENT);

    /* accumulator record slots: bit 1 of x and bit 0 of y exchanged */
    CHECK(vct_record_slot(0, 16) == 0);
    CHECK(vct_record_slot(2, 16) == 16);  /* x = 2, y = 0 */
    CHECK(vct_record_slot(16, 16) == 2);  /* x = 0, y = 1 */
    CHECK(vct_record_slot(3, 16) == 17);  /* x = 3, y = 0 */
    CHECK(vct_record_slot(18, 16) == 18); /* x = 2, y = 1 */
    CHECK(vct_record_slot(4096 + 17, 16) == 4096 + 3);

    if (failures == 0) printf("abi_check ok\n");
    return failures == 0 ? 0 : 1;
}
