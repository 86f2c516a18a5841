/* A plain C99 caller of the C-ABI (include/trax.h), as a cgo or FFI binding
 * would be: host-only calls must work without a GPU, and creating a context
 * must fail with a status and a message, never crash.  Prints one line per
 * check; exits 0 when every check passed. */
#include <stdio.h>
#include <string.h>

#include "trax.h"

static int failures = 0;

static void check(int ok, const char *what)
{
    printf("%s %s\n", ok ? "ok" : "FAIL", what);
    if (!ok) ++failures;
}

int main(void)
{
    check(trax_version() != NULL && strlen(trax_version()) > 0, "version");
    check(trax_abi_sizeof("trax_config") == sizeof(trax_config), "sizeof trax_config");
    check(trax_abi_sizeof("trax_event_batch") == sizeof(trax_event_batch),
          "sizeof trax_event_batch");
    check(trax_abi_sizeof("no_such_type") == 0, "sizeof unknown");
    check(trax_min_radius_curvature(1.0f, 0.0f) > 0.0f, "min radius curvature");

    /* one triplet (1, 2, 3) over three layers with geometry: valid */
    trax_config cfg;
    memset(&cfg, 0, sizeof cfg);
    cfg.n_layer_triplets = 1;
    cfg.triplets[0].layer1 = 1;
    cfg.triplets[0].layer2 = 2;
    cfg.triplets[0].layer3 = 3;
    cfg.n_geom_layers = 3;
    for (int l = 0; l < 3; ++l) {
        cfg.min_radius[l] = 4.0f + 3.0f * (float)l;
        cfg.max_radius[l] = 4.5f + 3.0f * (float)l;
    }
    cfg.min_pt = 1.0f;
    trax_grid_cfg grid = {1, 3, 8, 16};
    check(trax_config_validate(&cfg, &grid) == TRAX_OK, "config valid");
    cfg.triplets[0].layer1 = 2;  /* triplet 0 must start on layer 1 */
    check(trax_config_validate(&cfg, &grid) != TRAX_OK, "config rejected");

    trax_ctx *ctx = NULL;
    const trax_status st = trax_ctx_create(&ctx, 0);
    if (st == TRAX_OK) {
        printf("gpu present\n");
        trax_ctx_destroy(ctx);
    } else {
        const char *msg = trax_ctx_last_error(NULL);
        check(ctx == NULL, "no context without a device");
        check(msg != NULL && strlen(msg) > 0, "error message");
        printf("status %d: %s\n", (int)st, msg ? msg : "");
    }
    return failures ? 1 : 0;
}
