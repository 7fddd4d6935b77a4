/* A C99 host of the library, as the reference's driver would call it through
 * the C ABI (src/mcpolar.f90:79-94 reads res/input.params, :148-186 runs the
 * loop): read the input file and a config-mode extension file, check the
 * struct layouts the header declares against the library's, create a
 * context on the first device and run two coupled iterations.  Without a
 * CUDA device tam_create must fail with TAM_E_NODEV (no CPU fallback).
 * Usage: host <input.params> <extension file>.  Exit 0 on success. */
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "tam.h"

static int check(int rc, const char *what)
{
    if (rc != TAM_OK) fprintf(stderr, "%s: %d %s\n", what, rc, tam_last_error(NULL));
    return rc == TAM_OK;
}

int main(int argc, char **argv)
{
    tam_params p;
    tam_config c;
    struct tam_ctx *ctx = NULL;
    int rc;
    if (argc < 3) return 2;
    if (tam_struct_size(0) != (int64_t)sizeof(tam_params) || tam_struct_size(1) != (int64_t)sizeof(tam_config) ||
        tam_struct_size(2) != (int64_t)sizeof(tam_state) || tam_struct_size(3) != (int64_t)sizeof(tam_material)) {
        fprintf(stderr, "struct layouts differ from the library's\n");
        return 3;
    }
    if (!check(tam_params_default(&p), "tam_params_default")) return 4;  /* the fields the file does not hold */
    if (!check(tam_read_input_params(argv[1], &p), "tam_read_input_params")) return 4;
    if (!check(tam_config_default(&c), "tam_config_default")) return 5;
    if (!check(tam_read_config(argv[2], &c), "tam_read_config")) return 6;
    printf("params: grid %d %d %d, power %g W; config: %d materials, T0 %g K\n", p.nxg, p.nyg, p.nzg, p.power,
           c.nmat, c.T0);
    p.nxg = p.nyg = p.nzg = 8;
    rc = tam_create(&p, NULL, &ctx);
    if (rc == TAM_E_NODEV) {
        printf("no CUDA device: %s\n", tam_last_error(NULL));
        return 0;
    }
    if (!check(rc, "tam_create")) return 7;
    rc = tam_step_coupled(ctx, 2, 1);
    if (rc == TAM_OK) {
        double absorbed = 0, reflected = 0, transmitted = 0;
        rc = tam_get_tallies(ctx, &absorbed, &reflected, &transmitted);
        printf("absorbed %g, reflected %g, transmitted %g\n", absorbed, reflected, transmitted);
    } else {
        fprintf(stderr, "tam_step_coupled: %d %s\n", rc, tam_last_error(ctx));
    }
    tam_destroy(ctx);
    return rc == TAM_OK ? 0 : 8;
}
