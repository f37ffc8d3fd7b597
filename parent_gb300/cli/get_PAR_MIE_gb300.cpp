// Drop-in for get_PAR_MIE.x (src/process_output/get_PAR_MIE.cpp): prints
// every 1D entropy, every pair's 2D entropy and MI, and the 16 totals.
//   get_PAR_MIE_gb300 input.par > out_MIE.txt
// The pair lines are formatted on the GPU (pg_write_mie_text_device, device
// PG_DEVICE); PG_MIE_WRITER=host formats everything on the host threads.
#include <stdio.h>
#include <string.h>

#include "common.h"

int main(int argc, char **argv) {
    if (argc < 2) {
        fprintf(stderr, "ERROR: COULD NOT OPEN FILE !\n\nUSAGE:\n%s input.par\n", argv[0]);
        return 1;
    }
    pg_par *par = nullptr;
    if (pg_par_read(argv[1], &par) != PG_OK) {
        fprintf(stderr, "ERROR READING FILE %s !\n", argv[1]);
        return 1;
    }
    pg_par_body body;
    pg_par_body_of(par, &body);
    const char *ew = getenv("PG_MIE_WRITER");
    int rc;
    if (ew && strcmp(ew, "host") == 0) {
        rc = pg_write_mie_text(nullptr, pg_par_n_dihedrals(par), &body);
    } else {
        pg_ctx *ctx = nullptr;
        rc = pg_create(&ctx, env_device());
        if (rc != PG_OK) {
            fprintf(stderr, "ERROR: %s (PG_MIE_WRITER=host formats on the host)\n", pg_last_global_error());
        } else {
            rc = pg_write_mie_text_device(ctx, nullptr, pg_par_n_dihedrals(par), &body);
            if (rc != PG_OK) fprintf(stderr, "ERROR: %s\n", pg_last_error(ctx));
            pg_destroy(ctx);
        }
    }
    pg_par_free(par);
    return rc == PG_OK ? 0 : 1;
}
