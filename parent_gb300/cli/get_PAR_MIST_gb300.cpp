// Drop-in for get_PAR_MIST.x (src/process_output/get_PAR_MIST.cpp):
//   get_PAR_MIST_gb300 input.par output.txt
// Reads the .par, builds the MI matrix on the GPU and runs the MIST tree there.
#include <stdio.h>

#include <vector>

#include "common.h"

int main(int argc, char **argv) {
    const double t1 = wall_seconds();
    if (argc != 3) {  // get_PAR_MIST.cpp:74-77
        fprintf(stderr, "USAGE:\n%s input.par output.txt\n", argv[0]);
        return 1;
    }
    pg_par *par = nullptr;
    if (pg_par_read(argv[1], &par) != PG_OK) {
        fprintf(stderr, "An ERROR has occurred while reading the file %s . Quitting Program.\n", argv[1]);
        return 1;
    }
    const int nd = pg_par_n_dihedrals(par);
    pg_par_body body;
    pg_par_body_of(par, &body);
    pg_ctx *ctx = nullptr;
    if (pg_create(&ctx, env_device()) != PG_OK) {
        fprintf(stderr, "ERROR: %s\n", pg_last_global_error());
        pg_par_free(par);
        return 1;
    }
    std::vector<pg_mist_edge> edges((size_t)3 * nd + 2);
    double totals[10];
    const double t2 = wall_seconds();
    int rc = pg_mist(ctx, nd, &body, edges.data(), totals);
    if (rc != PG_OK) fprintf(stderr, "ERROR: %s\n", pg_last_error(ctx));
    const double t3 = wall_seconds();
    if (rc == PG_OK) {
        rc = pg_write_mist_text(argv[2], nd, edges.data(), totals);
        if (rc != PG_OK) fprintf(stderr, "ERROR: COULD NOT OPEN FILE %s !\n", argv[2]);
    }
    printf("Initialization + readin time: %g\n", t2 - t1);
    printf("Calculation time: %g\n", t3 - t2);
    printf("Total execution time: %g\n", wall_seconds() - t1);
    pg_destroy(ctx);
    pg_par_free(par);
    if (rc == PG_OK) printf("PROGRAM FINISHED SUCCESSFULLY.\n");
    return rc == PG_OK ? 0 : 1;
}
