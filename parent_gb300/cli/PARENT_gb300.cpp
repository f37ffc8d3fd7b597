// Drop-in for PARENT.x (src/PARENT/PARENT.cpp): same argv, same .bat input,
// same .par output, computed on one GPU through the parent_gb300 C ABI.
//   PARENT_gb300 input.bat entropy.par b1D a1D d1D b2D a2D d2D
#include <stdio.h>

#include <vector>

#include "common.h"

static const char *kUsage =
    " input.bat entropy.par #bondsbins1D #anglesbins1D #dihedralsbins1D #bondsbins2D "
    "#anglesbins2D #dihedralsbins2D\n";

int main(int argc, char **argv) {
    const double t1 = wall_seconds();
    if (argc != 9) {  // PARENT.cpp:190, :241-244
        fprintf(stderr, "USAGE: %s%s", argv[0], kUsage);
        return 1;
    }
    if (last_ext(argv[1]) != "bat" || last_ext(argv[2]) != "par") {  // PARENT.cpp:207-210
        fprintf(stderr, "USAGE: %s%s", argv[0], kUsage);
        return 1;
    }
    static const char *what[6] = {"1D bonds", "1D angles", "1D dihedrals", "2D bonds", "2D angles", "2D dihedrals"};
    int bins[6];
    for (int k = 0; k < 6; k++) {  // PARENT.cpp:211-234
        if (sscanf(argv[3 + k], "%d", &bins[k]) != 1) {
            fprintf(stderr, "ERROR: Could not read number of bins for %s from command line! Aborting\n", what[k]);
            return 1;
        }
    }
    const int form = env_form();
    if (form < 0) {
        fprintf(stderr, "ERROR: PG_FORM must be auto, hist or onehot\n");
        return 1;
    }
    printf("Reading file %s .\n", argv[1]);
    pg_bat *bat = nullptr;
    if (pg_bat_read(argv[1], &bat) != PG_OK) {
        fprintf(stderr, "AN ERROR HAS OCCURED WHILE READING THE HEADER OF THE FILE %s . QUITTING PROGRAM.\n", argv[1]);
        return 1;
    }
    const int nd = pg_bat_n_dihedrals(bat), nb = nd + 2, na = nd + 1;
    pg_bat_view view;
    pg_bat_view_of(bat, &view);
    printf("%s specs:\nPrecision: %s #Atoms: %d #Frames: %d\n", argv[1],
           view.double_prec == 1 ? "double" : "single", nd + 3, view.n_frames);
    pg_ctx *ctx = nullptr;
    if (pg_create(&ctx, env_device()) != PG_OK) {
        fprintf(stderr, "ERROR: %s\n", pg_last_global_error());
        pg_bat_free(bat);
        return 1;
    }
    std::vector<double> s1b(nb), s1a(na), s1d(nd), bb((size_t)nb * (nb - 1) / 2), ba((size_t)nb * na),
        bd((size_t)nb * nd), aa((size_t)na * (na - 1) / 2), ad((size_t)na * nd), dd((size_t)nd * (nd > 0 ? nd - 1 : 0) / 2);
    pg_par_body body{s1b.data(), s1a.data(), s1d.data(), bb.data(), ba.data(), bd.data(), aa.data(), ad.data(), dd.data()};
    const double t2 = wall_seconds();
    int rc = pg_entropy(ctx, &view, bins, form, &body);
    if (rc != PG_OK) {
        fprintf(stderr, "ERROR: %s\n", pg_last_error(ctx));
        pg_destroy(ctx);
        pg_bat_free(bat);
        return 1;
    }
    double ms[5];
    pg_last_timings(ctx, ms);
    printf("GPU form: %s; device time: preprocessing %.3f ms, pairs %.3f ms, copies %.3f ms\n",
           pg_last_form(ctx) == PG_FORM_ONEHOT ? "onehot" : "hist", ms[0], ms[1], ms[3]);
    const double t3 = wall_seconds();
    rc = pg_par_write(argv[2], bat, bins, &body);
    if (rc != PG_OK) fprintf(stderr, "AN ERROR HAS OCCURED WHILE WRITING THE FILE %s .\n", argv[2]);
    const double t4 = wall_seconds();
    printf("Initialization + readin time: %g\n", t2 - t1);
    printf("Calculation time: %g\n", t3 - t2);
    printf("Output time: %g\n", t4 - t3);
    printf("Total execution time: %g\n", t4 - t1);
    pg_destroy(ctx);
    pg_bat_free(bat);
    if (rc == PG_OK) printf("PROGRAM FINISHED SUCCESSFULLY.\n");
    return rc == PG_OK ? 0 : 1;
}
