// Drop-in for get_PAR_info.x (src/process_output/get_PAR_info.cpp): prints
// the bond/angle/dihedral atom indices stored in the .par header.
#include <stdio.h>

#include "common.h"

int main(int argc, char **argv) {
    if (argc != 2) {
        fprintf(stderr, "usage: %s entropyfile.par\n", argc > 0 ? argv[0] : "get_PAR_info_gb300");
        return 1;
    }
    pg_par *par = nullptr;
    if (pg_par_read(argv[1], &par) != PG_OK) {
        fprintf(stderr, "ERROR READING HEADER OF FILE %s !\n", argv[1]);
        return 1;
    }
    const int rc = pg_write_info_text(nullptr, par);
    pg_par_free(par);
    return rc == PG_OK ? 0 : 1;
}
