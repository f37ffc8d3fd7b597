/* Test infrastructure: dumps the Cartesian coordinates of a GROMACS .xtc
 * trajectory (decoded by the reference's own xdrfile library, compiled from
 * its sources into oracle/_ref) as raw little-endian data for the golden
 * fixtures of the BAT conversion:
 *   int32 n_atoms, int32 n_frames, then n_frames x n_atoms x 3 float32 (nm).
 * Used only by tests/golden/make_golden.py, where the reference exists.
 *   xtc_dump in.xtc out.raw */
#include <stdio.h>
#include <stdlib.h>

#include "xdrfile_xtc.h"

int main(int argc, char **argv) {
    if (argc != 3) {
        fprintf(stderr, "usage: %s in.xtc out.raw\n", argv[0]);
        return 1;
    }
    int natoms = 0;
    if (read_xtc_natoms(argv[1], &natoms) != exdrOK || natoms <= 0) {
        fprintf(stderr, "cannot read the atom count of %s\n", argv[1]);
        return 1;
    }
    XDRFILE *xd = xdrfile_open(argv[1], "r");
    FILE *out = fopen(argv[2], "wb");
    if (!xd || !out) {
        fprintf(stderr, "cannot open the files\n");
        return 1;
    }
    rvec *x = (rvec *)malloc(sizeof(rvec) * (size_t)natoms);
    int nframes = 0, step = 0;
    float time = 0.f, prec = 0.f;
    matrix box;
    fwrite(&natoms, 4, 1, out);
    fwrite(&nframes, 4, 1, out);
    while (read_xtc(xd, natoms, &step, &time, box, x, &prec) == exdrOK) {
        fwrite(x, sizeof(rvec), (size_t)natoms, out);
        nframes++;
    }
    fseek(out, 4, SEEK_SET);
    fwrite(&nframes, 4, 1, out);
    fclose(out);
    xdrfile_close(xd);
    free(x);
    printf("%d atoms, %d frames\n", natoms, nframes);
    return 0;
}
