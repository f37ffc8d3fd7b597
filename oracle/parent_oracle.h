/*
 * ORACLE — test infrastructure only. Nothing in the product links, loads or
 * calls this code; only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg use it, and only to check results or as the timed CPU reference.
 *
 * A plain-C restatement of the reference PARENT algorithm (markusfleck/PARENT):
 * .bat parsing, per-DOF extrema and dihedral "modfit" shift, 1D and 2D
 * histogram entropies, get_mutual, the MIE totals and the MIST spanning tree.
 * Every FP64 expression keeps the reference's operation order, so with the
 * same libm the results are bit-identical to the reference programs built in
 * oracle/_ref (pinned by tests/test_oracle_pins.py).
 */
#ifndef PARENT_ORACLE_H
#define PARENT_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* DOF type codes, as util.h:33-35 (TYPE_B/TYPE_A/TYPE_D). */
enum { OR_B = 0, OR_A = 1, OR_D = 2 };

/* Reads a .bat file (io_binary.cpp:107-200 header, :281-368 frames) into
 * DOF-major FP64 columns, promoting FP32 values exactly as read_BAT_frame.
 * The caller frees the three column arrays with or_free.
 * bonds: (nDih+2)*F, angles: (nDih+1)*F, dihedrals: nDih*F, column-major by DOF.
 * Returns 0 on success, nonzero on a read/header error. */
int or_read_bat(const char *path, int *n_dihedrals, int *n_frames, int *double_prec,
                double **bonds, double **angles, double **dihedrals);
void or_free(void *p);

/* Per-DOF extrema and dihedral shift, PARENT.cpp:504-638. Rewrites the
 * dihedral columns in place (as the reference does). Returns the number of
 * negative bonds (reference aborts on any, PARENT.cpp:522-525) plus the number
 * of out-of-range modfit indices (reference: undefined behaviour). */
int or_extrema(int n_dihedrals, int n_frames, double *bonds, double *angles, double *dihedrals,
               double *min_b, double *max_b, double *min_a, double *max_a,
               double *min_d, double *max_d, double *modfit /* nDih, may be NULL */);

/* 1D entropy of one DOF column, PARENT.cpp:650-671 (b), :694-715 (a), :738-757 (d). */
double or_entropy1d(int type, const double *x, int n_frames, double mn, double mx, int nbins,
                    int *bad_index);

/* 2D entropy of one pair (row DOF x, column DOF y) with the reference's
 * epilogue (PARENT.cpp:786-823 bb, :826-856 ba, :858-886 bd, :1141-1176 aa,
 * :1178-1206 ad, :1383-1414 dd). type1 <= type2. If counts != NULL the
 * B1*B2 histogram (int64, row-major) is written there. */
double or_entropy2d(int type1, const double *x, double min1, double max1, int b1,
                    int type2, const double *y, double min2, double max2, int b2,
                    int n_frames, int64_t *counts, int *bad_index);

/* The whole PARENT.x computation (after the read): extrema, 1D entropies,
 * all six 2D blocks in the .par body layout (reverse triangles for bb/aa/dd,
 * PARENT.cpp:896,1107-1112). bins = {b1D,a1D,d1D,b2D,a2D,d2D}. Dihedral
 * columns are shifted in place. OpenMP over pairs; results do not depend on
 * the thread count. Returns 0, or nonzero on invalid input. */
int or_parent(int n_dihedrals, int n_frames, double *bonds, double *angles, double *dihedrals,
              const int bins[6], double *s1_b, double *s1_a, double *s1_d,
              double *bb, double *ba, double *bd, double *aa, double *ad, double *dd);

/* get_mutual, util.cpp:47-81. type in TYPE_BB..TYPE_DD = 0..5. */
double or_mutual(int type, int i, int j, int n_dihedrals,
                 const double *s1_b, const double *s1_a, const double *s1_d,
                 const double *bb, const double *ba, const double *bd,
                 const double *aa, const double *ad, const double *dd);

/* The 16 MIE totals in get_PAR_MIE.cpp:184-199 order. */
void or_mie_totals(int n_dihedrals, const double *s1_b, const double *s1_a, const double *s1_d,
                   const double *bb, const double *ba, const double *bd,
                   const double *aa, const double *ad, const double *dd, double totals[16]);

/* MIST, get_PAR_MIST.cpp:290-327 (matrix), :400-748 (greedy tree, one-thread
 * scan order), :754-765 (totals). Edge k (k < nB+nA+nD-1):
 * edge_t1/t2 = In/Out types, edge_i1/i2 = 1-based DOF indices as printed,
 * edge_mi = MI, edge_left = |Out| before removal. totals[10] in print order. */
void or_mist(int n_dihedrals, const double *s1_b, const double *s1_a, const double *s1_d,
             const double *bb, const double *ba, const double *bd,
             const double *aa, const double *ad, const double *dd,
             int *edge_t1, int *edge_t2, int *edge_i1, int *edge_i2, double *edge_mi,
             int *edge_left, double totals[10]);

/* or_mist plus, per step, the gap between the winning MI and the largest
 * other candidate value of that step's scan (0 where the winner was decided
 * by the scan order among equal values; INFINITY for a single candidate).
 * The scan runs on all OpenMP threads over contiguous ranges of the step's
 * scan sequence, merged in order: the result is the serial scan's. */
void or_mist_gap(int n_dihedrals, const double *s1_b, const double *s1_a, const double *s1_d,
                 const double *bb, const double *ba, const double *bd,
                 const double *aa, const double *ad, const double *dd,
                 int *edge_t1, int *edge_t2, int *edge_i1, int *edge_i2, double *edge_mi,
                 int *edge_left, double *edge_gap, double totals[10]);

/* Full-size parity on a sample: for every DOF (global index, bonds | angles |
 * dihedrals) the extrema and dihedral shift of PARENT.cpp:504-638 and the 1D
 * entropy at bins[0..2] (s1[D], mn[D], mx[D], modfit[D], 0 for non-dihedrals);
 * for each listed pair g1[k] < g2[k] the 2D entropy of PARENT.cpp:786-1479
 * (s2[k]) and, for k < n_counts, its B1 x B2 counts at counts + k*count_stride.
 * Columns are FP32 (double_prec 0, promoted as read_BAT_frame does) or FP64,
 * DOF-major with leading dimension ld, per type; they are not modified and
 * no FP64 copy of the whole trajectory is made. Returns 0, or nonzero if a
 * bond was negative or an index left its range. */
int or_sample(int n_dihedrals, int n_frames, int double_prec, const void *bonds, const void *angles,
              const void *dihedrals, long long ld, const int bins[6], int n_pairs, const int *g1,
              const int *g2, double *s1, double *s2, int n_counts, int64_t *counts, long long count_stride,
              double *mn, double *mx, double *modfit);

/* Cartesian -> BAT columns as BAT_builder converts a trajectory frame by
 * frame (BAT_trajectory.cpp:114-125): coordinates scaled by 10 (nm ->
 * Angstrom, stored back as float), convert_to_BAT (:219-300),
 * convert_dihedrals_to_phaseangles (:303-310, in place, in dihedral order)
 * and shift_dihedrals_0_2pi_range (:209-214). xyz: n_frames x (nDih+3) x 3
 * floats; dih: nDih x 6 ints as in the .bat header (atoms 1-based, [5] the
 * parent dihedral 1-based or -1). Output columns DOF-major as or_read_bat:
 * bonds (nDih+2)*F, angles (nDih+1)*F, dihedrals nDih*F. Returns 0, or
 * nonzero for an atom or parent index out of range. */
int or_bat_from_xyz(int n_dihedrals, int n_frames, const float *xyz, const int *dih,
                    double *bonds, double *angles, double *dihedrals);

#ifdef __cplusplus
}
#endif
#endif
