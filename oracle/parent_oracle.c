/*
 * ORACLE — test infrastructure only (see parent_oracle.h). A CPU restatement
 * of the reference PARENT algorithm; the product never links or calls it.
 *
 * Every floating-point expression below is written in the same operation
 * order as the reference line it cites, so that (with -ffp-contract=off and
 * the same libm) the results are bit-identical to the reference programs.
 */
#include "parent_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
static int omp_nthreads(void) { return omp_get_num_threads(); }
static int omp_thread(void) { return omp_get_thread_num(); }
#else
static int omp_nthreads(void) { return 1; }
static int omp_thread(void) { return 0; }
#endif

#define MODFITNBINS 100 /* PARENT.cpp:51 */

void or_free(void *p) { free(p); }

/* ---------------------------------------------------------------- .bat read */

static int rd(FILE *f, void *dst, size_t n) { return fread(dst, 1, n, f) == n ? 0 : 1; }

/* io_binary.cpp:107-200 (header) and :281-368 (frames); the frame values are
 * scattered DOF-major as PARENT.cpp:443-473 does for its single rank. */
int or_read_bat(const char *path, int *n_dihedrals, int *n_frames, int *double_prec,
                double **bonds, double **angles, double **dihedrals) {
    FILE *f = fopen(path, "rb");
    if (!f) return 1;
    int version, prec, ndih, nfr;
    int fail = rd(f, &version, 4) | rd(f, &prec, 4) | rd(f, &ndih, 4) | rd(f, &nfr, 4);
    if (fail || version < 0 || (prec != 0 && prec != 1) || ndih < 0 || nfr < 1) {
        fclose(f);
        return 1;
    }
    if (version >= 3) { /* per atom: residue[8], resnum int, atom[8], molecule[31] */
        if (fseek(f, (long)(ndih + 3) * (8 + 4 + 8 + 31), SEEK_CUR)) { fclose(f); return 1; }
    }
    /* dihedral table (6 ints each) and masses (float per atom) */
    if (fseek(f, (long)ndih * 24 + (long)(ndih + 3) * 4, SEEK_CUR)) { fclose(f); return 1; }

    const int nb = ndih + 2, na = ndih + 1;
    const size_t F = (size_t)nfr;
    double *B = malloc(sizeof(double) * nb * F);
    double *A = malloc(sizeof(double) * na * F);
    double *D = malloc(sizeof(double) * (ndih > 0 ? ndih : 1) * F);
    const size_t vsz = prec ? 8 : 4;
    const size_t fbytes = 44 + (size_t)(9 + 3 * ndih) * vsz;
    unsigned char *buf = malloc(fbytes);
    if (!B || !A || !D || !buf) { fclose(f); free(B); free(A); free(D); free(buf); return 2; }
    for (size_t fr = 0; fr < F && !fail; fr++) {
        if (rd(f, buf, fbytes)) { fail = 1; break; }
        const unsigned char *p = buf + 44 + 6 * vsz; /* skip time,prec,box, 6 externals */
        double v[3];
        for (int k = 0; k < 3 + 3 * ndih; k++) {
            double val;
            if (prec) { memcpy(&val, p + (size_t)k * 8, 8); }
            else { float fv; memcpy(&fv, p + (size_t)k * 4, 4); val = fv; }
            if (k < 3) { v[k] = val; continue; }
            int d = (k - 3) / 3, c = (k - 3) % 3;
            if (c == 0) B[(size_t)(d + 2) * F + fr] = val;
            else if (c == 1) A[(size_t)(d + 1) * F + fr] = val;
            else D[(size_t)d * F + fr] = val;
        }
        B[fr] = v[0];
        B[F + fr] = v[1];
        A[fr] = v[2];
    }
    free(buf);
    fclose(f);
    if (fail) { free(B); free(A); free(D); return 1; }
    *n_dihedrals = ndih; *n_frames = nfr; *double_prec = prec;
    *bonds = B; *angles = A; *dihedrals = D;
    return 0;
}

/* ---------------------------------------------------------------- extrema */

/* One bond column, PARENT.cpp:511-536. Returns 1 for a negative bond. */
static int ext_bond(const double *x, size_t F, double *mn, double *mx) {
    double tmpMax = -1.0e100, tmpMin = 1.0e100;
    for (size_t i = 0; i < F; i++) {
        if (x[i] > tmpMax) tmpMax = x[i];
        if (x[i] < tmpMin) tmpMin = x[i];
    }
    const int bad = (tmpMin < 0.0) || (tmpMax < 0.0);
    tmpMin -= 0.000000005;
    tmpMax += 0.000000005;
    if (tmpMin < 0.0) tmpMin = 0.0;
    if ((tmpMax - tmpMin) < 1.0e-4) tmpMax += 0.05;
    *mx = tmpMax;
    *mn = tmpMin;
    return bad;
}

/* One angle column, PARENT.cpp:538-562. */
static void ext_angle(const double *x, size_t F, double pi, double *mn, double *mx) {
    double tmpMax = -1.0e100, tmpMin = 1.0e100;
    for (size_t i = 0; i < F; i++) {
        if (x[i] > tmpMax) tmpMax = x[i];
        if (x[i] < tmpMin) tmpMin = x[i];
    }
    tmpMin -= 0.000000005;
    tmpMax += 0.000000005;
    if (tmpMin < 0) tmpMin = 0;
    if (tmpMax > pi) tmpMax = pi;
    if ((tmpMax - tmpMin) < 1.0e-4) tmpMax += 0.05;
    *mx = tmpMax;
    *mn = tmpMin;
}

/* The periodic shift of one dihedral value, PARENT.cpp:611. */
static inline double dih_shift(double x, double modFit, double pi) {
    return x + modFit - 2 * pi * (int)((x + modFit) / (2 * pi));
}

/* One dihedral column, PARENT.cpp:564-637: the shift ("modfit") is found
 * from a 100-bin occupancy histogram and applied in place, then the extrema
 * of the shifted column. Returns the number of out-of-range histogram
 * indices (undefined behaviour in the reference). */
static int ext_dih(double *x, size_t F, double pi, double *mn, double *mx, double *modfit) {
    int bad = 0;
    long long histo[MODFITNBINS];
    for (int k = 0; k < MODFITNBINS; k++) histo[k] = 0;
    const double binsize = (2 * pi + 0.000000005) / MODFITNBINS;
    for (size_t i = 0; i < F; i++) {
        int idx = (int)((x[i]) / binsize);
        if (idx < 0 || idx >= MODFITNBINS) { bad++; idx = idx < 0 ? 0 : MODFITNBINS - 1; }
        histo[idx] += 1;
    }
    int zeroExists = 0;
    for (int k = 0; k < MODFITNBINS; k++) zeroExists = zeroExists || (histo[k] == 0);
    int longestZeroStretch, longestZeroStretchPos, currentZeroStretch, currentZeroStretchPos = 0;
    if (zeroExists) {
        longestZeroStretch = 0;
        currentZeroStretch = 0;
        longestZeroStretchPos = -1;
        for (int k = 0; k < 2 * MODFITNBINS; k++) {
            int l = k % MODFITNBINS;
            if ((currentZeroStretch == 0) && (histo[l] == 0)) {
                currentZeroStretch = 1;
                currentZeroStretchPos = k;
            }
            if ((currentZeroStretch > 0) && (histo[l] == 0)) currentZeroStretch += 1;
            if ((currentZeroStretch > 0) && (histo[l] != 0)) {
                if (currentZeroStretch > longestZeroStretch) {
                    longestZeroStretch = currentZeroStretch;
                    longestZeroStretchPos = currentZeroStretchPos;
                }
                currentZeroStretch = 0;
            }
        }
    } else {
        longestZeroStretchPos = 0;
        longestZeroStretch = (int)histo[0];
        for (int k = 0; k < MODFITNBINS; k++) {
            if (histo[k] < longestZeroStretch) {
                longestZeroStretch = (int)histo[k];
                longestZeroStretchPos = k;
            }
        }
    }
    const double modFit = 2 * pi - (longestZeroStretchPos + 0.5) * binsize;
    if (modfit) *modfit = modFit;
    for (size_t k = 0; k < F; k++) x[k] = dih_shift(x[k], modFit, pi);
    double tmpMax = -1.0e100, tmpMin = 1.0e100;
    for (size_t i = 0; i < F; i++) {
        if (x[i] > tmpMax) tmpMax = x[i];
        if (x[i] < tmpMin) tmpMin = x[i];
    }
    tmpMin -= 0.000000005;
    tmpMax += 0.000000005;
    if (tmpMin < 0.0) tmpMin = 0.0;
    if (tmpMax > 2 * pi) tmpMax = 2 * pi;
    if ((tmpMax - tmpMin) < 1.0e-4) tmpMax += 0.05;
    *mx = tmpMax;
    *mn = tmpMin;
    return bad;
}

int or_extrema(int n_dihedrals, int n_frames, double *bonds, double *angles, double *dihedrals,
               double *min_b, double *max_b, double *min_a, double *max_a,
               double *min_d, double *max_d, double *modfit) {
    const double pi = acos(-1); /* PARENT.cpp:112 */
    const int nb = n_dihedrals + 2, na = n_dihedrals + 1, nd = n_dihedrals;
    const size_t F = (size_t)n_frames;
    int bad = 0;
#pragma omp parallel for reduction(+ : bad) schedule(dynamic)
    for (int j = 0; j < nb; j++) bad += ext_bond(bonds + j * F, F, &min_b[j], &max_b[j]);
#pragma omp parallel for schedule(dynamic)
    for (int j = 0; j < na; j++) ext_angle(angles + j * F, F, pi, &min_a[j], &max_a[j]);
#pragma omp parallel for reduction(+ : bad) schedule(dynamic)
    for (int j = 0; j < nd; j++)
        bad += ext_dih(dihedrals + j * F, F, pi, &min_d[j], &max_d[j], modfit ? &modfit[j] : NULL);
    return bad;
}

/* ---------------------------------------------------------------- 1D */

static inline int bin_of(double x, double mn, double binsize, int nb, int *bad) {
    int idx = (int)((x - mn) / binsize);
    if (idx < 0 || idx >= nb) { (*bad)++; idx = idx < 0 ? 0 : nb - 1; }
    return idx;
}

double or_entropy1d(int type, const double *x, int n_frames, double mn, double mx, int nbins,
                    int *bad_index) {
    long long *histo = calloc((size_t)nbins, sizeof(long long));
    int bad = 0;
    const double binsize = (mx - mn) / (nbins);
    for (int i = 0; i < n_frames; i++) histo[bin_of(x[i], mn, binsize, nbins, &bad)] += 1;
    int occupbins = 0;
    double plnpsum = 0, probDens;
    if (type == OR_B) { /* PARENT.cpp:658-670 */
        double blen = mn + (binsize / 2.0);
        for (int k = 0; k < nbins; k++) {
            probDens = histo[k] / (n_frames * binsize * blen * blen);
            if (probDens > 0) {
                plnpsum = plnpsum + blen * blen * probDens * log(probDens);
                occupbins = occupbins + 1;
            }
            blen += binsize;
        }
    } else if (type == OR_A) { /* PARENT.cpp:702-714 */
        double theta = mn + (binsize / 2.0);
        for (int k = 0; k < nbins; k++) {
            probDens = histo[k] / (n_frames * binsize * sin(theta));
            if (probDens > 0) {
                plnpsum = plnpsum + sin(theta) * probDens * log(probDens);
                occupbins = occupbins + 1;
            }
            theta += binsize;
        }
    } else { /* PARENT.cpp:746-756 */
        for (int k = 0; k < nbins; k++) {
            probDens = histo[k] / (n_frames * binsize);
            if (probDens > 0) {
                plnpsum = plnpsum + probDens * log(probDens);
                occupbins = occupbins + 1;
            }
        }
    }
    plnpsum = -plnpsum * binsize;
    free(histo);
    if (bad_index) *bad_index += bad;
    return plnpsum + (occupbins - 1.0) / (2.0 * n_frames);
}

/* ---------------------------------------------------------------- 2D */

double or_entropy2d(int type1, const double *x, double min1, double max1, int b1,
                    int type2, const double *y, double min2, double max2, int b2,
                    int n_frames, int64_t *counts, int *bad_index) {
    int64_t stackbuf[64 * 64];
    int64_t *histo = counts ? counts
                            : (b1 * b2 <= 64 * 64 ? stackbuf : malloc(sizeof(int64_t) * b1 * b2));
    memset(histo, 0, sizeof(int64_t) * b1 * b2);
    int bad = 0;
    const double binsize1 = (max1 - min1) / b1;
    const double binsize2 = (max2 - min2) / b2;
    for (int i = 0; i < n_frames; i++) { /* e.g. PARENT.cpp:802-804 */
        int r = bin_of(x[i], min1, binsize1, b1, &bad);
        int c = bin_of(y[i], min2, binsize2, b2, &bad);
        histo[(size_t)r * b2 + c] += 1;
    }
    const double N = n_frames;
    int occupbins = 0;
    double plnpsum = 0, sum1, probDens;
    const int tt = type1 * 3 + type2;
    double c1 = min1 + binsize1 / 2.0; /* blen1 / theta1 */
    for (int k = 0; k < b1; k++) {
        sum1 = 0.0;
        double c2 = min2 + binsize2 / 2.0; /* blen2 / theta2 */
        const int64_t *row = histo + (size_t)k * b2;
        for (int l = 0; l < b2; l++) {
            const double h = (double)row[l];
            switch (tt) {
            case 0: /* bb, PARENT.cpp:812-814 */
                probDens = h / (N * binsize1 * binsize2 * c1 * c1 * c2 * c2);
                if (probDens > 0) {
                    sum1 = sum1 + c1 * c1 * c2 * c2 * probDens * log(probDens) * binsize1 * binsize2;
                    occupbins = occupbins + 1;
                }
                break;
            case 1: /* ba, PARENT.cpp:845-847 */
                probDens = h / (N * binsize1 * binsize2 * c1 * c1 * sin(c2));
                if (probDens > 0) {
                    sum1 = sum1 + c1 * c1 * sin(c2) * probDens * log(probDens) * binsize1 * binsize2;
                    occupbins = occupbins + 1;
                }
                break;
            case 2: /* bd, PARENT.cpp:876-878 */
                probDens = h / (N * binsize1 * binsize2 * c1 * c1);
                if (probDens > 0) {
                    sum1 = sum1 + c1 * c1 * probDens * log(probDens) * binsize1 * binsize2;
                    occupbins = occupbins + 1;
                }
                break;
            case 4: /* aa, PARENT.cpp:1165-1167 */
                probDens = h / (N * binsize1 * binsize2 * sin(c1) * sin(c2));
                if (probDens > 0) {
                    sum1 = sum1 + sin(c1) * sin(c2) * probDens * log(probDens) * binsize1 * binsize2;
                    occupbins = occupbins + 1;
                }
                break;
            case 5: /* ad, PARENT.cpp:1196-1198 */
                probDens = h / (N * binsize1 * binsize2 * sin(c1));
                if (probDens > 0) {
                    sum1 = sum1 + sin(c1) * probDens * log(probDens) * binsize1 * binsize2;
                    occupbins = occupbins + 1;
                }
                break;
            default: /* dd, PARENT.cpp:1405-1407 */
                probDens = h / (N * binsize1 * binsize2);
                if (probDens > 0) {
                    sum1 = sum1 + probDens * log(probDens) * binsize1 * binsize2;
                    occupbins = occupbins + 1;
                }
                break;
            }
            c2 = c2 + binsize2;
        }
        plnpsum = plnpsum + sum1;
        c1 = c1 + binsize1;
    }
    if (!counts && histo != stackbuf) free(histo);
    if (bad_index) *bad_index += bad;
    return -plnpsum + (occupbins - 1.0) / (2.0 * n_frames);
}

/* ---------------------------------------------------------------- PARENT.x */

/* position of pair (i<j) of an n-DOF same-type block in the reverse layout,
 * PARENT.cpp:1107-1112 / util.cpp:55 */
static inline long long rev_index(int n, int s, int b) {
    return (long long)(n - s) * (n - s - 1) / 2 + s - b;
}

int or_parent(int n_dihedrals, int n_frames, double *bonds, double *angles, double *dihedrals,
              const int bins[6], double *s1_b, double *s1_a, double *s1_d,
              double *bb, double *ba, double *bd, double *aa, double *ad, double *dd) {
    const int nb = n_dihedrals + 2, na = n_dihedrals + 1, nd = n_dihedrals;
    const size_t F = (size_t)n_frames;
    for (int k = 0; k < 6; k++)
        if (bins[k] < 1) return 1;
    double *mn[3], *mx[3];
    const int cnt[3] = {nb, na, nd};
    for (int t = 0; t < 3; t++) {
        mn[t] = malloc(sizeof(double) * (cnt[t] > 0 ? cnt[t] : 1));
        mx[t] = malloc(sizeof(double) * (cnt[t] > 0 ? cnt[t] : 1));
    }
    int bad = or_extrema(n_dihedrals, n_frames, bonds, angles, dihedrals, mn[0], mx[0], mn[1],
                         mx[1], mn[2], mx[2], NULL);
    double *col[3] = {bonds, angles, dihedrals};
    double *s1[3] = {s1_b, s1_a, s1_d};
    for (int t = 0; t < 3; t++) {
        int b = 0;
#pragma omp parallel for reduction(+ : b) schedule(dynamic)
        for (int j = 0; j < cnt[t]; j++)
            s1[t][j] = or_entropy1d(t, col[t] + j * F, n_frames, mn[t][j], mx[t][j], bins[t], &b);
        bad += b;
    }
    /* all six 2D blocks; row DOF has the lower type / lower index */
    double *blk[6] = {bb, ba, bd, aa, ad, dd};
    const int t1s[6] = {0, 0, 0, 1, 1, 2}, t2s[6] = {0, 1, 2, 1, 2, 2};
    for (int q = 0; q < 6; q++) {
        const int t1 = t1s[q], t2 = t2s[q], n1 = cnt[t1], n2 = cnt[t2];
        const int same = (t1 == t2);
        int b = 0;
#pragma omp parallel for reduction(+ : b) schedule(dynamic, 1)
        for (int i = 0; i < n1; i++) {
            for (int j = same ? i + 1 : 0; j < n2; j++) {
                double s = or_entropy2d(t1, col[t1] + i * F, mn[t1][i], mx[t1][i], bins[3 + t1],
                                        t2, col[t2] + j * F, mn[t2][j], mx[t2][j], bins[3 + t2],
                                        n_frames, NULL, &b);
                if (same) blk[q][rev_index(n1, i, j)] = s;
                else blk[q][(size_t)i * n2 + j] = s;
            }
        }
        bad += b;
    }
    for (int t = 0; t < 3; t++) { free(mn[t]); free(mx[t]); }
    return bad ? 2 : 0;
}

/* ------------------------------------------------ sampled full-size check */

/* Column j (global DOF index) as FP64, promoted from FP32 exactly as
 * read_BAT_frame does (io_binary.cpp:322-364). */
static void load_col(int prec, const void *base, long long ld, int j, size_t F, double *out) {
    if (prec) {
        const double *x = (const double *)base + (size_t)j * (size_t)ld;
        memcpy(out, x, sizeof(double) * F);
    } else {
        const float *x = (const float *)base + (size_t)j * (size_t)ld;
        for (size_t i = 0; i < F; i++) out[i] = x[i];
    }
}

int or_sample(int n_dihedrals, int n_frames, int double_prec, const void *bonds, const void *angles,
              const void *dihedrals, long long ld, const int bins[6], int n_pairs, const int *g1,
              const int *g2, double *s1, double *s2, int n_counts, int64_t *counts, long long count_stride,
              double *mn, double *mx, double *modfit) {
    const double pi = acos(-1); /* PARENT.cpp:112 */
    const int nb = n_dihedrals + 2, na = n_dihedrals + 1, D = nb + na + n_dihedrals;
    const size_t F = (size_t)n_frames;
    for (int k = 0; k < 6; k++)
        if (bins[k] < 1) return 1;
    const void *src[3] = {bonds, angles, dihedrals};
    const int lo[3] = {0, nb, nb + na};
    int bad = 0;
    /* per DOF: extrema (and the dihedral shift) and the 1D entropy */
#pragma omp parallel reduction(+ : bad)
    {
        double *x = malloc(sizeof(double) * (F ? F : 1));
#pragma omp for schedule(dynamic, 4)
        for (int g = 0; g < D; g++) {
            const int t = g < nb ? 0 : (g < nb + na ? 1 : 2);
            load_col(double_prec, src[t], ld, g - lo[t], F, x);
            modfit[g] = 0.0;
            if (t == 0) bad += ext_bond(x, F, &mn[g], &mx[g]);
            else if (t == 1) ext_angle(x, F, pi, &mn[g], &mx[g]);
            else bad += ext_dih(x, F, pi, &mn[g], &mx[g], &modfit[g]);
            s1[g] = or_entropy1d(t, x, n_frames, mn[g], mx[g], bins[t], &bad);
        }
        free(x);
    }
    /* per pair: both columns (shifted as above), the 2D entropy */
#pragma omp parallel reduction(+ : bad)
    {
        double *x = malloc(sizeof(double) * (F ? F : 1));
        double *y = malloc(sizeof(double) * (F ? F : 1));
#pragma omp for schedule(dynamic, 1)
        for (int k = 0; k < n_pairs; k++) {
            const int a = g1[k], b = g2[k];
            if (a < 0 || b >= D || a >= b) { s2[k] = NAN; bad++; continue; }
            const int ta = a < nb ? 0 : (a < nb + na ? 1 : 2), tb = b < nb ? 0 : (b < nb + na ? 1 : 2);
            load_col(double_prec, src[ta], ld, a - lo[ta], F, x);
            load_col(double_prec, src[tb], ld, b - lo[tb], F, y);
            if (ta == 2)
                for (size_t i = 0; i < F; i++) x[i] = dih_shift(x[i], modfit[a], pi);
            if (tb == 2)
                for (size_t i = 0; i < F; i++) y[i] = dih_shift(y[i], modfit[b], pi);
            s2[k] = or_entropy2d(ta, x, mn[a], mx[a], bins[3 + ta], tb, y, mn[b], mx[b], bins[3 + tb], n_frames,
                                 k < n_counts ? counts + (size_t)k * (size_t)count_stride : NULL, &bad);
        }
        free(x);
        free(y);
    }
    return bad ? 2 : 0;
}

/* ---------------------------------------------------------------- MI / MIE */

double or_mutual(int type, int index1, int index2, int n_dihedrals,
                 const double *s1_b, const double *s1_a, const double *s1_d,
                 const double *bb, const double *ba, const double *bd,
                 const double *aa, const double *ad, const double *dd) {
    const int nb = n_dihedrals + 2, na = n_dihedrals + 1, nd = n_dihedrals;
    int smaller = index1 < index2 ? index1 : index2;
    int bigger = index1 < index2 ? index2 : index1;
    switch (type) {
    case 0: if (index1 == index2) break;
        return s1_b[smaller] + s1_b[bigger] - bb[rev_index(nb, smaller, bigger)];
    case 1: return s1_b[index1] + s1_a[index2] - ba[(size_t)index1 * na + index2];
    case 2: return s1_b[index1] + s1_d[index2] - bd[(size_t)index1 * nd + index2];
    case 3: if (index1 == index2) break;
        return s1_a[smaller] + s1_a[bigger] - aa[rev_index(na, smaller, bigger)];
    case 4: return s1_a[index1] + s1_d[index2] - ad[(size_t)index1 * nd + index2];
    case 5: if (index1 == index2) break;
        return s1_d[smaller] + s1_d[bigger] - dd[rev_index(nd, smaller, bigger)];
    }
    return 0;
}

#define MARGS n_dihedrals, s1_b, s1_a, s1_d, bb, ba, bd, aa, ad, dd

void or_mie_totals(int n_dihedrals, const double *s1_b, const double *s1_a, const double *s1_d,
                   const double *bb, const double *ba, const double *bd,
                   const double *aa, const double *ad, const double *dd, double totals[16]) {
    /* get_PAR_MIE.cpp:109-199, same accumulation order */
    const int nb = n_dihedrals + 2, na = n_dihedrals + 1, nd = n_dihedrals;
    double tB = 0, tA = 0, tD = 0;
    for (int k = 0; k < nb; k++) tB += s1_b[k];
    for (int k = 0; k < na; k++) tA += s1_a[k];
    for (int k = 0; k < nd; k++) tD += s1_d[k];
    double e[6] = {0}, m[6] = {0};
    long long counter = (long long)nb * (nb - 1) / 2 - 1;
    for (int i = 0; i < nb - 1; i++)
        for (int j = i + 1; j < nb; j++) {
            double mu = or_mutual(0, i, j, MARGS);
            e[0] += bb[counter]; m[0] += mu; counter--;
        }
    for (int i = 0; i < nb; i++)
        for (int j = 0; j < na; j++) {
            double mu = or_mutual(1, i, j, MARGS);
            e[1] += ba[(size_t)i * na + j]; m[1] += mu;
        }
    for (int i = 0; i < nb; i++)
        for (int j = 0; j < nd; j++) {
            double mu = or_mutual(2, i, j, MARGS);
            e[2] += bd[(size_t)i * nd + j]; m[2] += mu;
        }
    counter = (long long)na * (na - 1) / 2 - 1;
    for (int i = 0; i < na - 1; i++)
        for (int j = i + 1; j < na; j++) {
            double mu = or_mutual(3, i, j, MARGS);
            e[3] += aa[counter]; m[3] += mu; counter--;
        }
    for (int i = 0; i < na; i++)
        for (int j = 0; j < nd; j++) {
            double mu = or_mutual(4, i, j, MARGS);
            e[4] += ad[(size_t)i * nd + j]; m[4] += mu;
        }
    counter = (long long)nd * (nd - 1) / 2 - 1;
    for (int i = 0; i < nd - 1; i++)
        for (int j = i + 1; j < nd; j++) {
            double mu = or_mutual(5, i, j, MARGS);
            e[5] += dd[counter]; m[5] += mu; counter--;
        }
    totals[0] = tB; totals[1] = tA; totals[2] = tD;
    for (int q = 0; q < 6; q++) { totals[3 + 2 * q] = e[q]; totals[4 + 2 * q] = m[q]; }
    totals[15] = tB + tA + tD - m[0] - m[1] - m[2] - m[3] - m[4] - m[5];
}

/* ---------------------------------------------------------------- MIST */

/* The step's first maximum of one thread's contiguous range of the scan
 * sequence, and the largest value elsewhere in that range. */
typedef struct {
    double best, second;
    long long at; /* position in the step's scan sequence, -1 if none */
} scan_best;

void or_mist_gap(int n_dihedrals, const double *s1_b, const double *s1_a, const double *s1_d,
                 const double *bb, const double *ba, const double *bd,
                 const double *aa, const double *ad, const double *dd,
                 int *edge_t1, int *edge_t2, int *edge_i1, int *edge_i2, double *edge_mi,
                 int *edge_left, double *edge_gap, double totals[10]) {
    const int nb = n_dihedrals + 2, na = n_dihedrals + 1, nd = n_dihedrals;
    const int cnt[3] = {nb, na, nd}, lo[3] = {0, nb, nb + na};
    const int D = nb + na + nd;
    /* the six matrices of get_PAR_MIST.cpp:290-327 (get_mutual values, bb/aa/dd
     * symmetrised) held as one symmetric D x D matrix over global DOF indices:
     * the scan below reads mutual[type(u)type(v)][u][v] as M[u][v] */
    double *M = calloc((size_t)D * D + 1, sizeof(double));
    const int t1s[6] = {0, 0, 0, 1, 1, 2}, t2s[6] = {0, 1, 2, 1, 2, 2};
#pragma omp parallel for schedule(dynamic, 8)
    for (int i = 0; i < D; i++) {
        const int ti = i < nb ? 0 : (i < nb + na ? 1 : 2);
        for (int j = i + 1; j < D; j++) {
            const int tj = j < nb ? 0 : (j < nb + na ? 1 : 2);
            int q = 0;
            while (!(t1s[q] == ti && t2s[q] == tj)) q++;
            const double v = or_mutual(q, i - lo[ti], j - lo[tj], MARGS);
            M[(size_t)i * D + j] = v;
            M[(size_t)j * D + i] = v;
        }
    }

    double tB = 0, tA = 0, tD = 0;
    for (int k = 0; k < nb; k++) tB += s1_b[k];
    for (int k = 0; k < na; k++) tA += s1_a[k];
    for (int k = 0; k < nd; k++) tD += s1_d[k];

    int *In[3], *Out[3], nIn[3] = {0, 0, 0}, nOut[3];
    for (int t = 0; t < 3; t++) {
        In[t] = malloc(sizeof(int) * (cnt[t] + 1));
        Out[t] = malloc(sizeof(int) * (cnt[t] + 1));
        for (int i = 0; i < cnt[t]; i++) Out[t][i] = i;
        nOut[t] = cnt[t];
    }
    /* In = {bond 0}, get_PAR_MIST.cpp:419-422 */
    In[0][nIn[0]++] = Out[0][0];
    memmove(Out[0], Out[0] + 1, sizeof(int) * (nOut[0] - 1));
    nOut[0]--;

    double tm = 0, tpair[6] = {0};
    int step = 0;
    int maxthr = 1;
#ifdef _OPENMP
    maxthr = omp_get_max_threads();
#endif
    scan_best *part = malloc(sizeof(scan_best) * (size_t)maxthr);
    while (nOut[0] + nOut[1] + nOut[2] > 0) {
        /* The step's scan sequence, get_PAR_MIST.cpp:481-606: blocks (In type,
         * Out type) in the order BB BA BD AB AA AD DB DA DD, within a block In
         * position i then Out position j; the FIRST strict maximum wins. The
         * sequence is cut into one contiguous range per thread; merging the
         * ranges in order with the same strict '>' gives the serial result. */
        long long bsz[9], bstart[10];
        bstart[0] = 0;
        for (int b = 0; b < 9; b++) {
            bsz[b] = (long long)nIn[b / 3] * nOut[b % 3];
            bstart[b + 1] = bstart[b] + bsz[b];
        }
        const long long W = bstart[9];
        int nthr = 1;
#pragma omp parallel num_threads(maxthr)
        {
            const int t = omp_thread();
            const int nthr_here = omp_nthreads();
#pragma omp single
            nthr = nthr_here;
            /* the single's implied barrier: every thread sees the team size */
            const long long p0 = W * t / nthr_here, p1 = W * (t + 1) / nthr_here;
            scan_best r = {-1e200, -INFINITY, -1};
            long long pos = p0;
            int b = 0;
            while (b < 9 && bstart[b + 1] <= pos) b++;
            while (pos < p1 && b < 9) {
                if (bsz[b] == 0) { b++; continue; }
                const int ti = b / 3, to = b % 3, no = nOut[to];
                const long long off = pos - bstart[b];
                int i = (int)(off / no), j = (int)(off % no);
                const long long bend = bstart[b + 1] < p1 ? bstart[b + 1] : p1;
                for (; pos < bend; i++, j = 0) {
                    const double *row = M + (size_t)(lo[ti] + In[ti][i]) * D + lo[to];
                    const int *o = Out[to];
                    const int jend = (int)((bend - pos) < (no - j) ? j + (bend - pos) : no);
                    for (int jj = j; jj < jend; jj++) {
                        const double val = row[o[jj]];
                        if (val > r.best) {
                            if (r.at >= 0 && r.best > r.second) r.second = r.best;
                            r.best = val;
                            r.at = pos + (jj - j);
                        } else if (val > r.second) {
                            r.second = val;
                        }
                    }
                    pos += jend - j;
                }
                b++;
            }
            part[t] = r;
        }
        scan_best g = {-1e200, -INFINITY, -1};
        for (int t = 0; t < nthr; t++) {
            const scan_best r = part[t];
            if (r.at >= 0 && r.best > g.best) {
                if (g.at >= 0 && g.best > g.second) g.second = g.best;
                g.best = r.best;
                g.at = r.at;
            } else if (r.at >= 0 && r.best > g.second) {
                g.second = r.best;
            }
            if (r.second > g.second) g.second = r.second;
        }
        int bt1 = 0, bt2 = 0, bi = 0, bj = 0;
        double best = g.best;
        if (g.at >= 0) {
            int b = 0;
            while (bstart[b + 1] <= g.at) b++;
            bt1 = b / 3;
            bt2 = b % 3;
            bi = (int)((g.at - bstart[b]) / nOut[bt2]);
            bj = (int)((g.at - bstart[b]) % nOut[bt2]);
        }
        tm += best;
        edge_t1[step] = bt1;
        edge_t2[step] = bt2;
        edge_i1[step] = In[bt1][bi] + 1;
        edge_i2[step] = Out[bt2][bj] + 1;
        edge_mi[step] = best;
        edge_left[step] = nOut[0] + nOut[1] + nOut[2];
        if (edge_gap) edge_gap[step] = W > 1 ? best - g.second : INFINITY;
        In[bt2][nIn[bt2]++] = Out[bt2][bj];
        memmove(Out[bt2] + bj, Out[bt2] + bj + 1, sizeof(int) * (nOut[bt2] - bj - 1));
        nOut[bt2]--;
        const int lo2 = bt1 < bt2 ? bt1 : bt2, hi2 = bt1 < bt2 ? bt2 : bt1;
        const int q = lo2 == 0 ? hi2 : (lo2 == 1 ? 2 + hi2 : 5);
        tpair[q] += best;
        step++;
    }
    free(part);
    totals[0] = tB; totals[1] = tA; totals[2] = tD;
    for (int q = 0; q < 6; q++) totals[3 + q] = tpair[q];
    totals[9] = tB + tA + tD - tm;
    for (int t = 0; t < 3; t++) { free(In[t]); free(Out[t]); }
    free(M);
}

void or_mist(int n_dihedrals, const double *s1_b, const double *s1_a, const double *s1_d,
             const double *bb, const double *ba, const double *bd,
             const double *aa, const double *ad, const double *dd,
             int *edge_t1, int *edge_t2, int *edge_i1, int *edge_i2, double *edge_mi,
             int *edge_left, double totals[10]) {
    or_mist_gap(MARGS, edge_t1, edge_t2, edge_i1, edge_i2, edge_mi, edge_left, NULL, totals);
}

/* ------------------------------------------------------- BAT conversion */

/* One frame of BAT_Trajectory::convert_to_BAT (BAT_trajectory.cpp:219-300):
 * difference vectors in float (the coordinates are float), everything after
 * in double, in the reference's operation order. */
static void or_bat_frame(int nd, const float *x, const int *dih, double *rb0, double *rb1, double *ra,
                         double *bond, double *angle, double *dihe) {
    double b1[3], b2[3], b3[3], A[3], B[3];
    const int r0 = dih[0] - 1, r1 = dih[1] - 1, r2 = dih[2] - 1;
    for (int c = 0; c < 3; c++) {
        b2[c] = (double)(float)(x[3 * r1 + c] - x[3 * r0 + c]);  /* :235-237 */
        b3[c] = (double)(float)(x[3 * r2 + c] - x[3 * r1 + c]);  /* :239-241 */
    }
    *rb0 = sqrt(b2[0] * b2[0] + b2[1] * b2[1] + b2[2] * b2[2]);  /* :246 */
    *rb1 = sqrt(b3[0] * b3[0] + b3[1] * b3[1] + b3[2] * b3[2]);  /* :247 */
    *ra = acos((b2[0] * b3[0] + b2[1] * b3[1] + b2[2] * b3[2]) / *rb0 / *rb1);  /* :265 */
    for (int i = 0; i < nd; i++) {  /* :270-298 */
        const int *d = dih + 6 * i;
        const int a0 = d[0] - 1, a1 = d[1] - 1, a2 = d[2] - 1, a3 = d[3] - 1;
        for (int c = 0; c < 3; c++) {
            b1[c] = (double)(float)(x[3 * a1 + c] - x[3 * a0 + c]);
            b2[c] = (double)(float)(x[3 * a2 + c] - x[3 * a1 + c]);
            b3[c] = (double)(float)(x[3 * a3 + c] - x[3 * a2 + c]);
        }
        const double bl = sqrt(b3[0] * b3[0] + b3[1] * b3[1] + b3[2] * b3[2]);
        const double prev = sqrt(b2[0] * b2[0] + b2[1] * b2[1] + b2[2] * b2[2]);
        bond[i] = bl;
        angle[i] = acos((b2[0] * b3[0] + b2[1] * b3[1] + b2[2] * b3[2]) / bl / prev);
        A[0] = b1[1] * b2[2] - b1[2] * b2[1];
        A[1] = b1[2] * b2[0] - b1[0] * b2[2];
        A[2] = b1[0] * b2[1] - b1[1] * b2[0];
        B[0] = b2[1] * b3[2] - b2[2] * b3[1];
        B[1] = b2[2] * b3[0] - b2[0] * b3[2];
        B[2] = b2[0] * b3[1] - b2[1] * b3[0];
        dihe[i] = atan2((A[2] * B[0] - A[0] * B[2]) * b2[1] / prev - (A[2] * B[1] - A[1] * B[2]) * b2[0] / prev -
                            (A[1] * B[0] - A[0] * B[1]) * b2[2] / prev,
                        A[0] * B[0] + A[1] * B[1] + A[2] * B[2]);
    }
}

int or_bat_from_xyz(int nd, int nf, const float *xyz, const int *dih, double *bonds, double *angles,
                    double *dihedrals) {
    const int na = nd + 3;
    if (nd < 1 || nf < 1) return 1;
    for (int i = 0; i < nd; i++) {
        for (int k = 0; k < 4; k++)
            if (dih[6 * i + k] < 1 || dih[6 * i + k] > na) return 2;
        if (dih[6 * i + 5] != -1 && (dih[6 * i + 5] < 1 || dih[6 * i + 5] > nd)) return 3;
    }
    const double pi = acos(-1);  /* :51 */
    float *x = (float *)malloc(sizeof(float) * 3 * (size_t)na);
    double *bl = (double *)malloc(sizeof(double) * (size_t)nd * 3);
    double *an = bl + nd, *dh = bl + 2 * (size_t)nd;
    const size_t F = (size_t)nf;
    for (size_t f = 0; f < F; f++) {
        for (int j = 0; j < 3 * na; j++) x[j] = (float)(xyz[f * 3 * na + j] * 10.0);  /* :115-119 */
        double rb0, rb1, ra;
        or_bat_frame(nd, x, dih, &rb0, &rb1, &ra, bl, an, dh);
        for (int i = 0; i < nd; i++)  /* :303-310, in place */
            if (dih[6 * i + 5] != -1) dh[i] -= dh[dih[6 * i + 5] - 1];
        for (int i = 0; i < nd; i++)  /* :209-214 */
            dh[i] = dh[i] + 2 * pi - (double)((int)((dh[i] + 2 * pi) / (2 * pi)) * 2) * pi;
        bonds[0 * F + f] = rb0;  /* :121-123 */
        bonds[1 * F + f] = rb1;
        angles[0 * F + f] = ra;
        for (int i = 0; i < nd; i++) {
            bonds[(2 + (size_t)i) * F + f] = bl[i];
            angles[(1 + (size_t)i) * F + f] = an[i];
            dihedrals[(size_t)i * F + f] = dh[i];
        }
    }
    free(x);
    free(bl);
    return 0;
}
