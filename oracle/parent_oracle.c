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

int or_extrema(int n_dihedrals, int n_frames, double *bonds, double *angles, double *dihedrals,
               double *min_b, double *max_b, double *min_a, double *max_a,
               double *min_d, double *max_d, double *modfit) {
    const double pi = acos(-1); /* PARENT.cpp:112 */
    const int nb = n_dihedrals + 2, na = n_dihedrals + 1, nd = n_dihedrals;
    const size_t F = (size_t)n_frames;
    int bad = 0;
#pragma omp parallel for reduction(+ : bad) schedule(dynamic)
    for (int j = 0; j < nb; j++) { /* PARENT.cpp:511-536 */
        const double *x = bonds + j * F;
        double tmpMax = -1.0e100, tmpMin = 1.0e100;
        for (size_t i = 0; i < F; i++) {
            if (x[i] > tmpMax) tmpMax = x[i];
            if (x[i] < tmpMin) tmpMin = x[i];
        }
        if ((tmpMin < 0.0) || (tmpMax < 0.0)) bad++;
        tmpMin -= 0.000000005;
        tmpMax += 0.000000005;
        if (tmpMin < 0.0) tmpMin = 0.0;
        if ((tmpMax - tmpMin) < 1.0e-4) tmpMax += 0.05;
        max_b[j] = tmpMax;
        min_b[j] = tmpMin;
    }
#pragma omp parallel for schedule(dynamic)
    for (int j = 0; j < na; j++) { /* PARENT.cpp:538-562 */
        const double *x = angles + j * F;
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
        max_a[j] = tmpMax;
        min_a[j] = tmpMin;
    }
#pragma omp parallel for reduction(+ : bad) schedule(dynamic)
    for (int j = 0; j < nd; j++) { /* PARENT.cpp:564-637 */
        double *x = dihedrals + j * F;
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
        if (modfit) modfit[j] = modFit;
        for (size_t k = 0; k < F; k++)
            x[k] = x[k] + modFit - 2 * pi * (int)((x[k] + modFit) / (2 * pi));
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
        max_d[j] = tmpMax;
        min_d[j] = tmpMin;
    }
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

void or_mist(int n_dihedrals, const double *s1_b, const double *s1_a, const double *s1_d,
             const double *bb, const double *ba, const double *bd,
             const double *aa, const double *ad, const double *dd,
             int *edge_t1, int *edge_t2, int *edge_i1, int *edge_i2, double *edge_mi,
             int *edge_left, double totals[10]) {
    const int nb = n_dihedrals + 2, na = n_dihedrals + 1, nd = n_dihedrals;
    const int cnt[3] = {nb, na, nd};
    /* dense matrices, get_PAR_MIST.cpp:290-327: mutual[BB|AA|DD] symmetric,
     * mutual[BA] nb x na, mutual[BD] nb x nd, mutual[AD] na x nd */
    double *M[6];
    const int r[6] = {nb, nb, nb, na, na, nd}, c[6] = {nb, na, nd, na, nd, nd};
    for (int q = 0; q < 6; q++) M[q] = calloc((size_t)r[q] * c[q] + 1, sizeof(double));
    for (int i = 0; i < nb - 1; i++)
        for (int j = i + 1; j < nb; j++)
            M[0][(size_t)i * nb + j] = M[0][(size_t)j * nb + i] = or_mutual(0, i, j, MARGS);
    for (int i = 0; i < nb; i++)
        for (int j = 0; j < na; j++) M[1][(size_t)i * na + j] = or_mutual(1, i, j, MARGS);
    for (int i = 0; i < nb; i++)
        for (int j = 0; j < nd; j++) M[2][(size_t)i * nd + j] = or_mutual(2, i, j, MARGS);
    for (int i = 0; i < na - 1; i++)
        for (int j = i + 1; j < na; j++)
            M[3][(size_t)i * na + j] = M[3][(size_t)j * na + i] = or_mutual(3, i, j, MARGS);
    for (int i = 0; i < na; i++)
        for (int j = 0; j < nd; j++) M[4][(size_t)i * nd + j] = or_mutual(4, i, j, MARGS);
    for (int i = 0; i < nd - 1; i++)
        for (int j = i + 1; j < nd; j++)
            M[5][(size_t)i * nd + j] = M[5][(size_t)j * nd + i] = or_mutual(5, i, j, MARGS);

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
    /* block order BB BA BD AB AA AD DB DA DD, get_PAR_MIST.cpp:481-606 */
    int step = 0;
    while (nOut[0] + nOut[1] + nOut[2] > 0) {
        double best = -1e200;
        int bt1 = 0, bt2 = 0, bi = 0, bj = 0;
        for (int ti = 0; ti < 3; ti++)
            for (int to = 0; to < 3; to++)
                for (int i = 0; i < nIn[ti]; i++)
                    for (int j = 0; j < nOut[to]; j++) {
                        int u = In[ti][i], v = Out[to][j];
                        double val;
                        if (ti <= to) {
                            int q = ti == 0 ? to : (ti == 1 ? 2 + to : 5);
                            val = M[q][(size_t)u * c[q] + v];
                        } else {
                            int q = to == 0 ? ti : 4; /* (1,0)->BA, (2,0)->BD, (2,1)->AD */
                            val = M[q][(size_t)v * c[q] + u];
                        }
                        if (val > best) { best = val; bt1 = ti; bt2 = to; bi = i; bj = j; }
                    }
        tm += best;
        edge_t1[step] = bt1;
        edge_t2[step] = bt2;
        edge_i1[step] = In[bt1][bi] + 1;
        edge_i2[step] = Out[bt2][bj] + 1;
        edge_mi[step] = best;
        edge_left[step] = nOut[0] + nOut[1] + nOut[2];
        In[bt2][nIn[bt2]++] = Out[bt2][bj];
        memmove(Out[bt2] + bj, Out[bt2] + bj + 1, sizeof(int) * (nOut[bt2] - bj - 1));
        nOut[bt2]--;
        const int lo = bt1 < bt2 ? bt1 : bt2, hi = bt1 < bt2 ? bt2 : bt1;
        const int q = lo == 0 ? hi : (lo == 1 ? 2 + hi : 5);
        tpair[q] += best;
        step++;
    }
    totals[0] = tB; totals[1] = tA; totals[2] = tD;
    for (int q = 0; q < 6; q++) totals[3 + q] = tpair[q];
    totals[9] = tB + tA + tD - tm;
    for (int t = 0; t < 3; t++) { free(In[t]); free(Out[t]); }
    for (int q = 0; q < 6; q++) free(M[q]);
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
