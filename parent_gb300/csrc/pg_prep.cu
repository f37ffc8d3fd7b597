// Per-DOF preprocessing: one CTA per DOF.
//   pass 1 (dihedrals only): 100-bin occupancy histogram and the "modfit"
//           shift that moves the longest empty stretch to 2 pi (PARENT.cpp:564-612)
//   pass 2: extrema of the (shifted) column, padding and clamps (PARENT.cpp:511-636)
//   pass 3: uint8 bin index at the 2D bin count for every frame (the pair
//           kernels' input), 1D histogram at the 1D bin count and the marginal
//           at the 2D bin count; then the 1D entropy (PARENT.cpp:650-757) and the
//           per-DOF constant A of the 2D entropy decomposition.
//
// Bit-exactness: every FP64 operation that decides a bin index is written
// with explicit round-to-nearest intrinsics (no FMA contraction), and this
// file is compiled with --fmad=false, so bin indices equal the reference's
// int((x - min) / binsize) on x86-64 (which never fuses).
#include <math.h>

#include "pg_internal.h"

namespace pg {

namespace {

constexpr int kThreads = 512;
constexpr int kWarps = kThreads / 32;
constexpr int kModfitBins = 100;  // PARENT.cpp:51

// q = int((x + modFit) / (2 pi)) and x + modFit - 2 pi q, PARENT.cpp:611,
// evaluated as the reference's left-to-right expression without contraction.
__device__ __forceinline__ int shift_quot(double t, double twopi) { return __double2int_rz(__ddiv_rn(t, twopi)); }
__device__ __forceinline__ double shift_apply(double t, int q, double twopi) {
    return __dsub_rn(t, __dmul_rn(twopi, (double)q));
}
__device__ __forceinline__ double shifted(double x, double modfit, double twopi) {
    const double t = __dadd_rn(x, modfit);
    return shift_apply(t, shift_quot(t, twopi), twopi);
}

__device__ __forceinline__ int bin_index(double x, double mn, double bs) {
    return __double2int_rz(__ddiv_rn(__dsub_rn(x, mn), bs));
}

// ---- FP32 screening of the FP64 bin decisions (FP32 input only).
// Every decision above is int(q*) for a quotient q* = fl64(a / b) >= 0. The
// screen forms q ~ q* in FP32 with a proven bound |q - q*| <= eps (from the
// operands' magnitudes; every bound below carries a factor >= 4 of slack) and
// accepts floor(q) only when no integer lies within eps of q; otherwise the
// caller evaluates q* with the exact FP64 expression. The result is therefore
// the reference's integer in every case; the FP64 pipe, a small fraction of
// this part's FP32 rate, only sees the values that fall next to a boundary.

// floor(q) if [q - eps, q + eps] (directed rounding) holds no integer and
// q - eps >= 0, else -1 (also for NaN).
__device__ __forceinline__ int screened_floor(float q, float eps) {
    const float lo = __fsub_rd(q, eps), hi = __fadd_ru(q, eps);
    const int il = __float2int_rd(lo), ih = __float2int_rd(hi);
    return (lo >= 0.f && il == ih) ? il : -1;
}

// v ~ hi + lo as two floats (|v - hi - lo| <= 2^-48 |v|)
struct F2 {
    float hi, lo;
};
__device__ __forceinline__ F2 split2(double v) {
    const float hi = __double2float_rn(v);
    return {hi, __double2float_rn(__dsub_rn(v, (double)hi))};
}

// Extrema of a dihedral column after the shift: within one value of
// q = int((x + modFit) / 2 pi) the shifted value is a non-decreasing function
// of x (FP64 rounding is monotone), so the largest / smallest x of each q
// region gives that region's extreme shifted value.
constexpr int kRegions = 3;  // x in [0, 2 pi + 5e-9) and modFit in (0, 2 pi] give q in {0, 1, 2}

// Order-preserving 64-bit image of a double for exact extrema on the
// integer pipe (NaN mapped below everything for maxima, above for minima, so
// it never wins either, as with the reference's strict comparisons).
__device__ __forceinline__ unsigned long long okey_raw(double x) {
    unsigned long long b = (unsigned long long)__double_as_longlong(x);
    if (b == 0x8000000000000000ull) b = 0ull;  // -0 == +0
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ bool is_nan_bits(double x) {
    return ((unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull) > 0x7ff0000000000000ull;
}
__device__ __forceinline__ double okey_double(unsigned long long k) {
    const unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    return __longlong_as_double((long long)b);
}

// One CTA's work on DOF g of one system; T is the input element type (float
// or double). Every bin decision is screened in FP32 (see above) with an
// exact FP64 fallback; FP64 inputs enter the screen rounded to FP32, an
// error the bounds below include.
template <typename T>
__device__ __forceinline__ void prep_body(const SysGeom &geo, const void *cb, const void *ca, const void *cd,
                                          int64_t ld, int prec, const DofArrays &dof, uint8_t *bins, int *err,
                                          double modfit_bs, double pi, int g, int h1_copies) {
    extern __shared__ unsigned int sh[];
    const int type = dof_type(g, geo.nb, geo.na);
    const int local = g - (type == TB ? 0 : (type == TA ? geo.nb : geo.nb + geo.na));
    const void *col = type == TB ? cb : (type == TA ? ca : cd);
    col = prec ? (const void *)((const double *)col + (int64_t)local * ld)
               : (const void *)((const float *)col + (int64_t)local * ld);
    const T *colT = (const T *)col;
    constexpr bool kDbl = sizeof(T) == 8;
    // relative error bound factor of an FP32 quotient: 3 roundings (2^-23)
    // for FP32 input, 4 for FP64 input rounded to FP32; both under 1/4 of it
    constexpr float kQRel = kDbl ? 0x1p-20f : 0x1p-21f;
    const int F = geo.F;
    const int B1 = geo.bins[type], B2 = geo.bins[3 + type];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const double twopi = 2 * pi;

    // shared layout: [kWarps][kModfitBins] | [kWarps][B1] | [kWarps][B2] | scalars
    unsigned int *hmod = sh;
    unsigned int *h1 = hmod + kWarps * kModfitBins;
    unsigned int *h2 = h1 + h1_copies * B1;  // per-warp 1D histograms, or one shared copy for large B1
    const int w1 = h1_copies > 1 ? warp : 0;
    __shared__ double s_shift, s_mn, s_mx;
    __shared__ double red_mn[kWarps], red_mx[kWarps];

    double modfit = 0.0;
    if (type == TD) {
        for (int k = tid; k < kWarps * kModfitBins; k += kThreads) hmod[k] = 0;
        __syncthreads();
        int bad = 0;
        // x / modfit_bs: relative error of x32 * fl32(1/bs) <= 2^-23 (2^-22.4
        // with the FP32 rounding of an FP64 input)
        const float rm = __double2float_rn(__drcp_rn(modfit_bs));
        for (int f = tid; f < F; f += kThreads) {
            const T xv = __ldg(colT + f);
            const float x = (float)xv;
            const float q = __fmul_rn(x, rm);
            int idx = screened_floor(q, __fmul_ru(q, kQRel));
            if (idx < 0) idx = __double2int_rz(__ddiv_rn((double)xv, modfit_bs));
            if (idx < 0 || idx >= kModfitBins) { bad++; idx = idx < 0 ? 0 : kModfitBins - 1; }
            atomicAdd(&hmod[warp * kModfitBins + idx], 1u);
        }
        if (bad) atomicAdd(&err[ERR_MODFIT_RANGE], bad);
        __syncthreads();
        for (int k = tid; k < kModfitBins; k += kThreads) {
            unsigned int s = 0;
            for (int w = 0; w < kWarps; w++) s += hmod[w * kModfitBins + k];
            hmod[k] = s;  // warp 0's row only read by thread k itself before this write
        }
        __syncthreads();
        if (tid == 0) {
            // longest circular stretch of empty bins, or the first minimum bin
            // when none is empty (PARENT.cpp:573-608, including the run
            // counter that starts at 2 because of the double increment)
            const unsigned int *histo = hmod;
            bool zeroExists = false;
            for (int k = 0; k < kModfitBins; k++) zeroExists = zeroExists || (histo[k] == 0);
            int longest = 0, longestPos = -1, cur = 0, curPos = 0;
            if (zeroExists) {
                for (int k = 0; k < 2 * kModfitBins; k++) {
                    const int l = k % kModfitBins;
                    if (cur == 0 && histo[l] == 0) { cur = 1; curPos = k; }
                    if (cur > 0 && histo[l] == 0) cur += 1;
                    if (cur > 0 && histo[l] != 0) {
                        if (cur > longest) { longest = cur; longestPos = curPos; }
                        cur = 0;
                    }
                }
            } else {
                longestPos = 0;
                unsigned int mn = histo[0];
                for (int k = 0; k < kModfitBins; k++)
                    if (histo[k] < mn) { mn = histo[k]; longestPos = k; }
            }
            // modFit = 2 pi - (pos + 0.5) * binsize, PARENT.cpp:609
            s_shift = __dsub_rn(twopi, __dmul_rn(__dadd_rn((double)longestPos, 0.5), modfit_bs));
        }
        __syncthreads();
        modfit = s_shift;
    }

    // FP32 images of the shift constants; t = x + modFit and its quotient by
    // 2 pi are screened with |t32 - t| <= 2^-23 (|x| + |modFit|) <= 2e-6 and
    // |q - t / 2 pi| <= 8e-7 for x < 2 pi + 5e-9, modFit <= 2 pi
    const F2 mf2 = split2(modfit), tp2 = split2(twopi);
    const float r2pi = __double2float_rn(__drcp_rn(twopi));
    constexpr float kShiftEps = 4e-6f;
    // exact quotient q of the shift of value xd (x = its FP32 rounding):
    // screened, else FP64
    auto shift_q = [&](float x, double xd, float &t32) -> int {
        t32 = __fadd_rn(__fadd_rn(x, mf2.hi), mf2.lo);
        int q = screened_floor(__fmul_rn(t32, r2pi), kShiftEps);
        if (q < 0) q = shift_quot(__dadd_rn(xd, modfit), twopi);
        return q;
    };

    // ---- extrema (PARENT.cpp:512-521, 539-548, 614-623): the largest and
    // smallest input value of each shift-quotient region (exact: FP32 values
    // compare exactly as floats, FP64 values through their integer images),
    // then the shifted FP64 value of each candidate
    double lmax = -1.0e100, lmin = 1.0e100;
    {
        unsigned long long kmax[kRegions], kmin[kRegions];
        for (int r = 0; r < kRegions; r++) { kmax[r] = 0ull; kmin[r] = ~0ull; }
        for (int f = tid; f < F; f += kThreads) {
            const T xv = __ldg(colT + f);
            const double xd = (double)xv;
            int r = 0;
            if (type == TD) {
                float t32;
                r = shift_q((float)xv, xd, t32);
                r = r < 0 ? 0 : (r >= kRegions ? kRegions - 1 : r);  // out of range: flagged above
            }
            const bool nan = is_nan_bits(xd);
            const unsigned long long k = okey_raw(xd);
#pragma unroll
            for (int q = 0; q < kRegions; q++) {
                if (q == r && !nan) {
                    kmax[q] = k > kmax[q] ? k : kmax[q];
                    kmin[q] = k < kmin[q] ? k : kmin[q];
                }
            }
        }
        __shared__ unsigned long long red_kmax[kWarps][kRegions], red_kmin[kWarps][kRegions];
        for (int q = 0; q < kRegions; q++) {
            for (int o = 16; o > 0; o >>= 1) {
                const unsigned long long a = __shfl_xor_sync(0xffffffffu, kmax[q], o);
                const unsigned long long b = __shfl_xor_sync(0xffffffffu, kmin[q], o);
                kmax[q] = a > kmax[q] ? a : kmax[q];
                kmin[q] = b < kmin[q] ? b : kmin[q];
            }
            if (lane == 0) { red_kmax[warp][q] = kmax[q]; red_kmin[warp][q] = kmin[q]; }
        }
        __syncthreads();
        if (tid == 0) {
            for (int q = 0; q < kRegions; q++) {
                unsigned long long a = 0ull, b = ~0ull;
                for (int w = 0; w < kWarps; w++) {
                    a = red_kmax[w][q] > a ? red_kmax[w][q] : a;
                    b = red_kmin[w][q] < b ? red_kmin[w][q] : b;
                }
                if (a < b) continue;  // empty region
                double va = okey_double(a), vb = okey_double(b);
                if (type == TD) {
                    va = shifted(va, modfit, twopi);
                    vb = shifted(vb, modfit, twopi);
                }
                if (va > lmax) lmax = va;
                if (vb < lmin) lmin = vb;
            }
            red_mx[0] = lmax;
            red_mn[0] = lmin;
        }
    }
    __syncthreads();
    if (tid == 0) {
        double tmpMax = -1.0e100, tmpMin = 1.0e100;
        for (int w = 0; w < 1; w++) {
            if (red_mx[w] > tmpMax) tmpMax = red_mx[w];
            if (red_mn[w] < tmpMin) tmpMin = red_mn[w];
        }
        if (type == TB && ((tmpMin < 0.0) || (tmpMax < 0.0))) atomicAdd(&err[ERR_NEG_BOND], 1);
        tmpMin = __dsub_rn(tmpMin, 0.000000005);
        tmpMax = __dadd_rn(tmpMax, 0.000000005);
        if (tmpMin < 0.0) tmpMin = 0.0;
        if (type == TA && tmpMax > pi) tmpMax = pi;
        if (type == TD && tmpMax > twopi) tmpMax = twopi;
        if (__dsub_rn(tmpMax, tmpMin) < 1.0e-4) tmpMax = __dadd_rn(tmpMax, 0.05);
        s_mn = tmpMin;
        s_mx = tmpMax;
        dof.mn[g] = tmpMin;
        dof.mx[g] = tmpMax;
        dof.shift[g] = modfit;
        dof.b2[g] = B2;
    }
    for (int k = tid; k < h1_copies * B1 + kWarps * B2; k += kThreads) h1[k] = 0;
    __syncthreads();

    // ---- binning (PARENT.cpp:654-656 1D; :800-803 and the other 2D fills)
    const double mn = s_mn, mx = s_mx;
    const double bs1 = __ddiv_rn(__dsub_rn(mx, mn), (double)B1);
    const double bs2 = __ddiv_rn(__dsub_rn(mx, mn), (double)B2);
    int bad = 0;
    {
        // d = fl64(x' - mn) (x' the shifted value for dihedrals) is formed in
        // FP32 from split constants, |d32 - d| <= 2^-20 E with
        // E = |mn| + |mx| (+ 2|modFit| + 8 pi for dihedrals), a bound >= 4x
        // the accumulated rounding (including an FP64 input's rounding to
        // FP32, <= 2^-24 E); q_k = d32 * fl32(1 / bs_k) then has
        // |q_k - q*| <= 2^-20 E / bs_k + 2^-22 q_k.
        const F2 mn2 = split2(mn);
        const float r1 = __double2float_rn(__drcp_rn(bs1)), r2 = __double2float_rn(__drcp_rn(bs2));
        double E = fabs(mn) + fabs(mx);
        if (type == TD) E = E + 2.0 * fabs(modfit) + 4.0 * twopi;
        const float e1 = __double2float_ru(E * 0x1p-20 / bs1), e2 = __double2float_ru(E * 0x1p-20 / bs2);
        for (int f = tid; f < F; f += kThreads) {
            const T xin = __ldg(colT + f);
            const float x = (float)xin;
            float d32;
            int q = 0;
            if (type == TD) {
                float t32;
                q = shift_q(x, (double)xin, t32);
                const float qf = (float)q;
                d32 = __fsub_rn(__fsub_rn(__fsub_rn(__fsub_rn(t32, __fmul_rn(qf, tp2.hi)), __fmul_rn(qf, tp2.lo)),
                                          mn2.hi),
                                mn2.lo);
            } else {
                d32 = __fsub_rn(__fsub_rn(x, mn2.hi), mn2.lo);
            }
            const float q1 = __fmul_rn(d32, r1), q2 = __fmul_rn(d32, r2);
            int i1 = screened_floor(q1, __fadd_ru(e1, __fmul_ru(fabsf(q1), kQRel)));
            int i2 = screened_floor(q2, __fadd_ru(e2, __fmul_ru(fabsf(q2), kQRel)));
            if (i1 < 0 || i2 < 0) {
                double xv = (double)xin;
                if (type == TD) xv = shift_apply(__dadd_rn(xv, modfit), q, twopi);
                if (i1 < 0) i1 = bin_index(xv, mn, bs1);
                if (i2 < 0) i2 = bin_index(xv, mn, bs2);
            }
            if (i1 < 0 || i1 >= B1) { bad++; i1 = i1 < 0 ? 0 : B1 - 1; }
            if (i2 < 0 || i2 >= B2) { bad++; i2 = i2 < 0 ? 0 : B2 - 1; }
            atomicAdd(&h1[w1 * B1 + i1], 1u);
            atomicAdd(&h2[warp * B2 + i2], 1u);
            // every bin matrix of the layout the pair kernel reads
            store_bin(bins, geo, g, f, i2);
        }
    }
    if (bad) atomicAdd(&err[ERR_BIN_RANGE], bad);
    __syncthreads();
    for (int k = tid; k < B1 + B2; k += kThreads) {
        unsigned int *h = k < B1 ? h1 : h2;
        const int kk = k < B1 ? k : k - B1, stride = k < B1 ? B1 : B2;
        const int copies = k < B1 ? h1_copies : kWarps;
        unsigned int s = 0;
        for (int w = 0; w < copies; w++) s += h[w * stride + kk];
        h[kk] = s;
    }
    __syncthreads();

    if (tid == 0) {
        // largest 2D-bin marginal count: no 2D bin of a pair with this DOF
        // can hold more frames
        unsigned int m2 = 0;
        for (int k = 0; k < B2; k++) m2 = h2[k] > m2 ? h2[k] : m2;
        dof.m2[g] = (int)m2;

        // 1D entropy in the reference's order (PARENT.cpp:658-670, 702-714, 746-756)
        const int N = F;
        int occupbins = 0;
        double plnpsum = 0.0, probDens;
        if (type == TB) {
            double blen = __dadd_rn(mn, bs1 / 2.0);
            for (int k = 0; k < B1; k++) {
                probDens = (double)h1[k] / (((N * bs1) * blen) * blen);
                if (probDens > 0) {
                    plnpsum = plnpsum + ((blen * blen) * probDens) * log(probDens);
                    occupbins++;
                }
                blen = __dadd_rn(blen, bs1);
            }
        } else if (type == TA) {
            double theta = __dadd_rn(mn, bs1 / 2.0);
            for (int k = 0; k < B1; k++) {
                const double st = sin(theta);
                probDens = (double)h1[k] / ((N * bs1) * st);
                if (probDens > 0) {
                    plnpsum = plnpsum + (st * probDens) * log(probDens);
                    occupbins++;
                }
                theta = __dadd_rn(theta, bs1);
            }
        } else {
            for (int k = 0; k < B1; k++) {
                probDens = (double)h1[k] / (N * bs1);
                if (probDens > 0) {
                    plnpsum = plnpsum + probDens * log(probDens);
                    occupbins++;
                }
            }
        }
        plnpsum = -plnpsum * bs1;
        dof.s1[g] = plnpsum + (occupbins - 1.0) / (2.0 * N);

        // A = ln(bs2) + (1/N) sum_k m(k) ln J(c_k), with c_k advanced by
        // repeated += binsize as the reference's 2D epilogues do
        // (e.g. PARENT.cpp:807-820); J = c^2 (bond), sin c (angle), 1 (dihedral).
        double acc = 0.0;
        if (type != TD) {
            double c = __dadd_rn(mn, bs2 / 2.0);
            for (int k = 0; k < B2; k++) {
                if (h2[k]) acc += (double)h2[k] * (type == TB ? log(c * c) : log(sin(c)));
                c = __dadd_rn(c, bs2);
            }
        }
        dof.acon[g] = log(bs2) + acc / (double)N;
    }
}

template <typename T>
__global__ void __launch_bounds__(kThreads) prep_kernel(SysGeom geo, const void *cb, const void *ca, const void *cd,
                                                        int64_t ld, int prec, DofArrays dof, uint8_t *bins, int *err,
                                                        double modfit_bs, double pi, int g_first, int h1_copies) {
    prep_body<T>(geo, cb, ca, cd, ld, prec, dof, bins, err, modfit_bs, pi, g_first + blockIdx.x, h1_copies);
}

// Many systems in one launch: CTA k preprocesses DOF map[k].y of system
// map[k].x (systems of one input precision per launch).
template <typename T>
__global__ void __launch_bounds__(kThreads) prep_batch_kernel(const PrepDesc *__restrict__ sys,
                                                              const int2 *__restrict__ map, int *err,
                                                              double modfit_bs, double pi, int h1_copies) {
    const int2 m = map[blockIdx.x];
    const PrepDesc &d = sys[m.x];
    prep_body<T>(d.geo, d.cols[0], d.cols[1], d.cols[2], d.ld, d.prec, d.dof, d.bins, err, modfit_bs, pi, m.y,
                   h1_copies);
}

__global__ void nlogn_kernel(double *t, int nmax) {
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n <= nmax; n += gridDim.x * blockDim.x)
        t[n] = n > 1 ? (double)n * log((double)n) : 0.0;
}

__global__ void nlogn_fix_kernel(unsigned long long *t, int nmax, double fix) {
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n <= nmax; n += gridDim.x * blockDim.x)
        t[n] = n > 1 ? __double2ull_rn((double)n * log((double)n) * fix) : 0ull;  // unsigned: entries reach 1.6e19
}

}  // namespace

cudaError_t launch_nlogn_fix_table(unsigned long long *nfix, int nmax, double fix, cudaStream_t st) {
    int blocks = (nmax + 1 + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    nlogn_fix_kernel<<<blocks, 256, 0, st>>>(nfix, nmax, fix);
    return cudaGetLastError();
}

cudaError_t launch_nlogn_table(double *nlogn, int nmax, cudaStream_t st) {
    int blocks = (nmax + 1 + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    nlogn_kernel<<<blocks, 256, 0, st>>>(nlogn, nmax);
    return cudaGetLastError();
}

// Per-warp private 1D histograms where they fit in 200 KB with the others,
// one shared copy otherwise (up to 16,384 1D bins).
static int prep_h1_copies(const SysGeom &g, int *m1_out, int *m2_out) {
    int m1 = 0, m2 = 0;
    for (int t = 0; t < 3; t++) {
        if (g.bins[t] > m1) m1 = g.bins[t];
        if (g.bins[3 + t] > m2) m2 = g.bins[3 + t];
    }
    *m1_out = m1;
    *m2_out = m2;
    return (size_t)kWarps * (kModfitBins + m1 + m2) * sizeof(unsigned int) <= 200 * 1024 ? kWarps : 1;
}

size_t prep_smem_bytes(const SysGeom &g) {
    int m1 = 0, m2 = 0;
    const int c1 = prep_h1_copies(g, &m1, &m2);
    return ((size_t)kWarps * (kModfitBins + m2) + (size_t)c1 * m1) * sizeof(unsigned int);
}

cudaError_t launch_prep(const SysGeom &g, const void *const cols[3], int64_t ld, int double_prec,
                        DofArrays dof, uint8_t *bins, int *err, cudaStream_t st, int g_first, int g_count) {
    if (g_count < 0) g_count = g.D - g_first;
    if (g_first < 0 || g_first + g_count > g.D) return cudaErrorInvalidValue;
    if (g_count == 0) return cudaSuccess;
    const double pi = acos(-1.0);  // PARENT.cpp:112
    const double modfit_bs = (2 * pi + 0.000000005) / kModfitBins;  // PARENT.cpp:569
    const size_t smem = prep_smem_bytes(g);
    auto kern = double_prec ? prep_kernel<double> : prep_kernel<float>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int m1 = 0, m2 = 0;
    const int c1 = prep_h1_copies(g, &m1, &m2);
    kern<<<g_count, kThreads, smem, st>>>(g, cols[0], cols[1], cols[2], ld, double_prec, dof, bins, err, modfit_bs,
                                          pi, g_first, c1);
    return cudaGetLastError();
}

cudaError_t launch_prep_batch(const SysGeom &bins_of, const PrepDesc *sys, const int2 *map, int n_cta,
                              int double_prec, int *err, cudaStream_t st) {
    if (n_cta <= 0) return cudaSuccess;
    const double pi = acos(-1.0);  // PARENT.cpp:112
    const double modfit_bs = (2 * pi + 0.000000005) / kModfitBins;  // PARENT.cpp:569
    const size_t smem = prep_smem_bytes(bins_of);
    int m1 = 0, m2 = 0;
    const int c1 = prep_h1_copies(bins_of, &m1, &m2);
    auto kern = double_prec ? prep_batch_kernel<double> : prep_batch_kernel<float>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<n_cta, kThreads, smem, st>>>(sys, map, err, modfit_bs, pi, c1);
    return cudaGetLastError();
}

}  // namespace pg
