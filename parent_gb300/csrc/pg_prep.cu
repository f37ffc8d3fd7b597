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
// The floors are read off the FP32 adder, not the conversion unit: for
// 0 <= v < 2^22, fl_rd(v + 2^23) = 2^23 + floor(v) exactly (the spacing of
// floats in [2^23, 2^24) is 1), whose bits minus those of 2^23 are floor(v).
__device__ __forceinline__ int screened_floor(float q, float eps) {
    const float lo = __fsub_rd(q, eps), hi = __fadd_ru(q, eps);
    const float yl = __fadd_rd(lo, 8388608.f), yh = __fadd_rd(hi, 8388608.f);
    return (lo >= 0.f && hi < 4194304.f && yl == yh) ? __float_as_int(yl) - 0x4B000000 : -1;
}

// (float)k for 0 <= k < 2^23, on the adder: the float with bits
// 0x4B000000 + k is exactly 2^23 + k
__device__ __forceinline__ float small_int_float(int k) { return __fsub_rn(__int_as_float(0x4B000000 + k), 8388608.f); }

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

// The same images for the input type: FP32 values keep 32-bit keys (the
// conversion to FP64 is exact and monotone, so the same values win; only the
// winners are converted), FP64 values the keys above.
template <typename T>
struct OKey;
template <>
struct OKey<float> {
    using K = unsigned int;
    static __device__ __forceinline__ K key(float x) {
        unsigned int b = __float_as_uint(x);
        if (b == 0x80000000u) b = 0u;
        return (b >> 31) ? ~b : (b | 0x80000000u);
    }
    static __device__ __forceinline__ bool nan(float x) { return (__float_as_uint(x) & 0x7fffffffu) > 0x7f800000u; }
    static __device__ __forceinline__ double value(unsigned long long k) {
        const unsigned int c = (unsigned int)k;
        return (double)__uint_as_float((c >> 31) ? (c & 0x7fffffffu) : ~c);
    }
    static constexpr K kNone = 0xffffffffu;
};
template <>
struct OKey<double> {
    using K = unsigned long long;
    static __device__ __forceinline__ K key(double x) { return okey_raw(x); }
    static __device__ __forceinline__ bool nan(double x) { return is_nan_bits(x); }
    static __device__ __forceinline__ double value(unsigned long long k) { return okey_double(k); }
    static constexpr K kNone = ~0ull;
};

// A column is streamed in runs of V = 16 / sizeof(T) consecutive frames, one
// 16-byte load each, with U runs per thread in flight: one CTA streams a
// column of up to millions of frames, and one 4-byte load in flight per
// thread left the kernel bound by memory latency.
template <typename T>
struct Run;
template <>
struct Run<float> {
    using V = float4;
    static constexpr int kN = 4;
    static __device__ __forceinline__ float at(const float4 &v, int k) {
        return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w));
    }
};
template <>
struct Run<double> {
    using V = double2;
    static constexpr int kN = 2;
    static __device__ __forceinline__ double at(const double2 &v, int k) { return k == 0 ? v.x : v.y; }
};

// run(f0, v) for every whole run this thread owns (f0 a multiple of kN when
// the column starts on a 16-byte boundary), fn(f, x) for the single frames
// before the first 16-byte boundary and after the last whole run.
template <int U, int NT, typename T, typename Fn, typename RunFn>
__device__ __forceinline__ void for_runs(const T *col, int F, int tid, Fn &&fn, RunFn &&run) {
    using R = Run<T>;
    using VT = typename R::V;
    const int head = min(F, (int)(((16u - ((unsigned)(uintptr_t)col & 15u)) & 15u) / sizeof(T)));
    if (tid < head) fn(tid, __ldg(col + tid));
    const VT *cv = (const VT *)(col + head);
    const int nv = (F - head) / R::kN;
    int i = tid;
    for (; i + (U - 1) * NT < nv; i += U * NT) {
        VT x[U];
#pragma unroll
        for (int u = 0; u < U; u++) x[u] = __ldg(cv + i + u * NT);
#pragma unroll
        for (int u = 0; u < U; u++) run(head + (i + u * NT) * R::kN, x[u]);
    }
    for (; i < nv; i += NT) run(head + i * R::kN, __ldg(cv + i));
    const int t = head + nv * R::kN + tid;  // fewer than kN frames are left
    if (t < F) fn(t, __ldg(col + t));
}

// fn(f, x) for every frame of the column, streamed as above
template <int U, int NT, typename T, typename Fn>
__device__ __forceinline__ void for_frames(const T *col, int F, int tid, Fn &&fn) {
    for_runs<U, NT>(col, F, tid, fn, [&](int f0, const typename Run<T>::V &v) {
#pragma unroll
        for (int k = 0; k < Run<T>::kN; k++) fn(f0 + k, Run<T>::at(v, k));
    });
}
constexpr int kUnroll = 2;
constexpr int kMinBlocks = 2;  // CTAs per SM (64 registers a thread)
constexpr int kTail = 256;  // bins per chunk of the per-DOF sums

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
        for_frames<kUnroll, kThreads>(colT, F, tid, [&](int, T xv) {
            const float x = (float)xv;
            const float q = __fmul_rn(x, rm);
            int idx = screened_floor(q, __fmul_ru(q, kQRel));
            if (idx < 0) idx = __double2int_rz(__ddiv_rn((double)xv, modfit_bs));
            if (idx < 0 || idx >= kModfitBins) { bad++; idx = idx < 0 ? 0 : kModfitBins - 1; }
            atomicAdd(&hmod[warp * kModfitBins + idx], 1u);
        });
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
    // exact quotient q of the shift of value xv: screened on its FP32
    // rounding, else FP64
    auto shift_q = [&](T xv, float &t32) -> int {
        t32 = __fadd_rn(__fadd_rn((float)xv, mf2.hi), mf2.lo);
        int q = screened_floor(__fmul_rn(t32, r2pi), kShiftEps);
        if (q < 0) q = shift_quot(__dadd_rn((double)xv, modfit), twopi);
        return q;
    };

    // ---- extrema (PARENT.cpp:512-521, 539-548, 614-623): the largest and
    // smallest input value of each shift-quotient region (exact: FP32 values
    // compare exactly as floats, FP64 values through their integer images),
    // then the shifted FP64 value of each candidate
    double lmax = -1.0e100, lmin = 1.0e100;
    {
        using Key = OKey<T>;
        using K = typename Key::K;
        K kmax[kRegions], kmin[kRegions];
        for (int r = 0; r < kRegions; r++) { kmax[r] = 0; kmin[r] = Key::kNone; }
        for_frames<kUnroll, kThreads>(colT, F, tid, [&](int, T xv) {
            int r = 0;
            if (type == TD) {
                float t32;
                r = shift_q(xv, t32);
                r = r < 0 ? 0 : (r >= kRegions ? kRegions - 1 : r);  // out of range: flagged above
            }
            const bool nan = Key::nan(xv);
            const K k = Key::key(xv);
#pragma unroll
            for (int q = 0; q < kRegions; q++) {
                if (q == r && !nan) {
                    kmax[q] = k > kmax[q] ? k : kmax[q];
                    kmin[q] = k < kmin[q] ? k : kmin[q];
                }
            }
        });
        __shared__ unsigned long long red_kmax[kWarps][kRegions], red_kmin[kWarps][kRegions];
        for (int q = 0; q < kRegions; q++) {
            for (int o = 16; o > 0; o >>= 1) {
                const K a = __shfl_xor_sync(0xffffffffu, kmax[q], o);
                const K b = __shfl_xor_sync(0xffffffffu, kmin[q], o);
                kmax[q] = a > kmax[q] ? a : kmax[q];
                kmin[q] = b < kmin[q] ? b : kmin[q];
            }
            if (lane == 0) { red_kmax[warp][q] = kmax[q]; red_kmin[warp][q] = kmin[q]; }
        }
        __syncthreads();
        if (tid == 0) {
            for (int q = 0; q < kRegions; q++) {
                unsigned long long a = 0ull, b = Key::kNone;
                for (int w = 0; w < kWarps; w++) {
                    a = red_kmax[w][q] > a ? red_kmax[w][q] : a;
                    b = red_kmin[w][q] < b ? red_kmin[w][q] : b;
                }
                if (a < b) continue;  // empty region
                double va = Key::value(a), vb = Key::value(b);
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
        // both bin indices of one value, counted in the 1D histograms; the 2D
        // bin is returned for the pair kernels' bin matrices
        auto bin_of = [&](T xin) -> int {
            const float x = (float)xin;
            float d32;
            int q = 0;
            if (type == TD) {
                float t32;
                q = shift_q(xin, t32);
                const float qf = q >= 0 ? small_int_float(q) : (float)q;
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
            return i2;
        };
        // every bin matrix of the layout the pair kernels read: a whole run
        // in one store per matrix where it starts on a multiple of its length
        for_runs<kUnroll, kThreads>(
            colT, F, tid, [&](int f, T xin) { store_bin(bins, geo, g, f, bin_of(xin)); },
            [&](int f0, const typename Run<T>::V &v) {
                int b[Run<T>::kN];
#pragma unroll
                for (int k = 0; k < Run<T>::kN; k++) b[k] = bin_of(Run<T>::at(v, k));
                if ((f0 & (Run<T>::kN - 1)) == 0) {
                    store_bin_run<Run<T>::kN>(bins, geo, g, f0, b);
                } else {
#pragma unroll
                    for (int k = 0; k < Run<T>::kN; k++) store_bin(bins, geo, g, f0 + k, b[k]);
                }
            });
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

    // ---- per-DOF sums on warp 0: lane 0 runs the reference's sequential
    // recurrences and sums, the 32 lanes take the per-bin logarithms and
    // sines (each FP64 warp instruction costs the same with 1 or 32 lanes
    // active, and the FP64 pipe is a small fraction of this part's rate)
    if (warp == 0) {
        __shared__ double s_x[kTail], s_t[kTail];
        __shared__ unsigned char s_f[kTail];
        const int N = F;
        // lane 0: x_k = x_{k-1} + step for the bins [c0, c0 + n) (the
        // reference's repeated +=, carried across chunks in x)
        auto points = [&](double &x, double step, int n) {
            if (lane == 0)
                for (int k = 0; k < n; k++) {
                    s_x[k] = x;
                    x = __dadd_rn(x, step);
                }
            __syncwarp();
        };
        // lane 0: sum of the flagged terms in bin order, counting them
        auto sum_terms = [&](double &sum, int &count, int n) {
            __syncwarp();
            if (lane == 0)
                for (int k = 0; k < n; k++)
                    if (s_f[k]) {
                        sum = sum + s_t[k];
                        count++;
                    }
            __syncwarp();
        };

        // 1D entropy in the reference's order (PARENT.cpp:658-670, 702-714, 746-756)
        int occupbins = 0;
        double plnpsum = 0.0, x1 = __dadd_rn(mn, bs1 / 2.0);
        for (int c0 = 0; c0 < B1; c0 += kTail) {
            const int n = min(kTail, B1 - c0);
            if (type != TD) points(x1, bs1, n);
            for (int k = lane; k < n; k += 32) {
                const double h = (double)h1[c0 + k];
                double probDens, t = 0.0;
                if (type == TB) {
                    const double blen = s_x[k];
                    probDens = h / (((N * bs1) * blen) * blen);
                    if (probDens > 0) t = ((blen * blen) * probDens) * log(probDens);
                } else if (type == TA) {
                    const double st = sin(s_x[k]);
                    probDens = h / ((N * bs1) * st);
                    if (probDens > 0) t = (st * probDens) * log(probDens);
                } else {
                    probDens = h / (N * bs1);
                    if (probDens > 0) t = probDens * log(probDens);
                }
                s_t[k] = t;
                s_f[k] = probDens > 0;
            }
            sum_terms(plnpsum, occupbins, n);
        }

        // A = ln(bs2) + (1/N) sum_k m(k) ln J(c_k), with c_k advanced by
        // repeated += binsize as the reference's 2D epilogues do
        // (e.g. PARENT.cpp:807-820); J = c^2 (bond), sin c (angle), 1 (dihedral).
        double acc = 0.0, x2 = __dadd_rn(mn, bs2 / 2.0);
        int unused = 0;
        unsigned int m2 = 0;
        for (int c0 = 0; c0 < B2; c0 += kTail) {
            const int n = min(kTail, B2 - c0);
            if (type != TD) points(x2, bs2, n);
            for (int k = lane; k < n; k += 32) {
                const unsigned int h = h2[c0 + k];
                m2 = h > m2 ? h : m2;
                if (type != TD && h) {
                    const double c = s_x[k];
                    s_t[k] = (double)h * (type == TB ? log(c * c) : log(sin(c)));
                }
                s_f[k] = type != TD && h != 0u;
            }
            sum_terms(acc, unused, n);
        }
        // largest 2D-bin marginal count: no 2D bin of a pair with this DOF
        // can hold more frames
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned int v = __shfl_xor_sync(0xffffffffu, m2, o);
            m2 = v > m2 ? v : m2;
        }
        if (lane == 0) {
            dof.m2[g] = (int)m2;
            plnpsum = -plnpsum * bs1;
            dof.s1[g] = plnpsum + (occupbins - 1.0) / (2.0 * N);
            dof.acon[g] = log(bs2) + acc / (double)N;
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(kThreads, kMinBlocks) prep_kernel(SysGeom geo, const void *cb, const void *ca, const void *cd,
                                                        int64_t ld, int prec, DofArrays dof, uint8_t *bins, int *err,
                                                        double modfit_bs, double pi, int g_first, int h1_copies) {
    prep_body<T>(geo, cb, ca, cd, ld, prec, dof, bins, err, modfit_bs, pi, g_first + blockIdx.x, h1_copies);
}

// Many systems in one launch: CTA k preprocesses DOF map[k].y of system
// map[k].x (systems of one input precision per launch).
template <typename T>
__global__ void __launch_bounds__(kThreads, kMinBlocks) prep_batch_kernel(const PrepDesc *__restrict__ sys,
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
