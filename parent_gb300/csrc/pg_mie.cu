// MIE text on the device: the 2D lines of get_PAR_MIE.x (get_PAR_MIE.cpp:
// 109-199), "<pair type> i  j   S2D   MI\n" for every DOF pair in the
// reference's line order, with S2D from the .par body (same-type blocks
// walked from the end of their reversed triangle, :123-131) and MI from
// get_mutual (util.cpp:47-81: S1[i] + S1[j] - S2D, left to right), both
// printed with %.12g (pg_fmt.h, byte-identical to the C library's).
//
// Four kernels:
//   mie_format_kernel  one CTA per row (i) of a pair block; every thread
//                      writes its lines into fixed 96-byte slots and their
//                      lengths; a value outside the exact formatter's range
//                      leaves the line to the host (listed, length 0);
//   mie_rowlen_kernel  one CTA per row: the row's text length;
//   mie_scan_rows_kernel  row offsets (one CTA of 1,024 threads);
//   mie_compact_kernel    every row packs its slots into the output text in
//                         line order.
#include <stdint.h>

#include <cuda_runtime.h>

#include "pg_fmt.h"
#include "pg_internal.h"

namespace pg {

namespace {

constexpr int kRowThreads = 128;

__device__ __forceinline__ char *put_str(char *p, const char *s, int n) {
    for (int k = 0; k < n; k++) p[k] = s[k];
    return p + n;
}
__device__ __forceinline__ char *put_int(char *p, int v) {  // v >= 1
    char t[12];
    int n = 0;
    while (v) {
        t[n++] = (char)('0' + v % 10);
        v /= 10;
    }
    while (n) *p++ = t[--n];
    return p;
}

// global row r -> (block q, row i inside it)
__device__ __forceinline__ void row_of(const MieArgs &a, int r, int &q, int &i) {
    q = 0;
    while (q < 5 && r >= a.row0[q + 1]) q++;  // empty blocks have row0[q] == row0[q + 1]
    i = r - a.row0[q];
}

__device__ __forceinline__ int64_t row_lines(const MieArgs &a, int q, int i, int64_t *first) {
    const int64_t n1 = a.n1[q], n2 = a.n2[q];
    if (a.same[q]) {
        *first = a.line0[q] + (int64_t)i * (n1 - 1) - (int64_t)i * (i - 1) / 2;
        return n2 - i - 1;
    }
    *first = a.line0[q] + (int64_t)i * n2;
    return n2;
}

__global__ void __launch_bounds__(kRowThreads) mie_format_kernel(const MieArgs a) {
    int q, i;
    row_of(a, blockIdx.x, q, i);
    int64_t first;
    const int64_t cnt = row_lines(a, q, i, &first);
    const bool same = a.same[q] != 0;
    const int64_t P = (int64_t)a.n1[q] * (a.n1[q] - 1) / 2;
    for (int64_t t = threadIdx.x; t < cnt; t += kRowThreads) {
        const int j = (same ? i + 1 : 0) + (int)t;
        const int64_t L = first + t;
        const double s2 = same ? a.blk[q][P - 1 - (L - a.line0[q])] : a.blk[q][(int64_t)i * a.n2[q] + j];
        const double mu = a.s1r[q][i] + a.s1c[q][j] - s2;
        char *p0 = a.slots + L * kMieSlot, *p = p0;
        p = put_str(p, a.name[q], a.name_len[q]);
        p = put_int(p, i + 1);
        p = put_str(p, "  ", 2);
        p = put_int(p, j + 1);
        p = put_str(p, "   ", 3);
        int n = format_g12(s2, p);
        int len = 0;
        if (n >= 0) {
            p = put_str(p + n, "   ", 3);
            n = format_g12(mu, p);
            if (n >= 0) {
                p[n] = '\n';
                len = (int)(p + n + 1 - p0);
            }
        }
        if (!len) {  // outside the exact range: the host formats this line
            const int k = atomicAdd(a.fb_count, 1);
            if (k < a.fb_cap) a.fb_list[k] = L;
        }
        a.lens[L] = (uint8_t)len;
    }
}

__global__ void __launch_bounds__(kRowThreads) mie_rowlen_kernel(const MieArgs a) {
    int q, i;
    row_of(a, blockIdx.x, q, i);
    int64_t first;
    const int64_t cnt = row_lines(a, q, i, &first);
    long long s = 0;
    for (int64_t t = threadIdx.x; t < cnt; t += kRowThreads) s += a.lens[first + t];
    for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    __shared__ long long ws[kRowThreads / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long tot = 0;
        for (int w = 0; w < kRowThreads / 32; w++) tot += ws[w];
        a.row_len[blockIdx.x] = tot;
    }
}

// exclusive scan of row_len into row_off (one CTA of 1024 threads), total at row_off[rows]
__global__ void __launch_bounds__(1024) mie_scan_rows_kernel(const long long *__restrict__ len, long long *off,
                                                             int rows) {
    __shared__ long long ws[32];
    __shared__ long long carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < rows; base += 1024) {
        const int r = base + threadIdx.x;
        const long long v = r < rows ? len[r] : 0;
        long long x = v;  // inclusive warp scan
        for (int o = 1; o < 32; o <<= 1) {
            const long long y = __shfl_up_sync(0xffffffffu, x, o);
            if ((threadIdx.x & 31) >= o) x += y;
        }
        if ((threadIdx.x & 31) == 31) ws[threadIdx.x >> 5] = x;
        __syncthreads();
        if (threadIdx.x < 32) {
            long long w = ws[threadIdx.x];
            for (int o = 1; o < 32; o <<= 1) {
                const long long y = __shfl_up_sync(0xffffffffu, w, o);
                if (threadIdx.x >= o) w += y;
            }
            ws[threadIdx.x] = w;
        }
        __syncthreads();
        const long long incl = x + ((threadIdx.x >> 5) ? ws[(threadIdx.x >> 5) - 1] : 0);
        if (r < rows) off[r] = carry + incl - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry += incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) off[rows] = carry;
}

__global__ void __launch_bounds__(kRowThreads) mie_compact_kernel(const MieArgs a) {
    int q, i;
    row_of(a, blockIdx.x, q, i);
    int64_t first;
    const int64_t cnt = row_lines(a, q, i, &first);
    __shared__ int ws[kRowThreads / 32];
    __shared__ long long carry;
    if (threadIdx.x == 0) carry = a.row_off[blockIdx.x];
    __syncthreads();
    for (int64_t base = 0; base < cnt; base += kRowThreads) {
        const int64_t t = base + threadIdx.x;
        const int v = t < cnt ? a.lens[first + t] : 0;
        int x = v;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if ((threadIdx.x & 31) >= o) x += y;
        }
        if ((threadIdx.x & 31) == 31) ws[threadIdx.x >> 5] = x;
        __syncthreads();
        int before = 0;
        for (int w = 0; w < (int)(threadIdx.x >> 5); w++) before += ws[w];
        const long long pos = carry + before + x - v;
        if (v) {
            const char *src = a.slots + (first + t) * kMieSlot;
            char *dst = a.text + pos;
            for (int k = 0; k < v; k++) dst[k] = src[k];
        }
        __syncthreads();
        if (threadIdx.x == kRowThreads - 1) carry = pos + v;
        __syncthreads();
    }
}

}  // namespace

cudaError_t launch_mie_format(const MieArgs &a, cudaStream_t st) {
    if (a.rows <= 0) return cudaSuccess;
    mie_format_kernel<<<a.rows, kRowThreads, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_mie_offsets(const MieArgs &a, cudaStream_t st) {
    if (a.rows <= 0) return cudaSuccess;
    mie_rowlen_kernel<<<a.rows, kRowThreads, 0, st>>>(a);
    mie_scan_rows_kernel<<<1, 1024, 0, st>>>(a.row_len, a.row_off, a.rows);
    return cudaGetLastError();
}

cudaError_t launch_mie_compact(const MieArgs &a, cudaStream_t st) {
    if (a.rows <= 0) return cudaSuccess;
    mie_compact_kernel<<<a.rows, kRowThreads, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace pg
