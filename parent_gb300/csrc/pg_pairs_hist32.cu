// Pair kernel, shared-memory histogram form with 32 conflict-free pair slots
// (2D bin counts up to 50).
//
// Same work as pairs_hist_kernel (the 2D fill + epilogue loops of
// PARENT.cpp :786-1479): per pair, the B1 x B2 histogram of (bin_i, bin_j)
// over all frames, reduced to sum n ln n and the occupied-bin count, then
// S2D and MI. The difference is the shared-memory layout:
//   - a tile is 4 row DOFs x 8 column DOFs = 32 pair slots, lane = slot, and
//     every lane of a warp counts the same 16 frames for its own pair;
//   - counters are 16-bit, two bins per word: word (b >> 1) * 32 + lane, half
//     b & 1, so lane l always hits bank l: one wavefront per warp-wide
//     reduction instead of two;
//   - a 16-bit counter holds at most 65,535, so every kWindowChunks chunks
//     (63,488 frames) the consumer warps fold the halves into a per-CTA
//     32-bit accumulator in global memory (L2-resident) and clear them.
// The grid is persistent (one CTA per SM, tiles strided by the grid size) so
// each CTA owns one accumulator slot. Staging is the warp-specialised
// TMA/mbarrier pipeline of the 16-slot kernel: one producer warp issues
// cp.async.bulk copies of the tile's 12 bin rows, 31 consumer warps count.
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "pg_internal.h"
#include "pg_sync.cuh"

namespace pg {

namespace {

using namespace dev;

constexpr int kThreads = 1024, kWarps = 32, kConsumers = kWarps - 1;
constexpr int kRows = 4, kCols = 8;        // tile: 4 row DOFs x 8 column DOFs
constexpr int kNRow = kRows + kCols;       // staged bin rows per chunk
constexpr int kFC = 2048;                  // frames per chunk
constexpr int kStages = 2;
constexpr int kPad = 32;                   // bytes between staged rows
constexpr int kFCS = kFC + kPad;
constexpr int kWindowChunks = 31;          // 31 x 2048 = 63,488 <= 65,535 counts per 16-bit half
constexpr int kBmax = 50;                  // 32 lanes x 1,250 words x 4 B = 160 KB of counters
constexpr int kSmemMax = 232448;

__host__ __device__ constexpr int words_per_lane(int bmax) { return (bmax * bmax + 1) / 2; }
__host__ __device__ constexpr size_t hist32_bytes(int bmax) {
    return ((size_t)words_per_lane(bmax) * 32 * 4 + 1023) / 1024 * 1024;
}
constexpr size_t kStageBytes = (size_t)kStages * kNRow * kFCS;
constexpr size_t kRedBytes = (size_t)kWarps * 32 * (8 + 4);  // epilogue partials

__global__ void __launch_bounds__(kThreads, 1)
pairs_hist32_kernel(SysGeom geo, const uint8_t *__restrict__ bins, DofArrays dof,
                    const double *__restrict__ nlogn, const PairTile *__restrict__ tiles, int n_tiles,
                    PairOut out, int *err, uint32_t *__restrict__ acc_all, int bmax, double lnN) {
    extern __shared__ __align__(1024) unsigned char smem[];
    const int wpl = words_per_lane(bmax);
    const int nwords = wpl * 32;
    uint32_t *hist = (uint32_t *)smem;
    unsigned char *stage = smem + hist32_bytes(bmax);
    uint64_t *full = (uint64_t *)(stage + (kStageBytes > kRedBytes ? kStageBytes : kRedBytes));
    uint64_t *empty = full + kStages;
    uint32_t *acc = acc_all + (size_t)blockIdx.x * 2 * nwords;  // this CTA's 32-bit counters [bin][lane]
    __shared__ int s_abort;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int F = geo.F;
    const int nchunks = (F + kFC - 1) / kFC;
    const uint32_t hbase = smem_u32(hist) + lane * 4;

    for (int ti = blockIdx.x; ti < n_tiles; ti += gridDim.x) {
        const PairTile tile = tiles[ti];
        auto row_dof = [&](int k) -> int {
            if (k < kRows) return k < tile.nrow ? tile.row0 + k : -1;
            return (k - kRows) < tile.ncol ? tile.col0 + (k - kRows) : -1;
        };
        for (int i = tid * 4; i < nwords; i += kThreads * 4) *(uint4 *)(hist + i) = make_uint4(0u, 0u, 0u, 0u);
        if (tid == 0) {
            s_abort = 0;
            for (int k = 0; k < kStages; k++) {
                mbar_init(smem_u32(&full[k]), 1);
                mbar_init(smem_u32(&empty[k]), kConsumers);
            }
            mbar_init_fence();
        }
        __syncthreads();

        bool flushed = false;  // uniform over the consumer warps
        if (warp == kConsumers) {
            if (lane == 0) {
                for (int chunk = 0; chunk < nchunks; chunk++) {
                    const int st = chunk % kStages;
                    if (chunk >= kStages &&
                        !mbar_wait_bounded(smem_u32(&empty[st]), (uint32_t)(((chunk / kStages) - 1) & 1))) {
                        s_abort = 1;
                        break;
                    }
                    fence_proxy_async();
                    uint32_t bytes = 0;
                    for (int k = 0; k < kNRow; k++) bytes += row_dof(k) >= 0 ? (uint32_t)kFC : 0u;
                    const uint32_t bar = smem_u32(&full[st]);
                    mbar_expect_tx(bar, bytes);
                    for (int k = 0; k < kNRow; k++) {
                        const int g = row_dof(k);
                        if (g < 0) continue;
                        bulk_g2s(smem_u32(stage + (size_t)(st * kNRow + k) * kFCS),
                                 bins + (int64_t)g * geo.ldb + (int64_t)chunk * kFC, (uint32_t)kFC, bar);
                    }
                }
            }
        } else {
            const int pr = lane / kCols, pc = lane % kCols;
            const int gr = pr < tile.nrow ? tile.row0 + pr : -1;
            const int gc = pc < tile.ncol ? tile.col0 + pc : -1;
            const bool valid = gr >= 0 && gc >= 0 && gr < gc;
            const uint32_t Bc = valid ? (uint32_t)dof.b2[gc] : 0u;
            // 16-frame groups round-robin over the consumer warps, rotating the
            // leftover groups from chunk to chunk
            const int gstep = (kFC / 16) % kConsumers;
            int g0 = warp;
            // A warp whose wait timed out stops waiting and counting but keeps
            // going through the chunks, so that it still reaches every
            // window barrier of the other consumer warps.
            bool dead = false;
            for (int chunk = 0; chunk < nchunks; chunk++) {
                const int st = chunk % kStages;
                if (!dead && !mbar_wait_bounded(smem_u32(&full[st]), (uint32_t)((chunk / kStages) & 1))) {
                    dead = true;
                    s_abort = 1;
                }
                const int fvalid = min(kFC, F - chunk * kFC);
                const unsigned char *rrow = stage + (size_t)(st * kNRow + pr) * kFCS;
                const unsigned char *crow = stage + (size_t)(st * kNRow + kRows + pc) * kFCS;
                if (valid && !dead) {
                    for (int off = g0 * 16; off < fvalid; off += kConsumers * 16) {
                        const uint4 rv = *(const uint4 *)(rrow + off);
                        const uint4 cv = *(const uint4 *)(crow + off);
                        const uint32_t rw[4] = {rv.x, rv.y, rv.z, rv.w};
                        const uint32_t cw[4] = {cv.x, cv.y, cv.z, cv.w};
                        const int n = fvalid - off;  // frames of this group that exist
                        if (n >= 16) {
#pragma unroll
                            for (int q = 0; q < 4; q++) {
                                // two frames per IMAD (idx < 2500 never carries into the upper half);
                                // word (idx >> 1) of this lane, half idx & 1
                                const uint32_t i01 = __byte_perm(rw[q], 0u, 0x4140) * Bc + __byte_perm(cw[q], 0u, 0x4140);
                                const uint32_t i23 = __byte_perm(rw[q], 0u, 0x4342) * Bc + __byte_perm(cw[q], 0u, 0x4342);
                                red_add_nc(hbase + ((i01 & 0xfffeu) << 6), (i01 & 1u) * 0xffffu + 1u);
                                red_add_nc(hbase + ((i01 >> 17) << 7), ((i01 >> 16) & 1u) * 0xffffu + 1u);
                                red_add_nc(hbase + ((i23 & 0xfffeu) << 6), (i23 & 1u) * 0xffffu + 1u);
                                red_add_nc(hbase + ((i23 >> 17) << 7), ((i23 >> 16) & 1u) * 0xffffu + 1u);
                            }
                        } else {  // ragged end of the trajectory
#pragma unroll
                            for (int k = 0; k < 16; k++) {
                                if (k < n) {
                                    const uint32_t br = (rw[k >> 2] >> (8 * (k & 3))) & 0xffu;
                                    const uint32_t bc = (cw[k >> 2] >> (8 * (k & 3))) & 0xffu;
                                    const uint32_t idx = br * Bc + bc;
                                    red_add_nc(hbase + ((idx >> 1) << 7), (idx & 1u) * 0xffffu + 1u);
                                }
                            }
                        }
                    }
                }
                __syncwarp();
                if (lane == 0) mbar_arrive_relaxed(smem_u32(&empty[st]));
                g0 -= gstep;
                if (g0 < 0) g0 += kConsumers;
                if ((chunk + 1) % kWindowChunks == 0 && chunk + 1 < nchunks) {
                    // fold the 16-bit halves into the 32-bit accumulator before
                    // any can reach 65,536; the barrier also drains the
                    // consumers' outstanding reductions
                    named_barrier(kConsumers * 32);
                    for (int w = tid; w < nwords; w += kConsumers * 32) {
                        const uint32_t v = hist[w];
                        hist[w] = 0u;
                        const int b2 = (w >> 5) * 2, l = w & 31;
                        uint32_t *a = acc + (size_t)b2 * 32 + l;
                        if (flushed) {
                            a[0] += v & 0xffffu;
                            a[32] += v >> 16;
                        } else {
                            a[0] = v & 0xffffu;
                            a[32] = v >> 16;
                        }
                    }
                    flushed = true;
                    named_barrier(kConsumers * 32);
                }
            }
        }
        // consumers tell everyone whether the accumulator holds earlier windows
        const int any_flush = __syncthreads_or(flushed ? 1 : 0);
        if (s_abort) {
            if (tid == 0) {
                atomicAdd(&err[ERR_TIMEOUT], 1);
                for (int c = 0; c < kStages; c++) (void)mbar_wait_bounded(smem_u32(&full[c]), 0u);
            }
            __syncthreads();
            return;
        }

        // ---- epilogue: thread t handles pair slot t % 32 and bins t/32, +32, ...
        const int el = tid & 31, ew = tid >> 5;
        const int er = el / kCols, ec = el % kCols;
        const int egr = er < tile.nrow ? tile.row0 + er : -1;
        const int egc = ec < tile.ncol ? tile.col0 + ec : -1;
        const bool evalid = egr >= 0 && egc >= 0 && egr < egc;
        double snl = 0.0;
        int occ = 0;
        if (evalid) {
            const int nbin = dof.b2[egr] * dof.b2[egc];
            int64_t *dump = out.counts ? out.counts + ((int64_t)ti * 32 + el) * out.counts_bmax * out.counts_bmax : nullptr;
            for (int b = ew; b < nbin; b += kWarps) {
                uint32_t n = (hist[(b >> 1) * 32 + el] >> ((b & 1) * 16)) & 0xffffu;
                if (any_flush) n += acc[(size_t)b * 32 + el];
                if (n) {
                    snl += __ldg(nlogn + n);
                    occ++;
                }
                if (dump) dump[b] = n;
            }
        }
        double *red_snl = (double *)stage;                // [kWarps][32]
        int *red_occ = (int *)(red_snl + kWarps * 32);    // [kWarps][32]
        red_snl[ew * 32 + el] = snl;
        red_occ[ew * 32 + el] = occ;
        __syncthreads();
        if (tid < 32) {
            const int pr2 = tid / kCols, pc2 = tid % kCols;
            const int g1 = pr2 < tile.nrow ? tile.row0 + pr2 : -1;
            const int g2 = pc2 < tile.ncol ? tile.col0 + pc2 : -1;
            if (g1 >= 0 && g2 >= 0 && g1 < g2) {
                double s = 0.0;
                int o = 0;
                for (int w = 0; w < kWarps; w++) {
                    s += red_snl[w * 32 + tid];
                    o += red_occ[w * 32 + tid];
                }
                const double N = (double)F;
                const double S2 = lnN + dof.acon[g1] + dof.acon[g2] - s / N + (o - 1.0) / (2.0 * N);
                if (out.par) out.par[par_pair_index(out.L, geo.nb, geo.na, geo.nd, g1, g2)] = S2;
                if (out.mi) {
                    const double mi = dof.s1[g1] + dof.s1[g2] - S2;
                    out.mi[(int64_t)g1 * geo.D + g2] = mi;
                    out.mi[(int64_t)g2 * geo.D + g1] = mi;
                }
            }
        }
        __syncthreads();  // smem (counters, stages, barriers) is reused by the next tile
    }
}

size_t smem_bytes(int bmax) {
    return hist32_bytes(bmax) + (kStageBytes > kRedBytes ? kStageBytes : kRedBytes) + 8 * 2 * kStages;
}

}  // namespace

bool pairs_hist32_supported(int bmax) { return bmax <= kBmax && smem_bytes(bmax) + 1024 <= (size_t)kSmemMax; }

// accumulator bytes for `grid` CTAs
size_t pairs_hist32_scratch_bytes(int bmax, int grid) {
    return (size_t)grid * 2 * words_per_lane(bmax) * 32 * sizeof(uint32_t);
}

// Tiles of 4 row DOFs x 8 column DOFs with at least one pair r < c, in
// super-blocks of 16 x 16 tiles (L2 reuse among the CTAs running together).
std::vector<PairTile> build_tiles32(int D) {
    const int nrb = (D + kRows - 1) / kRows, ncb = (D + kCols - 1) / kCols, S = 16;
    std::vector<PairTile> t;
    for (int sc = 0; sc < (ncb + S - 1) / S; sc++)
        for (int sr = 0; sr < (nrb + S - 1) / S; sr++)
            for (int cb = sc * S; cb < std::min(ncb, (sc + 1) * S); cb++)
                for (int rb = sr * S; rb < std::min(nrb, (sr + 1) * S); rb++) {
                    const int r0 = rb * kRows, c0 = cb * kCols;
                    const int ncol = std::min(kCols, D - c0);
                    if (c0 + ncol - 1 <= r0) continue;  // every pair has r >= c
                    t.push_back(PairTile{r0, c0, std::min(kRows, D - r0), ncol});
                }
    return t;
}

cudaError_t launch_pairs_hist32(const SysGeom &g, const uint8_t *bins, const DofArrays &dof, const double *nlogn,
                                const PairTile *tiles, int64_t n_tiles, int grid, PairOut out, int *err,
                                void *scratch, size_t scratch_bytes, cudaStream_t st) {
    int bmax = 1;
    for (int t = 0; t < 3; t++) bmax = bmax > g.bins[3 + t] ? bmax : g.bins[3 + t];
    if (!pairs_hist32_supported(bmax) || n_tiles > INT32_MAX || grid < 1) return cudaErrorInvalidValue;
    if (scratch_bytes < pairs_hist32_scratch_bytes(bmax, grid)) return cudaErrorInvalidValue;
    if ((int64_t)g.ldb < (int64_t)((g.F + kFC - 1) / kFC) * kFC) return cudaErrorInvalidValue;
    if (n_tiles <= 0) return cudaSuccess;
    const size_t smem = smem_bytes(bmax);
    cudaError_t e = cudaFuncSetAttribute(pairs_hist32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    pairs_hist32_kernel<<<grid, kThreads, smem, st>>>(g, bins, dof, nlogn, tiles, (int)n_tiles, out, err,
                                                      (uint32_t *)scratch, bmax, log((double)g.F));
    return cudaGetLastError();
}

}  // namespace pg
