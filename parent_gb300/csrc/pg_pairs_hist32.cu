// Pair kernel, shared-memory histogram form with 32 conflict-free pair slots
// (2D bin counts up to 50).
//
// Same work as the 16-slot kernel (the 2D fill + epilogue loops of
// PARENT.cpp :786-1479): per pair, the B1 x B2 histogram of (bin_i, bin_j)
// over all frames, reduced to sum n ln n and the occupied-bin count, then
// S2D and MI. The difference is the shared-memory layout: a tile is 4 row
// DOFs x 8 column DOFs = 32 pair slots, lane = slot, every lane of a warp
// counts the same 16 frames for its own pair, and lane l's counters all sit
// in bank l, so a warp-wide reduction is one wavefront where the 16-slot
// layout (two lanes per pair) needs two. The counters are
//   - 32-bit, word b * 32 + lane, for 2D bin counts up to 35 (157 KB): the
//     fastest layout there (17.2 updates/clock/SM in the inner loop alone,
//     against 12.3 for the 16-slot layout);
//   - 16-bit, for 36 to 50 bins (160 KB): the two bins (2h, c) and
//     (2h + 1, c) of a pair share word (h * Bc + c) * 32 + lane. The row
//     DOF's bins are staged from a second matrix that the preprocessing
//     kernel writes as row codes (b >> 1) | (b & 1) << 7, so the word index
//     comes from the same byte-pair IMAD as in the 32-bit layout, and the
//     value added comes from one byte permute that replicates the code's top
//     bit: 0x00000001 for an even row bin, 0xFFFF0001 (= 1 - 65536) for an
//     odd one. A word then holds lo = n_even + n_odd in its low half and
//     -n_odd mod 65536 in its high half (no carry crosses the halves while
//     n_even + n_odd <= 65,535), i.e. n_odd = -hi mod 65536, n_even = lo - n_odd.
//     At 50 bins it runs at 12.3 updates/clock/SM (2,048-frame chunks: the
//     counters leave no room for 4,096), level with the 16-slot layout, so
//     the library keeps the 16-slot layout there (it needs no second bin
//     matrix) and runs this one on request.
//
// n_even + n_odd of a word counts frames in one column bin, so it cannot pass
// the column DOF's largest marginal bin count (computed by the preprocessing
// kernel): a tile whose column DOFs all stay within 65,535 runs without any
// check. Other tiles (long trajectories with peaked distributions) stop every
// 32,768 frames: the consumer warps move both counts of every word whose low
// half reached 32,768 into a per-CTA overflow area in global memory (rare,
// L2-resident) and clear the word, so no low half can pass 65,535 within the
// next 32,768 frames; the epilogue adds those counts back.
//
// Persistent grid (one CTA per SM, tiles strided by the grid size), with the
// warp-specialised TMA/mbarrier pipeline of the 16-slot kernel: the producer
// warp streams every chunk of every tile of the CTA (12 bin rows per chunk,
// one row copy per lane) and runs ahead into the next tile; 31 consumer warps
// count. The epilogue
// (fixed-point n ln n table, integer atomics) matches the 16-slot kernel's.
#include <stdint.h>
#include <stdlib.h>

#include <algorithm>
#include <vector>

#include "pg_internal.h"
#include "pg_sync.cuh"

namespace pg {

namespace {

using namespace dev;

constexpr int kThreads = 1024, kWarps = 32, kConsumers = kWarps - 1;
constexpr int kConsumerThreads = kConsumers * 32;
constexpr int kRows = 4, kCols = 8;        // tile: 4 row DOFs x 8 column DOFs
constexpr int kNRow = kRows + kCols;       // staged bin rows per chunk
constexpr int kMaxStages = 6;
constexpr int kPad = 16;                   // bytes between staged rows: a row stride of an odd number of
                                           // 16-byte units puts the 8 column rows of a stage on distinct banks
constexpr int kFoldFrames = 32768;         // counts moved out per fold; frames between folds
constexpr int kBmax16 = 50;                // 16-bit: 32 lanes x 1,250 words x 4 B = 160 KB of counters
constexpr int kBmax32 = 35;                // 32-bit: 32 lanes x 1,225 words x 4 B = 157 KB
constexpr int kSmemMax = 232448;

// 32-bit counters (one bin per word) where they fit, else 16-bit halves
__host__ __device__ constexpr bool wide_counters(int bmax) { return bmax <= kBmax32; }
__host__ __device__ constexpr int words_per_lane(int bmax) {
    return wide_counters(bmax) ? bmax * bmax : (bmax + 1) / 2 * bmax;
}
__host__ __device__ constexpr size_t hist32_bytes(int bmax) {
    return ((size_t)words_per_lane(bmax) * 32 * 4 + 127) / 128 * 128;
}
size_t smem_bytes(int bmax, int fc, int nst) {
    return hist32_bytes(bmax) + (size_t)nst * kNRow * (fc + kPad) + 8 * 2 * kMaxStages;
}

// hist word += 1, result unused (ordering from the barriers' clobbers)
__device__ __forceinline__ void red_add1_nc(uint32_t saddr) { asm volatile("red.shared.add.u32 [%0], 1;" ::"r"(saddr)); }

// Value added for frame k (0..3) of a 4-frame word of row codes: bytes
// 0x01, 0x00 (from the constant 1) and twice the sign of code byte k, i.e.
// 0x00000001 for an even row bin and 0xFFFF0001 for an odd one.
template <int K>
__device__ __forceinline__ uint32_t half_value(uint32_t codes4) {
    uint32_t r;
    constexpr uint32_t sel = ((8u | K) << 12) | ((8u | K) << 8) | 0x54u;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(r) : "r"(codes4), "r"(1u), "n"(sel));
    return r;
}

struct Hist32Args {
    SysDesc one;  // single-system launch (tile_sys == nullptr)
    const SysDesc *many;
    const PairTile *tiles;
    const int *tile_sys;
    int64_t n_tiles;
    const unsigned long long *nfix;
    double fix;
    int *err;
    uint32_t *ovf_all;  // per CTA: [2 * words_per_lane][32] overflow counts
    int fc, nst, bmax;
    uint32_t kw, kneg;  // 128 (bytes per counter word row) and -128 * 65536
};

// W32: 32-bit counters, word idx * 32 + lane, reduction value 1, no folding.
// Otherwise 16-bit halves as described above.
template <bool W32>
__global__ void __launch_bounds__(kThreads, 1) pairs_hist32_kernel(const __grid_constant__ Hist32Args a) {
    extern __shared__ __align__(128) unsigned char smem[];
    const int fc = a.fc, nst = a.nst;
    const int wpl = words_per_lane(a.bmax);
    const int nwords = wpl * 32;
    uint32_t *hist = (uint32_t *)smem;
    const int fcs = fc + kPad;
    unsigned char *stage = smem + hist32_bytes(a.bmax);
    uint64_t *full = (uint64_t *)(stage + (size_t)nst * kNRow * fcs);
    uint64_t *empty = full + kMaxStages;
    __shared__ unsigned long long s_snl[32];
    __shared__ unsigned int s_occ[32];
    __shared__ int s_heavy[32];
    __shared__ volatile int s_abort;   // consumers only
    __shared__ volatile int s_pabort;  // producer
    __shared__ long long s_issued;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int i = tid * 4; i < nwords; i += kThreads * 4) *(uint4 *)(hist + i) = make_uint4(0u, 0u, 0u, 0u);
    if (tid < 32) {
        s_snl[tid] = 0ull;
        s_occ[tid] = 0u;
        s_heavy[tid] = 0;
    }
    if (tid == 0) {
        s_abort = 0;
        s_pabort = 0;
        s_issued = 0;
        for (int k = 0; k < nst; k++) {
            mbar_init(smem_u32(&full[k]), 1);
            mbar_init(smem_u32(&empty[k]), kConsumers);
        }
        mbar_init_fence();
    }
    __syncthreads();

    auto sys_of = [&](int64_t t) -> const SysDesc & { return a.tile_sys ? a.many[a.tile_sys[t]] : a.one; };

    if (warp == kConsumers) {
        // ---------------------------------------------------------- producer
        // lane 0 waits for a free stage and arms its full barrier; lanes
        // 0..kNRow-1 then issue one row copy each, in parallel
        long long seq = 0;
        bool ok = true;
        for (int64_t t = blockIdx.x; t < a.n_tiles && ok; t += gridDim.x) {
            const SysDesc &d = sys_of(t);
            const PairTile tile = a.tiles[t];
            const int nchunks = (d.geo.F + fc - 1) / fc;
            const uint8_t *src = nullptr;
            if (lane < kNRow) {
                const int k = lane;
                const int g = k < kRows ? (k < tile.nrow ? tile.row0 + k : -1)
                                    : ((k - kRows) < tile.ncol ? tile.col0 + (k - kRows) : -1);
                // 16-bit layout: row DOFs from the row-code matrix
                const int64_t m = (!W32 && k < kRows) ? (int64_t)d.geo.D : 0;
                src = g >= 0 ? d.bins + (m + g) * d.geo.ldb : nullptr;
            }
            const uint32_t bytes = (uint32_t)__popc(__ballot_sync(0xffffffffu, src != nullptr)) * (uint32_t)fc;
            for (int chunk = 0; chunk < nchunks; chunk++, seq++) {
                const int st = (int)(seq % nst);
                int go = 1;
                if (lane == 0) {
                    if (seq >= nst &&
                        !mbar_wait_bounded(smem_u32(&empty[st]), (uint32_t)(((seq / nst) - 1) & 1))) {
                        s_pabort = 1;
                        go = 0;
                    } else if (s_abort) {  // the consumers gave up: stop issuing
                        go = 0;
                    }
                    if (go) mbar_expect_tx(smem_u32(&full[st]), bytes);
                }
                if (!__shfl_sync(0xffffffffu, go, 0)) {
                    ok = false;
                    break;
                }
                if (src) {
                    // generic-proxy reads of this stage (released by the empty
                    // barrier) before the async-proxy writes refilling it
                    fence_proxy_async();
                    bulk_g2s(smem_u32(stage + (size_t)(st * kNRow + lane) * fcs), src + (int64_t)chunk * fc,
                             (uint32_t)fc, smem_u32(&full[st]));
                }
            }
        }
        if (lane == 0) s_issued = seq;
    } else {
        // --------------------------------------------------------- consumers
        const int pr = lane / kCols, pc = lane % kCols;
        const uint32_t hbase = smem_u32(hist) + lane * 4;
        uint32_t *ovf = a.ovf_all + (size_t)blockIdx.x * 2 * nwords;  // [bin][lane]
        const int gstep = (fc / 16) % kConsumers;
        const int fold_every = kFoldFrames / fc;  // chunks between folds
        const int ctid = tid;
        const int ew = ctid >> 5;  // epilogue / fold: words j = ew + 31 k of slot `lane`
        long long seq = 0;
        for (int64_t t = blockIdx.x; t < a.n_tiles; t += gridDim.x) {
            const SysDesc &d = sys_of(t);
            const PairTile tile = a.tiles[t];
            const int F = d.geo.F;
            const int nchunks = (F + fc - 1) / fc;
            const int gr = pr < tile.nrow ? tile.row0 + pr : -1;
            const int gc = pc < tile.ncol ? tile.col0 + pc : -1;
            const bool valid = gr >= 0 && gc >= 0 && gr < gc;
            const uint32_t Bc = valid ? (uint32_t)d.dof.b2[gc] : 0u;
            // every warp holds all 32 slots, so this vote is the same in all
            // consumer warps (it decides who takes the fold barriers)
            const bool risky = valid && (W32 ? false : d.dof.m2[gc] > 65535);
            const bool folding = !W32 && __any_sync(0xffffffffu, risky) && nchunks > fold_every;
            int g0 = warp;
            bool dead = false;  // a timed-out warp keeps taking the fold barriers
            for (int chunk = 0; chunk < nchunks; chunk++, seq++) {
                const int st = (int)(seq % nst);
                if (!dead && !mbar_wait_bounded(smem_u32(&full[st]), (uint32_t)((seq / nst) & 1))) {
                    s_abort = 1;
                    dead = true;
                }
                if (!dead) {
                    const int fvalid = min(fc, F - chunk * fc);
                    const unsigned char *rrow = stage + (size_t)(st * kNRow + pr) * fcs;
                    const unsigned char *crow = stage + (size_t)(st * kNRow + kRows + pc) * fcs;
                    if (valid) {
                        const int fend = fvalid & ~15;  // frames in whole 16-frame groups
                        int off = g0 * 16;
                        for (; off < fend; off += kConsumers * 16) {
                            const uint4 rv = *(const uint4 *)(rrow + off);
                            const uint4 cv = *(const uint4 *)(crow + off);
                            const uint32_t rw[4] = {rv.x, rv.y, rv.z, rv.w};
                            const uint32_t cw[4] = {cv.x, cv.y, cv.z, cv.w};
                            {
                                if (W32) {
                                    // word addresses hbase + 128 idx for the 16 frames, with
                                    // the multiplies on the FMA pipe (multipliers come from
                                    // the launch arguments, so they stay IMADs): the ALU
                                    // pipe is this loop's busiest unit
                                    uint32_t ad[16];
#pragma unroll
                                    for (int q = 0; q < 4; q++) {
#pragma unroll
                                        for (int h = 0; h < 2; h++) {
                                            const uint32_t sel = h ? 0x4342u : 0x4140u;
                                            const uint32_t v = __byte_perm(rw[q], 0u, sel) * Bc + __byte_perm(cw[q], 0u, sel);
                                            const uint32_t hi = v >> 16;
                                            ad[4 * q + 2 * h + 1] = hi * a.kw + hbase;
                                            ad[4 * q + 2 * h] = v * a.kw + hbase + hi * a.kneg;
                                        }
                                    }
                                    // frames 0, 4, 8, 12, 1, 5, ...
#pragma unroll
                                    for (int k = 0; k < 4; k++) {
#pragma unroll
                                        for (int q = 0; q < 4; q++) red_add1_nc(ad[4 * q + k]);
                                    }
                                } else {
                                    // word index (code & 0x7f) * Bc + bc, two frames per IMAD
                                    // as above; the value from the code's top bit
#pragma unroll
                                    for (int q = 0; q < 4; q++) {
                                        const uint32_t rs = rw[q] & 0x7f7f7f7fu;
#pragma unroll
                                        for (int h = 0; h < 2; h++) {
                                            const uint32_t sel = h ? 0x4342u : 0x4140u;
                                            const uint32_t v = __byte_perm(rs, 0u, sel) * Bc + __byte_perm(cw[q], 0u, sel);
                                            const uint32_t hi = v >> 16;
                                            const uint32_t a_hi = hi * a.kw + hbase;
                                            const uint32_t a_lo = v * a.kw + hbase + hi * a.kneg;
                                            if (h == 0) {
                                                red_add_nc(a_lo, half_value<0>(rw[q]));
                                                red_add_nc(a_hi, half_value<1>(rw[q]));
                                            } else {
                                                red_add_nc(a_lo, half_value<2>(rw[q]));
                                                red_add_nc(a_hi, half_value<3>(rw[q]));
                                            }
                                        }
                                    }
                                }
                            }
                        }
                        if (off < fvalid) {  // the ragged last group of the trajectory (off == fend)
                            const uint4 rv = *(const uint4 *)(rrow + off);
                            const uint4 cv = *(const uint4 *)(crow + off);
                            const uint32_t rw[4] = {rv.x, rv.y, rv.z, rv.w};
                            const uint32_t cw[4] = {cv.x, cv.y, cv.z, cv.w};
                            {
                                const int n = fvalid - off;
#pragma unroll
                                for (int k = 0; k < 16; k++) {
                                    if (k < n) {
                                        const uint32_t br = (rw[k >> 2] >> (8 * (k & 3))) & 0xffu;
                                        const uint32_t bc = (cw[k >> 2] >> (8 * (k & 3))) & 0xffu;
                                        if (W32) red_add1_nc(hbase + ((br * Bc + bc) << 7));
                                        else red_add_nc(hbase + (((br & 0x7fu) * Bc + bc) << 7),
                                                       (br & 0x80u) ? 0xFFFF0001u : 1u);
                                    }
                                }
                            }
                        }
                    }
                    __syncwarp();
                    if (lane == 0) mbar_arrive_relaxed(smem_u32(&empty[st]));
                }
                g0 -= gstep;
                if (g0 < 0) g0 += kConsumers;
                if (folding && (chunk + 1) % fold_every == 0 && chunk + 1 < nchunks) {
                    // every consumer's reductions so far are done; move both
                    // counts of every word whose low half reached 32,768
                    // out (w & 31 == lane: kConsumerThreads is a multiple of 32)
                    named_barrier(kConsumerThreads);
                    for (int w = ctid; w < nwords; w += kConsumerThreads) {
                        const uint32_t v = hist[w];
                        if (v & 0x8000u) {
                            const uint32_t n_odd = (0u - (v >> 16)) & 0xffffu, n_even = (v & 0xffffu) - n_odd;
                            hist[w] = 0u;
                            const int b = (w >> 5) * 2;
                            ovf[b * 32 + lane] += n_even;
                            ovf[(b + 1) * 32 + lane] += n_odd;
                            s_heavy[lane] = 1;
                        }
                    }
                    named_barrier(kConsumerThreads);
                }
            }
            named_barrier(kConsumerThreads);
            if (s_abort) break;  // the same value for every consumer

            // ---- epilogue: this thread reads words j = ew, ew + 31, ... of
            // slot `lane` (the words its folds handled), zeroing them
            const int egr = gr, egc = gc;
            unsigned long long snl = 0ull;
            int occ = 0;
            if (valid && W32) {
                const int nbin = d.dof.b2[egr] * d.dof.b2[egc];
                int64_t *dump = d.out.counts ? d.out.counts + (t * 32 + lane) * d.out.counts_bmax * d.out.counts_bmax
                                             : nullptr;
                for (int j = ew; j < nbin; j += kConsumers) {
                    const int w = j * 32 + lane;
                    const uint32_t n = hist[w];
                    hist[w] = 0u;
                    snl += __ldg(a.nfix + n);
                    occ += n != 0u;
                    if (dump) dump[j] = n;
                }
                atomicAdd(&s_snl[lane], snl);
                atomicAdd(&s_occ[lane], (unsigned int)occ);
            } else if (valid) {
                // word j = h * Bc + c holds bins (2h, c) and (2h + 1, c)
                const int Br = d.dof.b2[egr], Bcc = d.dof.b2[egc];
                const int nw = (Br + 1) / 2 * Bcc;
                const bool heavy = s_heavy[lane] != 0;
                int64_t *dump = d.out.counts ? d.out.counts + (t * 32 + lane) * d.out.counts_bmax * d.out.counts_bmax
                                             : nullptr;
                for (int j = ew; j < nw; j += kConsumers) {
                    const int w = j * 32 + lane;
                    const uint32_t v = hist[w];
                    hist[w] = 0u;
                    uint32_t n1 = (0u - (v >> 16)) & 0xffffu;  // odd row bin
                    uint32_t n0 = (v & 0xffffu) - n1;           // even row bin
                    if (heavy) {
                        uint32_t *o = ovf + (size_t)(2 * j) * 32 + lane;
                        const uint32_t o0 = o[0], o1 = o[32];
                        if (o0 | o1) {
                            n0 += o0;
                            n1 += o1;
                            o[0] = 0u;
                            o[32] = 0u;
                        }
                    }
                    snl += __ldg(a.nfix + n0) + __ldg(a.nfix + n1);
                    occ += (n0 != 0u) + (n1 != 0u);
                    if (dump) {
                        const int h = j / Bcc, c = j - h * Bcc;
                        dump[2 * h * Bcc + c] = n0;
                        if (2 * h + 1 < Br) dump[(2 * h + 1) * Bcc + c] = n1;
                    }
                }
                atomicAdd(&s_snl[lane], snl);
                atomicAdd(&s_occ[lane], (unsigned int)occ);
            }
            named_barrier(kConsumerThreads);
            if (ctid < 32) {
                if (valid) {
                    const double N = (double)F;
                    const double sn = (double)s_snl[ctid] / a.fix;
                    const int o = (int)s_occ[ctid];
                    const double S2 = d.lnN + d.dof.acon[egr] + d.dof.acon[egc] - sn / N + (o - 1.0) / (2.0 * N);
                    if (d.out.par) d.out.par[par_pair_index(d.out.L, d.geo.nb, d.geo.na, d.geo.nd, egr, egc)] = S2;
                    if (d.out.mi) {
                        const double mi = d.dof.s1[egr] + d.dof.s1[egc] - S2;
                        d.out.mi[(int64_t)egr * d.geo.D + egc] = mi;
                        d.out.mi[(int64_t)egc * d.geo.D + egr] = mi;
                    }
                }
                s_snl[ctid] = 0ull;
                s_occ[ctid] = 0u;
                s_heavy[ctid] = 0;
            }
        }
    }
    __syncthreads();

    if (s_abort || s_pabort) {
        if (tid == 0) {
            atomicAdd(&a.err[ERR_TIMEOUT], 1);
            const long long n = s_issued;
            for (long long k = n > nst ? n - nst : 0; k < n; k++)
                (void)mbar_wait_bounded(smem_u32(&full[k % nst]), (uint32_t)((k / nst) & 1));
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Streamed form of the same layouts. The TMA ring above makes every consumer
// warp wait on, and release, every chunk of the tile: each warp only counts
// fc/31 frames of a chunk, so the per-chunk synchronisation is paid every few
// hundred updates, and beside 160 KB of 16-bit counters only two 2,048-frame
// stages fit. Here there is no ring: all 32 warps count, each streams its own
// 16-frame groups (group k goes to warp k mod 32) straight from global memory
// into registers from the frame-group interleaved bin layout (ilv_index), in
// which a tile's 8 column DOFs are one 128-byte line per group, its 4 row
// DOFs half of one, and a warp's consecutive groups are 4 KB apart: three
// register buffers rotate, so every load is issued two groups before its
// bytes are counted, at constant offsets from one pointer per operand. The
// warps meet only at the end of a tile (and at the 16-bit folds). Counting,
// folds and the epilogue are those of the ring kernel.
constexpr int kFoldGroups = kFoldFrames / 16;
constexpr int kQueue = 32;  // finished tiles per FP64 epilogue round (one per warp)

// 16 bytes from global memory, not kept in L1 (each line is read once)
__device__ __forceinline__ uint4 ldg_stream(const void *p) {
    uint4 r;
    asm("ld.global.nc.L1::no_allocate.v4.u32 {%0, %1, %2, %3}, [%4];"
        : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
        : "l"(p));
    return r;
}

// One lane's 16 updates of a whole group: row bins (W32) or row codes
// (16-bit) in rv, column bins in cv; the same arithmetic as the ring kernel.
template <bool W32>
__device__ __forceinline__ void count_group(const uint4 rv, const uint4 cv, uint32_t Bc, uint32_t hbase,
                                            uint32_t kw, uint32_t kneg) {
    const uint32_t rw[4] = {rv.x, rv.y, rv.z, rv.w};
    const uint32_t cw[4] = {cv.x, cv.y, cv.z, cv.w};
    if (W32) {
        uint32_t ad[16];
#pragma unroll
        for (int q = 0; q < 4; q++) {
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const uint32_t sel = h ? 0x4342u : 0x4140u;
                const uint32_t v = __byte_perm(rw[q], 0u, sel) * Bc + __byte_perm(cw[q], 0u, sel);
                const uint32_t hi = v >> 16;
                ad[4 * q + 2 * h + 1] = hi * kw + hbase;
                ad[4 * q + 2 * h] = v * kw + hbase + hi * kneg;
            }
        }
#pragma unroll
        for (int k = 0; k < 4; k++) {
#pragma unroll
            for (int q = 0; q < 4; q++) red_add1_nc(ad[4 * q + k]);
        }
    } else {
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const uint32_t rs = rw[q] & 0x7f7f7f7fu;
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const uint32_t sel = h ? 0x4342u : 0x4140u;
                const uint32_t v = __byte_perm(rs, 0u, sel) * Bc + __byte_perm(cw[q], 0u, sel);
                const uint32_t hi = v >> 16;
                const uint32_t a_hi = hi * kw + hbase;
                const uint32_t a_lo = v * kw + hbase + hi * kneg;
                if (h == 0) {
                    red_add_nc(a_lo, half_value<0>(rw[q]));
                    red_add_nc(a_hi, half_value<1>(rw[q]));
                } else {
                    red_add_nc(a_lo, half_value<2>(rw[q]));
                    red_add_nc(a_hi, half_value<3>(rw[q]));
                }
            }
        }
    }
}

template <bool W32>
__global__ void __launch_bounds__(kThreads, 1) pairs_hist32s_kernel(const __grid_constant__ Hist32Args a) {
    extern __shared__ __align__(128) unsigned char smem[];
    const int wpl = words_per_lane(a.bmax);
    const int nwords = wpl * 32;
    uint32_t *hist = (uint32_t *)smem;
    __shared__ unsigned long long s_snl[32];
    __shared__ unsigned int s_occ[32];
    __shared__ int s_heavy[32];
    // sums of finished tiles whose FP64 epilogue waits for kQueue of them;
    // then warp q finishes the pairs of tile q (the FP64 pipe is a small
    // fraction of this part's rate, and one warp finishing every tile
    // alone held back the next tile, whose frame groups are split evenly
    // over all warps)
    __shared__ unsigned long long s_qsnl[kQueue][32];
    __shared__ unsigned int s_qocc[kQueue][32];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int i = tid * 4; i < nwords; i += kThreads * 4) *(uint4 *)(hist + i) = make_uint4(0u, 0u, 0u, 0u);
    if (tid < 32) {
        s_snl[tid] = 0ull;
        s_occ[tid] = 0u;
        s_heavy[tid] = 0;
    }
    __syncthreads();

    auto sys_of = [&](int64_t t) -> const SysDesc & { return a.tile_sys ? a.many[a.tile_sys[t]] : a.one; };
    const int pr = lane / kCols, pc = lane % kCols;
    const uint32_t hbase = smem_u32(hist) + lane * 4;
    uint32_t *ovf = a.ovf_all + (size_t)blockIdx.x * 2 * nwords;  // [bin][lane]
    for (int it = 0;; it++) {
        const int64_t t = blockIdx.x + (int64_t)it * gridDim.x;
        if (t >= a.n_tiles) break;
        const SysDesc &d = sys_of(t);
        const PairTile tile = a.tiles[t];
        const int F = d.geo.F, D = d.geo.D;
        const int G = (F + 15) >> 4, Gfull = F >> 4;
        const int gr = pr < tile.nrow ? tile.row0 + pr : -1;
        const int gc = pc < tile.ncol ? tile.col0 + pc : -1;
        const bool valid = gr >= 0 && gc >= 0 && gr < gc;
        const uint32_t Bc = valid ? (uint32_t)d.dof.b2[gc] : 0u;
        // every warp holds all 32 slots, so this vote is the same in every
        // warp (it decides who takes the fold barriers: all of them or none)
        const bool risky = valid && (W32 ? false : d.dof.m2[gc] > 65535);
        const bool folding = !W32 && __any_sync(0xffffffffu, risky) && G > kFoldGroups;
        // rows: bins (32-bit counters) or row codes (16-bit), after the bins
        const uint8_t *rbase = (W32 ? d.bins : d.bins + ilv_bytes(D, F)) + ilv_dof_base(F, valid ? gr : 0);
        const uint8_t *cbase = d.bins + ilv_dof_base(F, valid ? gc : 0);
        constexpr int kStep = 32 * 128;  // bytes from one of a warp's groups to its next
        const int span = folding ? kFoldGroups : G;
        for (int g0 = 0; g0 < G; g0 += span) {
            const int gend = min(G, g0 + span);
            const int fe = min(gend, Gfull);  // whole groups of this span end here
            if (valid) {
                // this warp's whole groups of the span: g0 + warp + 32 k, k < nk
                const int first = g0 + warp;
                const int nk = fe > first ? (fe - first + 31) / 32 : 0;
                const uint8_t *rp = rbase + (int64_t)first * 128;
                const uint8_t *cp = cbase + (int64_t)first * 128;
                uint4 ar = make_uint4(0u, 0u, 0u, 0u), ac = ar, br = ar, bc = ar, cr = ar, cc = ar;
                if (nk > 0) {
                    ar = ldg_stream(rp);
                    ac = ldg_stream(cp);
                }
                if (nk > 1) {
                    br = ldg_stream(rp + kStep);
                    bc = ldg_stream(cp + kStep);
                }
                int k = 0;
                for (; k + 2 < nk; k += 3) {
                    cr = ldg_stream(rp + 2 * kStep);
                    cc = ldg_stream(cp + 2 * kStep);
                    count_group<W32>(ar, ac, Bc, hbase, a.kw, a.kneg);
                    if (k + 3 < nk) {
                        ar = ldg_stream(rp + 3 * kStep);
                        ac = ldg_stream(cp + 3 * kStep);
                    }
                    count_group<W32>(br, bc, Bc, hbase, a.kw, a.kneg);
                    if (k + 4 < nk) {
                        br = ldg_stream(rp + 4 * kStep);
                        bc = ldg_stream(cp + 4 * kStep);
                    }
                    count_group<W32>(cr, cc, Bc, hbase, a.kw, a.kneg);
                    rp += 3 * kStep;
                    cp += 3 * kStep;
                }
                if (k < nk) count_group<W32>(ar, ac, Bc, hbase, a.kw, a.kneg);
                if (k + 1 < nk) count_group<W32>(br, bc, Bc, hbase, a.kw, a.kneg);
                // the ragged last group of the trajectory, on the warp whose
                // turn it is
                if (Gfull < gend && Gfull >= g0 && ((Gfull - g0) & 31) == warp) {
                    const uint4 rv = ldg_stream(rbase + (int64_t)Gfull * 128);
                    const uint4 cv = ldg_stream(cbase + (int64_t)Gfull * 128);
                    const uint32_t rw[4] = {rv.x, rv.y, rv.z, rv.w};
                    const uint32_t cw[4] = {cv.x, cv.y, cv.z, cv.w};
                    const int n = F - Gfull * 16;
#pragma unroll
                    for (int q = 0; q < 16; q++) {
                        if (q < n) {
                            const uint32_t brow = (rw[q >> 2] >> (8 * (q & 3))) & 0xffu;
                            const uint32_t bcol = (cw[q >> 2] >> (8 * (q & 3))) & 0xffu;
                            if (W32) red_add1_nc(hbase + ((brow * Bc + bcol) << 7));
                            else red_add_nc(hbase + (((brow & 0x7fu) * Bc + bcol) << 7),
                                            (brow & 0x80u) ? 0xFFFF0001u : 1u);
                        }
                    }
                }
            }
            if (folding && gend < G) {
                // every warp's reductions so far are done; move both counts of
                // every word whose low half reached 32,768 out (w & 31 == lane)
                __syncthreads();
                for (int w = tid; w < nwords; w += kThreads) {
                    const uint32_t v = hist[w];
                    if (v & 0x8000u) {
                        const uint32_t n_odd = (0u - (v >> 16)) & 0xffffu, n_even = (v & 0xffffu) - n_odd;
                        hist[w] = 0u;
                        const int b = (w >> 5) * 2;
                        ovf[b * 32 + lane] += n_even;
                        ovf[(b + 1) * 32 + lane] += n_odd;
                        s_heavy[lane] = 1;
                    }
                }
                __syncthreads();
            }
        }
        __syncthreads();

        // ---- epilogue: this thread reads words j = warp, warp + 32, ... of
        // slot `lane`, zeroing them
        unsigned long long snl = 0ull;
        int occ = 0;
        if (valid && W32) {
            const int nbin = d.dof.b2[gr] * d.dof.b2[gc];
            int64_t *dump = d.out.counts ? d.out.counts + (t * 32 + lane) * d.out.counts_bmax * d.out.counts_bmax
                                         : nullptr;
            int j = warp;
            if (!dump) {
                // four words in flight; n ln n is 0 below 2, so no table read
                for (; j + 3 * kWarps < nbin; j += 4 * kWarps) {
                    uint32_t n[4];
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        n[u] = hist[(j + u * kWarps) * 32 + lane];
                        hist[(j + u * kWarps) * 32 + lane] = 0u;
                    }
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        if (n[u] > 1u) snl += __ldg(a.nfix + n[u]);
                        occ += n[u] != 0u;
                    }
                }
            }
            for (; j < nbin; j += kWarps) {
                const int w = j * 32 + lane;
                const uint32_t n = hist[w];
                hist[w] = 0u;
                snl += __ldg(a.nfix + n);
                occ += n != 0u;
                if (dump) dump[j] = n;
            }
            atomicAdd(&s_snl[lane], snl);
            atomicAdd(&s_occ[lane], (unsigned int)occ);
        } else if (valid) {
            // word j = h * Bc + c holds bins (2h, c) and (2h + 1, c)
            const int Br = d.dof.b2[gr], Bcc = d.dof.b2[gc];
            const int nw = (Br + 1) / 2 * Bcc;
            const bool heavy = s_heavy[lane] != 0;
            int64_t *dump = d.out.counts ? d.out.counts + (t * 32 + lane) * d.out.counts_bmax * d.out.counts_bmax
                                         : nullptr;
            int j = warp;
            if (!heavy && !dump) {
                // four words in flight; n ln n is 0 below 2, so no table read
                for (; j + 3 * kWarps < nw; j += 4 * kWarps) {
                    uint32_t v[4];
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        v[u] = hist[(j + u * kWarps) * 32 + lane];
                        hist[(j + u * kWarps) * 32 + lane] = 0u;
                    }
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        const uint32_t n1 = (0u - (v[u] >> 16)) & 0xffffu, n0 = (v[u] & 0xffffu) - n1;
                        if (n0 > 1u) snl += __ldg(a.nfix + n0);
                        if (n1 > 1u) snl += __ldg(a.nfix + n1);
                        occ += (n0 != 0u) + (n1 != 0u);
                    }
                }
            }
            for (; j < nw; j += kWarps) {
                const int w = j * 32 + lane;
                const uint32_t v = hist[w];
                hist[w] = 0u;
                uint32_t n1 = (0u - (v >> 16)) & 0xffffu;  // odd row bin
                uint32_t n0 = (v & 0xffffu) - n1;           // even row bin
                if (heavy) {
                    uint32_t *o = ovf + (size_t)(2 * j) * 32 + lane;
                    const uint32_t o0 = o[0], o1 = o[32];
                    if (o0 | o1) {
                        n0 += o0;
                        n1 += o1;
                        o[0] = 0u;
                        o[32] = 0u;
                    }
                }
                snl += __ldg(a.nfix + n0) + __ldg(a.nfix + n1);
                occ += (n0 != 0u) + (n1 != 0u);
                if (dump) {
                    const int h = j / Bcc, c = j - h * Bcc;
                    dump[2 * h * Bcc + c] = n0;
                    if (2 * h + 1 < Br) dump[(2 * h + 1) * Bcc + c] = n1;
                }
            }
            atomicAdd(&s_snl[lane], snl);
            atomicAdd(&s_occ[lane], (unsigned int)occ);
        }
        __syncthreads();
        if constexpr (W32) {
            // 32-bit counters: this layout's tiles finish on warp 0 at once
            // (measured faster there than the queue below)
            if (tid < 32) {
                if (valid) {
                    const double N = (double)F;
                    const double sn = (double)s_snl[tid] / a.fix;
                    const int o = (int)s_occ[tid];
                    const double S2 = d.lnN + d.dof.acon[gr] + d.dof.acon[gc] - sn / N + (o - 1.0) / (2.0 * N);
                    if (d.out.par) d.out.par[par_pair_index(d.out.L, d.geo.nb, d.geo.na, d.geo.nd, gr, gc)] = S2;
                    if (d.out.mi) {
                        const double mi = d.dof.s1[gr] + d.dof.s1[gc] - S2;
                        d.out.mi[(int64_t)gr * d.geo.D + gc] = mi;
                        d.out.mi[(int64_t)gc * d.geo.D + gr] = mi;
                    }
                }
                // the next tile's epilogue atomics come after its first barrier
                s_snl[tid] = 0ull;
                s_occ[tid] = 0u;
                s_heavy[tid] = 0;
            }
            continue;
        }
        const int q = it & (kQueue - 1);
        if (tid < 32) {
            s_qsnl[q][tid] = s_snl[tid];
            s_qocc[q][tid] = s_occ[tid];
            // the next tile's epilogue atomics come after its first barrier
            s_snl[tid] = 0ull;
            s_occ[tid] = 0u;
            s_heavy[tid] = 0;
        }
        if (q == kQueue - 1 || t + gridDim.x >= a.n_tiles) {
            __syncthreads();
            // warp w finishes queued tile w: this CTA's tile q - w before t
            // (the same expression as every other pair kernel and the branch
            // above, so bodies agree bit for bit); warp 0 refills the queue
            // only after the next tile's barrier before its epilogue, which
            // every warp reaches after this
            if (warp <= q) {
                const int64_t tq = t - (int64_t)(q - warp) * gridDim.x;
                const SysDesc &dq = sys_of(tq);
                const PairTile tl = a.tiles[tq];
                const int r = pr < tl.nrow ? tl.row0 + pr : -1, c = pc < tl.ncol ? tl.col0 + pc : -1;
                if (r >= 0 && c >= 0 && r < c) {
                    const double N = (double)dq.geo.F;
                    const double sn = (double)s_qsnl[warp][lane] / a.fix;
                    const int o = (int)s_qocc[warp][lane];
                    const double S2 = dq.lnN + dq.dof.acon[r] + dq.dof.acon[c] - sn / N + (o - 1.0) / (2.0 * N);
                    if (dq.out.par) dq.out.par[par_pair_index(dq.out.L, dq.geo.nb, dq.geo.na, dq.geo.nd, r, c)] = S2;
                    if (dq.out.mi) {
                        const double mi = dq.dof.s1[r] + dq.dof.s1[c] - S2;
                        dq.out.mi[(int64_t)r * dq.geo.D + c] = mi;
                        dq.out.mi[(int64_t)c * dq.geo.D + r] = mi;
                    }
                }
            }
        }
    }
}

int sm_count() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 1;
    }
    return n;
}

// Staging geometry for a bin count: frames per chunk x stages, the largest
// chunks that fit (measured at 30 bins: 11.2, 13.3 and 14.2 updates/clock/SM
// for 1,024-, 2,048- and 4,096-frame chunks), at most 4096 frames (the
// padding of every bin row). PG_HIST32_FC / PG_HIST32_STAGES override it for
// sweeps when they fit.
bool config(int bmax, int *fc, int *nst) {
    static const int cand[][2] = {{4096, 2}, {2048, 4}, {2048, 3}, {2048, 2}, {1024, 4}, {1024, 2}};
    int ofc = 0, onst = 0;
    if (const char *e = getenv("PG_HIST32_FC")) ofc = atoi(e);
    if (const char *e = getenv("PG_HIST32_STAGES")) onst = atoi(e);
    if (ofc >= 256 && ofc <= 4096 && ofc % 16 == 0 && onst >= 2 && onst <= kMaxStages &&
        smem_bytes(bmax, ofc, onst) + 1024 <= (size_t)kSmemMax) {
        *fc = ofc;
        *nst = onst;
        return true;
    }
    for (const auto &c : cand)
        if (smem_bytes(bmax, c[0], c[1]) + 1024 <= (size_t)kSmemMax) {
            *fc = c[0];
            *nst = c[1];
            return true;
        }
    return false;
}

// codes: the row-code matrix follows every system's bin matrix (required by
// the 16-bit layout)
cudaError_t launch(Hist32Args &a, bool codes, bool streamed, void *scratch, size_t scratch_bytes, cudaStream_t st) {
    if (!config(a.bmax, &a.fc, &a.nst)) return cudaErrorInvalidValue;
    if (!wide_counters(a.bmax) && !codes) return cudaErrorInvalidValue;
    if (a.n_tiles <= 0) return cudaSuccess;
    const int grid = (int)std::min<int64_t>(a.n_tiles, sm_count());
    const size_t need = pairs_hist32_scratch_bytes(a.bmax, grid);
    if (!scratch || scratch_bytes < need) return cudaErrorInvalidValue;
    cudaError_t e = wide_counters(a.bmax) ? cudaSuccess : cudaMemsetAsync(scratch, 0, need, st);
    if (e != cudaSuccess) return e;
    a.ovf_all = (uint32_t *)scratch;
    a.kw = 128u;
    a.kneg = 0u - (128u << 16);
    const size_t smem = streamed ? hist32_bytes(a.bmax) : smem_bytes(a.bmax, a.fc, a.nst);
    auto go = [&](auto kern) -> cudaError_t {
        cudaError_t e2 = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e2 != cudaSuccess) return e2;
        kern<<<grid, kThreads, smem, st>>>(a);
        return cudaGetLastError();
    };
    if (streamed) return wide_counters(a.bmax) ? go(pairs_hist32s_kernel<true>) : go(pairs_hist32s_kernel<false>);
    return wide_counters(a.bmax) ? go(pairs_hist32_kernel<true>) : go(pairs_hist32_kernel<false>);
}

}  // namespace

bool pairs_hist32_supported(int bmax) {
    int fc = 0, nst = 0;
    return bmax >= 1 && bmax <= kBmax16 && config(bmax, &fc, &nst);
}

bool pairs_hist32_wide(int bmax) { return pairs_hist32_supported(bmax) && wide_counters(bmax); }

int pairs_hist32_grid(int64_t n_tiles) { return (int)std::max<int64_t>(1, std::min<int64_t>(n_tiles, sm_count())); }

// overflow-count bytes for `grid` CTAs
size_t pairs_hist32_scratch_bytes(int bmax, int grid) {
    if (wide_counters(bmax)) return 256;  // 32-bit counters never move counts out
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

cudaError_t launch_pairs_hist32(const SysGeom &g, const uint8_t *bins, const DofArrays &dof,
                                const unsigned long long *nfix, double fix, const PairTile *tiles, int64_t n_tiles,
                                PairOut out, int *err, void *scratch, size_t scratch_bytes, cudaStream_t st) {
    int bmax = 1;
    for (int t = 0; t < 3; t++) bmax = bmax > g.bins[3 + t] ? bmax : g.bins[3 + t];
    if (!pairs_hist32_supported(bmax)) return cudaErrorInvalidValue;
    if (!g.ilv && g.ldb < bins_ld(g.F)) return cudaErrorInvalidValue;
    Hist32Args a{};
    a.one.geo = g;
    a.one.bins = bins;
    a.one.dof = dof;
    a.one.out = out;
    a.one.lnN = log((double)g.F);
    a.tiles = tiles;
    a.n_tiles = n_tiles;
    a.nfix = nfix;
    a.fix = fix;
    a.err = err;
    a.bmax = bmax;
    return launch(a, g.codes != 0, g.ilv != 0, scratch, scratch_bytes, st);
}

cudaError_t launch_pairs_hist32_batch(int bmax, bool codes, bool ilv, const SysDesc *sys, const PairTile *tiles,
                                      const int *tile_sys, int64_t n_tiles, const unsigned long long *nfix,
                                      double fix, int *err, void *scratch, size_t scratch_bytes, cudaStream_t st) {
    if (!pairs_hist32_supported(bmax)) return cudaErrorInvalidValue;
    Hist32Args a{};
    a.many = sys;
    a.tiles = tiles;
    a.tile_sys = tile_sys;
    a.n_tiles = n_tiles;
    a.nfix = nfix;
    a.fix = fix;
    a.err = err;
    a.bmax = bmax;
    return launch(a, codes, ilv, scratch, scratch_bytes, st);
}

}  // namespace pg
