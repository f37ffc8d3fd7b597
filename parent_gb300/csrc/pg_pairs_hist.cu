// Pair kernel, shared-memory histogram form.
//
// Replaces the fifteen 2D fill + epilogue loops of PARENT.cpp (bb :786-823,
// ba :826-856, bd :858-886, aa :1141-1176, ad :1178-1206, dd :1383-1414 and
// their remote-rank copies). A pair tile is T row DOFs x T column DOFs
// (T = 4 -> 16 pairs). The kernel is persistent: one CTA per SM walks the
// tile list with a stride of the grid size, so the CTA's shared-memory
// histograms, barriers and staging ring live across tiles.
//
// Warp 31 is the producer: it streams every chunk of every tile of the CTA,
// the tile's 2T uint8 bin rows per chunk, into a ring of shared-memory stages
// with bulk TMA copies (cp.async.bulk, completion on a full[] mbarrier), one
// row per lane issued in parallel, and refills a stage once every consumer
// warp has released it (empty[]). It runs ahead into the next tile while the
// consumers finish the current one, so no tile starts with an empty pipeline.
//
// Warps 0-30 consume: every lane owns one pair slot p and a frame sub-stream
// and adds 1 to hist[(br*Bc + bc)*PPS + p] with a shared-memory reduction, so
// the PPS pair histograms are interleaved word by word and lanes of different
// pairs never share a bank.
//
// Epilogue (consumers only, per tile): each histogram is reduced to
// sum n ln n and the occupied bin count while the words are reset to zero
// for the next tile. n ln n comes from a fixed-point table (n ln n * 2^s, s
// chosen from F so that any histogram's total stays below 2^64): the sums
// are 64-bit integer additions, exact and independent of the order the warps
// arrive in, and they keep the FP64 pipe (a small fraction of the integer
// rate on this part) out of the per-bin work. The
// 2D entropy then follows from the exact decomposition
//   S_ij = ln N + A_i + A_j - (1/N) sum n ln n + (occ - 1) / (2N)
// (A from the preprocessing kernel), the mutual information from
//   MI = S1_i + S1_j - S_ij   (get_mutual, util.cpp:47-81),
// S_ij goes into the .par body layout and MI into the dense matrix. No
// histogram ever reaches global memory.
#include <stdio.h>
#include <stdlib.h>

#include "pg_internal.h"
#include "pg_sync.cuh"

namespace pg {

namespace {

using namespace dev;

constexpr int kThreads = 1024;
constexpr int kWarps = kThreads / 32;
constexpr int kConsumers = kWarps - 1;           // warps 0..30
constexpr int kConsumerThreads = kConsumers * 32;
constexpr int kMaxStages = 4;
constexpr int kSmemMax = 232448;   // 227 KB opt-in per block on sm_100-class parts
constexpr int kStagePad = 32;      // bytes between staged rows: puts the 2T rows on distinct banks

__host__ __device__ __forceinline__ size_t hist_bytes(int bmax, int pps) {
    return ((size_t)bmax * bmax * pps * 4 + 127) / 128 * 128;
}

// hist[word] += 1 in shared memory, result unused; ordering with the stage
// release and the barriers comes from those instructions' own clobbers
__device__ __forceinline__ void red_add1_at(uint32_t saddr) {
    asm volatile("red.shared.add.u32 [%0], 1;" ::"r"(saddr));
}
__device__ __forceinline__ void red_add1(unsigned int *p) { red_add1_at(smem_u32(p)); }

template <int T>
struct TileCfg {
    static constexpr int PPS = T * T;      // pair slots
    static constexpr int NSUB = 32 / PPS;  // frame sub-streams per warp
    static constexpr int NROW = 2 * T;     // staged bin rows
    static constexpr int SHIFT = T == 4 ? 6 : (T == 2 ? 4 : 2);  // log2(PPS * 4)
};

// Launch arguments. A single-system launch passes its system in `one` and
// tile_sys = nullptr; a batched launch passes per-tile system indices into
// `many`.
struct HistArgs {
    SysDesc one;
    const SysDesc *many;
    const PairTile *tiles;
    const int *tile_sys;
    int64_t n_tiles;
    const unsigned long long *nfix;
    double fix;
    int *err;
    int fc, nst, bmax;
};

template <int T>
__global__ void __launch_bounds__(kThreads, 1) pairs_hist_kernel(const __grid_constant__ HistArgs a) {
    using C = TileCfg<T>;
    constexpr int PPS = C::PPS, NSUB = C::NSUB, NROW = C::NROW;
    constexpr int SH = C::SHIFT;  // log2(bytes between consecutive bins of one slot)
    constexpr int NJ = kConsumerThreads / PPS;  // epilogue threads per slot
    extern __shared__ __align__(128) unsigned char smem[];
    const int fc = a.fc, nst = a.nst;
    const int hist_words = a.bmax * a.bmax * PPS;
    unsigned int *hist = (unsigned int *)smem;
    const int fcs = fc + kStagePad;
    unsigned char *stage = smem + hist_bytes(a.bmax, PPS);  // [nst][NROW][fcs], 128-B aligned
    uint64_t *full = (uint64_t *)(stage + (size_t)nst * NROW * fcs);
    uint64_t *empty = full + kMaxStages;
    __shared__ unsigned long long s_snl[PPS];
    __shared__ unsigned int s_occ[PPS];
    __shared__ volatile int s_abort;    // written by consumers only (read by all after a barrier)
    __shared__ volatile int s_pabort;   // written by the producer
    __shared__ long long s_issued;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    for (int i = tid * 4; i < hist_words; i += kThreads * 4) {
        if (i + 4 <= hist_words) *(uint4 *)(hist + i) = make_uint4(0u, 0u, 0u, 0u);
        else for (int k = i; k < hist_words; k++) hist[k] = 0u;
    }
    if (tid < PPS) {
        s_snl[tid] = 0ull;
        s_occ[tid] = 0u;
    }
    if (tid == 0) {
        s_abort = 0;
        s_pabort = 0;
        s_issued = 0;
        for (int k = 0; k < nst; k++) {
            mbar_init(smem_u32(&full[k]), 1);             // producer arrival + tx bytes
            mbar_init(smem_u32(&empty[k]), kConsumers);   // one arrival per consumer warp
        }
        mbar_init_fence();
    }
    __syncthreads();

    auto sys_of = [&](int64_t t) -> const SysDesc & { return a.tile_sys ? a.many[a.tile_sys[t]] : a.one; };

    if (warp == kConsumers) {
        // ---------------------------------------------------------- producer
        // lane 0 waits for a free stage and arms its full barrier; lanes
        // 0..NROW-1 then issue one row copy each, in parallel
        long long seq = 0;
        bool ok = true;
        for (int64_t t = blockIdx.x; t < a.n_tiles && ok; t += gridDim.x) {
            const SysDesc &d = sys_of(t);
            const PairTile tile = a.tiles[t];
            const int nchunks = (d.geo.F + fc - 1) / fc;
            const uint8_t *src = nullptr;
            if (lane < NROW) {
                const int k = lane;
                const int g = k < T ? (k < tile.nrow ? tile.row0 + k : -1)
                                    : ((k - T) < tile.ncol ? tile.col0 + (k - T) : -1);
                src = g >= 0 ? d.bins + (int64_t)g * d.geo.ldb : nullptr;
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
                    bulk_g2s(smem_u32(stage + (size_t)(st * NROW + lane) * fcs), src + (int64_t)chunk * fc,
                             (uint32_t)fc, smem_u32(&full[st]));
                }
            }
        }
        if (lane == 0) s_issued = seq;
    } else {
        // --------------------------------------------------------- consumers
        const int p = lane % PPS, sub = lane / PPS;
        const int pr = p / T, pc = p % T;
        const uint32_t hbase = smem_u32(hist + p);
        constexpr int S = kConsumers * NSUB;
        const int gstep = (fc / 16) % S;
        const int ctid = tid;  // 0 .. kConsumerThreads-1
        const int ep = ctid % PPS, ej = ctid / PPS;
        const int er = ep / T, ec = ep % T;
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
            // 16-frame groups go round-robin over the S (warp, sub-stream)
            // slots; each chunk starts one chunk's group count further along,
            // so the leftover groups rotate over the warps
            int g0 = warp * NSUB + sub;
            for (int chunk = 0; chunk < nchunks; chunk++, seq++) {
                const int st = (int)(seq % nst);
                if (!mbar_wait_bounded(smem_u32(&full[st]), (uint32_t)((seq / nst) & 1))) {
                    s_abort = 1;
                    break;
                }
                const int fvalid = min(fc, F - chunk * fc);
                const unsigned char *rrow = stage + (size_t)(st * NROW + pr) * fcs;
                const unsigned char *crow = stage + (size_t)(st * NROW + T + pc) * fcs;
                if (valid) {
                    const int fend = fvalid & ~15;  // frames in whole 16-frame groups
                    int off = g0 * 16;
                    for (; off < fend; off += S * 16) {
                        const uint4 rv = *(const uint4 *)(rrow + off);
                        const uint4 cv = *(const uint4 *)(crow + off);
                        const uint32_t rw[4] = {rv.x, rv.y, rv.z, rv.w};
                        const uint32_t cw[4] = {cv.x, cv.y, cv.z, cv.w};
                        {
                            // two frames per 32-bit IMAD: bytes spread into
                            // 16-bit halves, idx = br*Bc + bc < 65536 never
                            // carries across
                            uint32_t ix[8];
#pragma unroll
                            for (int q = 0; q < 4; q++) {
                                ix[2 * q] = __byte_perm(rw[q], 0u, 0x4140) * Bc + __byte_perm(cw[q], 0u, 0x4140);
                                ix[2 * q + 1] = __byte_perm(rw[q], 0u, 0x4342) * Bc + __byte_perm(cw[q], 0u, 0x4342);
                            }
                            // frames in the order 0, 4, 8, 12, 1, 5, ...: consecutive
                            // reductions of a lane are four frames apart (runs of one
                            // bin do not queue back-to-back read-modify-writes on one word)
#pragma unroll
                            for (int k = 0; k < 4; k++) {
#pragma unroll
                                for (int q = 0; q < 4; q++) {
                                    const uint32_t v = ix[2 * q + (k >> 1)];
                                    red_add1_at(hbase + (((k & 1) ? (v >> 16) : (v & 0xffffu)) << SH));
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
                                    red_add1_at(hbase + ((br * Bc + bc) << SH));
                                }
                            }
                        }
                    }
                }
                __syncwarp();
                if (lane == 0) mbar_arrive_relaxed(smem_u32(&empty[st]));
                g0 -= gstep;
                if (g0 < 0) g0 += S;
            }
            // every consumer's reductions for this tile are done
            named_barrier(kConsumerThreads);
            if (s_abort) break;  // the same value for every consumer (no writes until the next tile)

            // ---- epilogue: sum n ln n and occupied bins per slot; zero the
            // words for the next tile
            const int egr = er < tile.nrow ? tile.row0 + er : -1;
            const int egc = ec < tile.ncol ? tile.col0 + ec : -1;
            const bool evalid = egr >= 0 && egc >= 0 && egr < egc;
            unsigned long long snl = 0ull;
            int occ = 0;
            if (evalid) {
                const int nbin = d.dof.b2[egr] * d.dof.b2[egc];
                unsigned int *h = hist + ep;
                if (d.out.counts) {
                    int64_t *dst = d.out.counts + (t * PPS + ep) * d.out.counts_bmax * d.out.counts_bmax;
                    for (int bin = ej; bin < nbin; bin += NJ) dst[bin] = h[bin * PPS];
                }
                int bin = ej;
                for (; bin + 3 * NJ < nbin; bin += 4 * NJ) {
                    const unsigned int n0 = h[bin * PPS], n1 = h[(bin + NJ) * PPS];
                    const unsigned int n2 = h[(bin + 2 * NJ) * PPS], n3 = h[(bin + 3 * NJ) * PPS];
                    h[bin * PPS] = 0u;
                    h[(bin + NJ) * PPS] = 0u;
                    h[(bin + 2 * NJ) * PPS] = 0u;
                    h[(bin + 3 * NJ) * PPS] = 0u;
                    snl += __ldg(a.nfix + n0) + __ldg(a.nfix + n1) + __ldg(a.nfix + n2) + __ldg(a.nfix + n3);
                    occ += (n0 != 0u) + (n1 != 0u) + (n2 != 0u) + (n3 != 0u);
                }
                for (; bin < nbin; bin += NJ) {
                    const unsigned int n = h[bin * PPS];
                    h[bin * PPS] = 0u;
                    snl += __ldg(a.nfix + n);
                    occ += n != 0u;
                }
            }
            // lanes l and l+PPS*k of a warp hold the same slot: fold them
            for (int o = 16; o >= PPS; o >>= 1) {
                snl += __shfl_down_sync(0xffffffffu, snl, o);
                occ += __shfl_down_sync(0xffffffffu, occ, o);
            }
            if (lane < PPS && evalid) {
                atomicAdd(&s_snl[ep], snl);
                atomicAdd(&s_occ[ep], (unsigned int)occ);
            }
            named_barrier(kConsumerThreads);
            if (ctid < PPS) {
                if (evalid) {
                    const double N = (double)F;
                    const double s = (double)s_snl[ctid] / a.fix;
                    const int o = (int)s_occ[ctid];
                    const double S2 = d.lnN + d.dof.acon[egr] + d.dof.acon[egc] - s / N + (o - 1.0) / (2.0 * N);
                    if (d.out.par) d.out.par[par_pair_index(d.out.L, d.geo.nb, d.geo.na, d.geo.nd, egr, egc)] = S2;
                    if (d.out.mi) {
                        const double mi = d.dof.s1[egr] + d.dof.s1[egc] - S2;
                        d.out.mi[(int64_t)egr * d.geo.D + egc] = mi;
                        d.out.mi[(int64_t)egc * d.geo.D + egr] = mi;
                    }
                }
                // the next tile's atomics follow its streaming barrier
                s_snl[ctid] = 0ull;
                s_occ[ctid] = 0u;
            }
        }
    }
    __syncthreads();

    if (s_abort || s_pabort) {
        // a wait ran out: record it, let every copy that may still be in
        // flight land (bounded), and leave
        if (tid == 0) {
            atomicAdd(&a.err[ERR_TIMEOUT], 1);
            const long long n = s_issued;
            for (long long k = n > nst ? n - nst : 0; k < n; k++)
                (void)mbar_wait_bounded(smem_u32(&full[k % nst]), (uint32_t)((k / nst) & 1));
        }
        __syncthreads();
    }
}

template <int T>
size_t smem_bytes(int bmax, int fc, int nst) {
    const size_t stage = (size_t)nst * TileCfg<T>::NROW * (fc + kStagePad);
    return hist_bytes(bmax, TileCfg<T>::PPS) + stage + 8 * 2 * kMaxStages;
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

template <int T>
cudaError_t launch_t(const HistArgs &a, int smem, cudaStream_t st) {
    cudaError_t e = cudaFuncSetAttribute(pairs_hist_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    const int64_t grid = a.n_tiles < sm_count() ? a.n_tiles : sm_count();
    pairs_hist_kernel<T><<<(unsigned)grid, kThreads, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_any(const HistArgs &a, int T, int smem, cudaStream_t st) {
    if (T == 4) return launch_t<4>(a, smem, st);
    if (T == 2) return launch_t<2>(a, smem, st);
    return launch_t<1>(a, smem, st);
}

}  // namespace

// Roofline probe: warp-wide shared-memory reductions where lane l always hits
// bank l (one wavefront per instruction), the access pattern the pair kernel
// is built around. Unrolled with immediate offsets so the loop is one RED per
// reduction; the measured rate is the denominator of the kernel's roofline.
__global__ void __launch_bounds__(1024) smem_red_probe(int iters, unsigned int *sink) {
    __shared__ unsigned int h[64 * 32];
    for (int i = threadIdx.x; i < 64 * 32; i += blockDim.x) h[i] = 0u;
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int it = 0; it < iters; it++) {
        unsigned int *p = h + lane + ((w + it) & 31) * 32;
#pragma unroll
        for (int k = 0; k < 32; k++) red_add1(p + k * 32);
    }
    __syncthreads();
    if (threadIdx.x == 0) sink[blockIdx.x] = h[0];
}

// Chooses the tile side T (4, 2, 1 DOFs: 16, 4, 1 pair slots) and the
// staging geometry (frames per chunk x stages) that fit the shared memory for
// the largest 2D bin count. PG_HIST_FC / PG_HIST_STAGES override the staging
// for tuning sweeps when they fit.
int pairs_hist_config(int bmax, int *tile_dim, int *chunk_frames, int *stages) {
    // the largest chunks that fit: measured rates fall with the chunk size
    // (per-chunk synchronisation), and a chunk size that splits evenly over
    // the 62 (warp, sub-stream) slots (3,968) measured no better than 4,096
    static const int cand[][2] = {{4096, 2}, {2048, 4}, {2048, 3}, {2048, 2}, {1024, 4}, {1024, 2}};
    int ofc = 0, onst = 0;
    if (const char *e = getenv("PG_HIST_FC")) ofc = atoi(e);
    if (const char *e = getenv("PG_HIST_STAGES")) onst = atoi(e);
    for (int T : {4, 2, 1}) {
        auto need = [&](int fc, int nst) -> size_t {
            return T == 4 ? smem_bytes<4>(bmax, fc, nst)
                          : (T == 2 ? smem_bytes<2>(bmax, fc, nst) : smem_bytes<1>(bmax, fc, nst));
        };
        // a chunk of at most 4096 frames never reads past its row (bins_ld)
        const bool ovr = ofc >= 256 && ofc <= 4096 && ofc % 16 == 0 && onst >= 2 && onst <= kMaxStages;
        if (ovr && need(ofc, onst) + 1024 <= (size_t)kSmemMax) {
            *tile_dim = T; *chunk_frames = ofc; *stages = onst;
            return (int)need(ofc, onst);
        }
        for (const auto &c : cand) {
            if (need(c[0], c[1]) + 1024 <= (size_t)kSmemMax) {  // + the kernel's static smem
                *tile_dim = T; *chunk_frames = c[0]; *stages = c[1];
                return (int)need(c[0], c[1]);
            }
        }
    }
    return 0;
}

cudaError_t launch_pairs_hist(const SysGeom &g, const uint8_t *bins, const DofArrays &dof,
                              const unsigned long long *nfix, double fix, const PairTile *tiles, int64_t n_tiles,
                              int tile_dim, PairOut out, int *err, cudaStream_t st) {
    int bmax = 1;
    for (int t = 0; t < 3; t++) bmax = bmax > g.bins[3 + t] ? bmax : g.bins[3 + t];
    int T = 0, fc = 0, nst = 0;
    const int smem = pairs_hist_config(bmax, &T, &fc, &nst);
    if (!smem || T != tile_dim) return cudaErrorInvalidValue;
    if (n_tiles <= 0) return cudaSuccess;
    if ((int64_t)g.ldb < (int64_t)((g.F + fc - 1) / fc) * fc) return cudaErrorInvalidValue;
    HistArgs a{};
    a.one.geo = g;
    a.one.bins = bins;
    a.one.dof = dof;
    a.one.out = out;
    a.one.lnN = log((double)g.F);
    a.many = nullptr;
    a.tiles = tiles;
    a.tile_sys = nullptr;
    a.n_tiles = n_tiles;
    a.nfix = nfix;
    a.fix = fix;
    a.err = err;
    a.fc = fc;
    a.nst = nst;
    a.bmax = bmax;
    return launch_any(a, T, smem, st);
}

cudaError_t launch_pairs_hist_batch(int bmax, const SysDesc *sys, const PairTile *tiles, const int *tile_sys,
                                    int64_t n_tiles, const unsigned long long *nfix, double fix, int *err,
                                    int tile_dim, cudaStream_t st) {
    int T = 0, fc = 0, nst = 0;
    const int smem = pairs_hist_config(bmax, &T, &fc, &nst);
    if (!smem || T != tile_dim) return cudaErrorInvalidValue;
    if (n_tiles <= 0) return cudaSuccess;
    HistArgs a{};
    a.many = sys;
    a.tiles = tiles;
    a.tile_sys = tile_sys;
    a.n_tiles = n_tiles;
    a.nfix = nfix;
    a.fix = fix;
    a.err = err;
    a.fc = fc;
    a.nst = nst;
    a.bmax = bmax;
    return launch_any(a, T, smem, st);
}

// A wait that nothing completes: thread 0 waits on a fresh mbarrier (one
// expected arrival, none made) with the pair kernels' bounded wait and
// records the timeout the way they do.
__global__ void wait_timeout_probe(long long limit, int *err) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(smem_u32(&bar), 1);
        mbar_init_fence();
        if (!mbar_wait_bounded(smem_u32(&bar), 0u, limit)) atomicAdd(&err[ERR_TIMEOUT], 1);
    }
}

cudaError_t launch_wait_timeout_probe(long long limit_cycles, int *err, cudaStream_t st) {
    wait_timeout_probe<<<1, 32, 0, st>>>(limit_cycles, err);
    return cudaGetLastError();
}

double probe_smem_red_rate(int n_sm, cudaStream_t st, int *launches) {
    unsigned int *sink = nullptr;
    if (cudaMalloc(&sink, sizeof(unsigned int) * 2 * n_sm) != cudaSuccess) return -1.0;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const int iters = 4096, blocks = 2 * n_sm;
    smem_red_probe<<<blocks, 1024, 0, st>>>(64, sink);  // warm-up
    cudaEventRecord(a, st);
    smem_red_probe<<<blocks, 1024, 0, st>>>(iters, sink);
    cudaEventRecord(b, st);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    *launches += 2;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(sink);
    if (cudaGetLastError() != cudaSuccess || ms <= 0.f) return -1.0;
    return (double)blocks * 1024.0 * iters * 32.0 / (ms * 1e-3);
}

}  // namespace pg
