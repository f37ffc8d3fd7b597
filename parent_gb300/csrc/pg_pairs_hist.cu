// Pair kernel, shared-memory histogram form.
//
// Replaces the fifteen 2D fill + epilogue loops of PARENT.cpp (bb :786-823,
// ba :826-856, bd :858-886, aa :1141-1176, ad :1178-1206, dd :1383-1414 and
// their remote-rank copies). One CTA owns one pair tile: T row DOFs x T
// column DOFs (T = 4 -> 16 pairs). Per frame chunk, one elected thread
// stages the tile's 2T uint8 bin rows into shared memory with bulk TMA copies
// (cp.async.bulk, completion on an mbarrier; two stages). Every lane owns one
// pair slot p and a frame sub-stream s; it adds 1 to hist[(br*Bc + bc)*PPS + p]
// with a shared-memory reduction, so the PPS pair histograms are interleaved
// word by word and lanes of different pairs never share a bank.
//
// The epilogue reduces each histogram to sum n ln n (FP64 table lookup) and
// the occupied-bin count, then forms the 2D entropy through the exact
// decomposition
//   S_ij = ln N + A_i + A_j - (1/N) sum n ln n + (occ - 1) / (2N)
// (A from the preprocessing kernel), the mutual information
//   MI = S1_i + S1_j - S_ij   (get_mutual, util.cpp:47-81)
// and writes S_ij into the .par body layout and MI into the dense matrix.
// No histogram ever reaches global memory.
#include <stdio.h>
#include <stdlib.h>

#include "pg_internal.h"

namespace pg {

namespace {

constexpr int kThreads = 1024;
constexpr int kWarps = kThreads / 32;
constexpr int kMaxStages = 4;
constexpr int kSmemMax = 232448;   // 227 KB opt-in per block on sm_100-class parts
constexpr int kStagePad = 32;      // bytes between staged rows: puts the 2T rows on distinct banks
constexpr long long kWaitCycles = 4000000000LL;  // ~2 s at 2 GHz, then report a timeout

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// Relaxed arrive: a consumer warp releases a stage after the values it read
// from it have been used, without waiting for its own shared-memory
// reductions (which never touch the stage) to drain.
__device__ __forceinline__ void mbar_arrive_relaxed(uint32_t bar) {
    asm volatile("mbarrier.arrive.relaxed.cta.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
// Bounded wait: gives up after kWaitCycles and returns false.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (clock64() - t0 > kWaitCycles) return false;
    }
    return true;
}
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
        "l"(src), "r"(bytes), "r"(bar)
        : "memory");
}

__host__ __device__ __forceinline__ size_t hist_bytes(int bmax, int pps) {
    return ((size_t)bmax * bmax * pps * 4 + 127) / 128 * 128;
}

// hist[word] += 1 in shared memory, result unused
__device__ __forceinline__ void red_add1_at(uint32_t saddr) {
    asm volatile("red.shared.add.u32 [%0], 1;" ::"r"(saddr));  // ordering comes from the arrive/barrier clobbers
}
__device__ __forceinline__ void red_add1(unsigned int *p) { red_add1_at(smem_u32(p)); }

template <int T>
struct TileCfg {
    static constexpr int PPS = T * T;      // pair slots
    static constexpr int NSUB = 32 / PPS;  // frame sub-streams per warp
    static constexpr int NROW = 2 * T;     // staged bin rows
    static constexpr int SHIFT = T == 4 ? 6 : (T == 2 ? 4 : 2);  // log2(PPS * 4)
};

// One CTA's work on one tile; shared by the single-system kernel and the
// batched kernel (which reads geometry and outputs per tile from SysDesc).
template <int T>
__device__ __forceinline__ void pairs_hist_body(const SysGeom &geo, const uint8_t *__restrict__ bins,
                                                const DofArrays &dof, const double *__restrict__ nlogn,
                                                const PairTile tile, int64_t tile_index, const PairOut &out,
                                                int *err, int fc, int nst, int bmax, double lnN) {
    using C = TileCfg<T>;
    constexpr int PPS = C::PPS, NSUB = C::NSUB, NROW = C::NROW;
    constexpr int SH = C::SHIFT;  // log2(bytes between consecutive bins of one slot)
    extern __shared__ __align__(128) unsigned char smem[];
    const int hist_words = bmax * bmax * PPS;
    unsigned int *hist = (unsigned int *)smem;
    const int fcs = fc + kStagePad;
    unsigned char *stage = smem + hist_bytes(bmax, PPS);  // [nst][NROW][fcs], 128-B aligned
    uint64_t *mbar = (uint64_t *)(stage + (size_t)nst * NROW * fcs);
    __shared__ volatile int s_abort;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int F = geo.F;

    // staged row k: row DOF row0+k (k < T), column DOF col0+k-T (k >= T)
    auto row_dof = [&](int k) -> int {
        if (k < T) return k < tile.nrow ? tile.row0 + k : -1;
        return (k - T) < tile.ncol ? tile.col0 + (k - T) : -1;
    };

    for (int i = tid * 4; i < hist_words; i += kThreads * 4) {
        if (i + 4 <= hist_words) *(uint4 *)(hist + i) = make_uint4(0u, 0u, 0u, 0u);
        else for (int k = i; k < hist_words; k++) hist[k] = 0u;
    }
    if (tid == 0) {
        s_abort = 0;
        for (int k = 0; k < nst; k++) {
            mbar_init(smem_u32(&mbar[k]), 1);                            // full[k]: producer + tx bytes
            mbar_init(smem_u32(&mbar[kMaxStages + k]), kWarps - 1);      // empty[k]: one per consumer warp
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    const int nchunks = (F + fc - 1) / fc;
    // Warp-specialised pipeline: warp kWarps-1 is the producer (one lane
    // issues the bulk copies); warps 0..kWarps-2 consume. full[st] completes
    // when a stage's bytes have landed; empty[st] when every consumer warp is
    // done reading it. No CTA-wide barrier inside the loop, so the warps'
    // in-flight shared-memory reductions never have to drain together.
    constexpr int kConsumers = kWarps - 1;
    uint64_t *full = mbar, *empty = mbar + kMaxStages;
    if (warp == kConsumers) {
        if (lane == 0) {
            for (int chunk = 0; chunk < nchunks; chunk++) {
                const int st = chunk % nst;
                if (chunk >= nst &&
                    !mbar_wait_bounded(smem_u32(&empty[st]), (uint32_t)(((chunk / nst) - 1) & 1))) {
                    s_abort = 1;
                    break;
                }
                // generic-proxy reads of this stage (released by the empty
                // barrier) before the async-proxy writes that refill it
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                uint32_t bytes = 0;
                for (int k = 0; k < NROW; k++) bytes += row_dof(k) >= 0 ? (uint32_t)fc : 0u;
                const uint32_t bar = smem_u32(&full[st]);
                mbar_expect_tx(bar, bytes);
                for (int k = 0; k < NROW; k++) {
                    const int g = row_dof(k);
                    if (g < 0) continue;
                    bulk_g2s(smem_u32(stage + (size_t)(st * NROW + k) * fcs),
                             bins + (int64_t)g * geo.ldb + (int64_t)chunk * fc, (uint32_t)fc, bar);
                }
            }
        }
    } else {
        // this lane's pair slot
        const int p = lane % PPS, sub = lane / PPS;
        const int pr = p / T, pc = p % T;
        const int gr = pr < tile.nrow ? tile.row0 + pr : -1;
        const int gc = pc < tile.ncol ? tile.col0 + pc : -1;
        const bool valid = gr >= 0 && gc >= 0 && gr < gc;
        const uint32_t Bc = valid ? (uint32_t)dof.b2[gc] : 0u;
        const uint32_t hbase = smem_u32(hist + p);
        // 16-frame groups go round-robin over the S (warp, sub-stream) slots;
        // each chunk starts one chunk's group count further along, so the
        // leftover groups rotate over the warps instead of always landing on
        // the first ones
        constexpr int S = kConsumers * NSUB;
        const int gstep = (fc / 16) % S;
        int g0 = warp * NSUB + sub;
        for (int chunk = 0; chunk < nchunks; chunk++) {
            const int st = chunk % nst;
            if (!mbar_wait_bounded(smem_u32(&full[st]), (uint32_t)((chunk / nst) & 1))) {
                s_abort = 1;
                break;
            }
            const int fvalid = min(fc, F - chunk * fc);
            const unsigned char *rrow = stage + (size_t)(st * NROW + pr) * fcs;
            const unsigned char *crow = stage + (size_t)(st * NROW + T + pc) * fcs;
            if (valid) {
                for (int off = g0 * 16; off < fvalid; off += S * 16) {
                    const uint4 rv = *(const uint4 *)(rrow + off);
                    const uint4 cv = *(const uint4 *)(crow + off);
                    const uint32_t rw[4] = {rv.x, rv.y, rv.z, rv.w};
                    const uint32_t cw[4] = {cv.x, cv.y, cv.z, cv.w};
                    if (off + 16 <= fvalid) {
                        // two frames per 32-bit IMAD: bytes spread into 16-bit
                        // halves, idx = br*Bc + bc < 65536 never carries across
#pragma unroll
                        for (int q = 0; q < 4; q++) {
                            const uint32_t i01 = __byte_perm(rw[q], 0u, 0x4140) * Bc + __byte_perm(cw[q], 0u, 0x4140);
                            const uint32_t i23 = __byte_perm(rw[q], 0u, 0x4342) * Bc + __byte_perm(cw[q], 0u, 0x4342);
                            red_add1_at(hbase + ((i01 & 0xffffu) << SH));
                            red_add1_at(hbase + ((i01 >> 16) << SH));
                            red_add1_at(hbase + ((i23 & 0xffffu) << SH));
                            red_add1_at(hbase + ((i23 >> 16) << SH));
                        }
                    } else {  // ragged end of the trajectory
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
    }
    __syncthreads();

    if (s_abort) {
        // a stage never completed: record it, drain every copy that may still
        // be in flight (bounded), and leave without writing results
        if (tid == 0) {
            atomicAdd(&err[ERR_TIMEOUT], 1);
            for (int c = 0; c < nst; c++) (void)mbar_wait_bounded(smem_u32(&full[c]), 0u);
        }
        __syncthreads();
        return;
    }

    // ---- epilogue: per pair slot, sum n ln n and occupied bins. The staging
    // area is free now and holds the cross-warp partial sums.
    double *red_snl = (double *)stage;               // [kWarps][PPS]
    int *red_occ = (int *)(red_snl + kWarps * PPS);  // [kWarps][PPS]
    const int ep = tid % PPS, ej = tid / PPS;  // kThreads/PPS threads per slot
    const int er = ep / T, ec = ep % T;
    const int egr = er < tile.nrow ? tile.row0 + er : -1;
    const int egc = ec < tile.ncol ? tile.col0 + ec : -1;
    const bool evalid = egr >= 0 && egc >= 0 && egr < egc;
    double snl = 0.0;
    int occ = 0;
    if (evalid) {
        const int nbin = dof.b2[egr] * dof.b2[egc];
        for (int bin = ej; bin < nbin; bin += kThreads / PPS) {
            const unsigned int n = hist[bin * PPS + ep];
            if (n) {
                snl += __ldg(nlogn + n);
                occ++;
            }
        }
        if (out.counts) {
            int64_t *dst = out.counts + (tile_index * PPS + ep) * out.counts_bmax * out.counts_bmax;
            for (int bin = ej; bin < nbin; bin += kThreads / PPS) dst[bin] = hist[bin * PPS + ep];
        }
    }
    // lanes l and l+PPS*k of a warp hold the same slot: fold them first
    for (int o = 16; o >= PPS; o >>= 1) {
        snl += __shfl_down_sync(0xffffffffu, snl, o);
        occ += __shfl_down_sync(0xffffffffu, occ, o);
    }
    if (lane < PPS) {
        red_snl[warp * PPS + lane] = snl;
        red_occ[warp * PPS + lane] = occ;
    }
    __syncthreads();
    if (tid < PPS && evalid) {
        double s = 0.0;
        int o = 0;
        for (int w = 0; w < kWarps; w++) {
            s += red_snl[w * PPS + tid];
            o += red_occ[w * PPS + tid];
        }
        const double N = (double)F;
        const double S2 = lnN + dof.acon[egr] + dof.acon[egc] - s / N + (o - 1.0) / (2.0 * N);
        if (out.par) out.par[par_pair_index(out.L, geo.nb, geo.na, geo.nd, egr, egc)] = S2;
        if (out.mi) {
            const double mi = dof.s1[egr] + dof.s1[egc] - S2;
            out.mi[(int64_t)egr * geo.D + egc] = mi;
            out.mi[(int64_t)egc * geo.D + egr] = mi;
        }
    }
}

template <int T>
__global__ void __launch_bounds__(kThreads, 1)
pairs_hist_kernel(SysGeom geo, const uint8_t *__restrict__ bins, DofArrays dof,
                  const double *__restrict__ nlogn, const PairTile *__restrict__ tiles,
                  PairOut out, int *err, int fc, int nst, int bmax, double lnN) {
    pairs_hist_body<T>(geo, bins, dof, nlogn, tiles[blockIdx.x], blockIdx.x, out, err, fc, nst, bmax, lnN);
}

// Many independent systems in one launch: tile k belongs to system tile_sys[k].
template <int T>
__global__ void __launch_bounds__(kThreads, 1)
pairs_hist_batch_kernel(const SysDesc *__restrict__ sys, const PairTile *__restrict__ tiles,
                        const int *__restrict__ tile_sys, const double *__restrict__ nlogn, int *err, int fc,
                        int nst, int bmax) {
    const SysDesc &d = sys[tile_sys[blockIdx.x]];
    pairs_hist_body<T>(d.geo, d.bins, d.dof, nlogn, tiles[blockIdx.x], blockIdx.x, d.out, err, fc, nst, bmax,
                       d.lnN);
}

template <int T>
size_t smem_bytes(int bmax, int fc, int nst) {
    const size_t stage = (size_t)nst * TileCfg<T>::NROW * (fc + kStagePad);
    const size_t scratch = (size_t)kWarps * TileCfg<T>::PPS * (sizeof(double) + sizeof(int));
    return hist_bytes(bmax, TileCfg<T>::PPS) + (stage > scratch ? stage : scratch) + 8 * 2 * kMaxStages;
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
    static const int cand[][2] = {{4096, 2}, {2048, 4}, {2048, 3}, {2048, 2}, {1024, 4}, {1024, 2}};
    int ofc = 0, onst = 0;
    if (const char *e = getenv("PG_HIST_FC")) ofc = atoi(e);
    if (const char *e = getenv("PG_HIST_STAGES")) onst = atoi(e);
    for (int T : {4, 2, 1}) {
        auto need = [&](int fc, int nst) -> size_t {
            return T == 4 ? smem_bytes<4>(bmax, fc, nst)
                          : (T == 2 ? smem_bytes<2>(bmax, fc, nst) : smem_bytes<1>(bmax, fc, nst));
        };
        const bool ovr = ofc >= 512 && ofc <= 8192 && ofc % 512 == 0 && onst >= 2 && onst <= kMaxStages;
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
                              const double *nlogn, const PairTile *tiles, int64_t n_tiles,
                              int tile_dim, PairOut out, int *err, cudaStream_t st) {
    int bmax = 1;
    for (int t = 0; t < 3; t++) bmax = bmax > g.bins[3 + t] ? bmax : g.bins[3 + t];
    int T = 0, fc = 0, nst = 0;
    const int smem = pairs_hist_config(bmax, &T, &fc, &nst);
    if (!smem || T != tile_dim) return cudaErrorInvalidValue;
    if (n_tiles <= 0) return cudaSuccess;
    if ((int64_t)g.ldb < (int64_t)((g.F + fc - 1) / fc) * fc) return cudaErrorInvalidValue;
    const double lnN = log((double)g.F);
    cudaError_t e;
#define PG_LAUNCH(TT)                                                                              \
    e = cudaFuncSetAttribute(pairs_hist_kernel<TT>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                             smem);                                                               \
    if (e != cudaSuccess) return e;                                                               \
    pairs_hist_kernel<TT><<<(unsigned)n_tiles, kThreads, smem, st>>>(g, bins, dof, nlogn, tiles,  \
                                                                      out, err, fc, nst, bmax, lnN);
    if (T == 4) { PG_LAUNCH(4) } else if (T == 2) { PG_LAUNCH(2) } else { PG_LAUNCH(1) }
#undef PG_LAUNCH
    return cudaGetLastError();
}

cudaError_t launch_pairs_hist_batch(int bmax, const SysDesc *sys, const PairTile *tiles, const int *tile_sys,
                                    int64_t n_tiles, const double *nlogn, int *err, int tile_dim, cudaStream_t st) {
    int T = 0, fc = 0, nst = 0;
    const int smem = pairs_hist_config(bmax, &T, &fc, &nst);
    if (!smem || T != tile_dim) return cudaErrorInvalidValue;
    if (n_tiles <= 0) return cudaSuccess;
    cudaError_t e;
#define PG_LAUNCH(TT)                                                                                    \
    e = cudaFuncSetAttribute(pairs_hist_batch_kernel<TT>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                             smem);                                                                     \
    if (e != cudaSuccess) return e;                                                                     \
    pairs_hist_batch_kernel<TT><<<(unsigned)n_tiles, kThreads, smem, st>>>(sys, tiles, tile_sys, nlogn, \
                                                                            err, fc, nst, bmax);
    if (T == 4) { PG_LAUNCH(4) } else if (T == 2) { PG_LAUNCH(2) } else { PG_LAUNCH(1) }
#undef PG_LAUNCH
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
