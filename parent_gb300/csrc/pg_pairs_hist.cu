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

#include "pg_internal.h"

namespace pg {

namespace {

constexpr int kThreads = 512;
constexpr int kWarps = kThreads / 32;
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
__device__ __forceinline__ void red_add1(unsigned int *p) {
    asm volatile("red.shared.add.u32 [%0], 1;" ::"r"(smem_u32(p)) : "memory");
}

template <int T>
struct TileCfg {
    static constexpr int PPS = T * T;      // pair slots
    static constexpr int NSUB = 32 / PPS;  // frame sub-streams per warp
    static constexpr int NROW = 2 * T;     // staged bin rows
};

template <int T>
__global__ void __launch_bounds__(kThreads, 1)
pairs_hist_kernel(SysGeom geo, const uint8_t *__restrict__ bins, DofArrays dof,
                  const double *__restrict__ nlogn, const PairTile *__restrict__ tiles,
                  PairOut out, int *err, int fc, int bmax, double lnN) {
    using C = TileCfg<T>;
    constexpr int PPS = C::PPS, NSUB = C::NSUB, NROW = C::NROW;
    extern __shared__ __align__(128) unsigned char smem[];
    const int hist_words = bmax * bmax * PPS;
    unsigned int *hist = (unsigned int *)smem;
    const int fcs = fc + kStagePad;
    unsigned char *stage = smem + hist_bytes(bmax, PPS);  // [2][NROW][fcs], 128-B aligned
    uint64_t *mbar = (uint64_t *)(stage + 2 * NROW * fcs);
    __shared__ double red_snl[kWarps][PPS];
    __shared__ int red_occ[kWarps][PPS];
    __shared__ int s_abort;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const PairTile tile = tiles[blockIdx.x];
    const int F = geo.F;

    // staged row k: row DOF row0+k (k < T), column DOF col0+k-T (k >= T)
    auto row_dof = [&](int k) -> int {
        if (k < T) return k < tile.nrow ? tile.row0 + k : -1;
        return (k - T) < tile.ncol ? tile.col0 + (k - T) : -1;
    };

    for (int i = tid; i < hist_words; i += kThreads) hist[i] = 0u;
    if (tid == 0) {
        s_abort = 0;
        mbar_init(smem_u32(&mbar[0]), 1);
        mbar_init(smem_u32(&mbar[1]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    const int nchunks = (F + fc - 1) / fc;
    auto issue = [&](int chunk) {  // one thread
        const int st = chunk & 1;
        uint32_t bytes = 0;
        for (int k = 0; k < NROW; k++) bytes += row_dof(k) >= 0 ? (uint32_t)fc : 0u;
        const uint32_t bar = smem_u32(&mbar[st]);
        mbar_expect_tx(bar, bytes);
        for (int k = 0; k < NROW; k++) {
            const int g = row_dof(k);
            if (g < 0) continue;
            bulk_g2s(smem_u32(stage + (size_t)(st * NROW + k) * fcs),
                     bins + (int64_t)g * geo.ldb + (int64_t)chunk * fc, (uint32_t)fc, bar);
        }
    };
    if (tid == 0) {
        issue(0);
        if (nchunks > 1) issue(1);
    }

    // this lane's pair slot
    const int p = lane % PPS, sub = lane / PPS;
    const int pr = p / T, pc = p % T;
    const int gr = pr < tile.nrow ? tile.row0 + pr : -1;
    const int gc = pc < tile.ncol ? tile.col0 + pc : -1;
    const bool valid = gr >= 0 && gc >= 0 && gr < gc;
    const int Bc = valid ? dof.b2[gc] : 0;
    unsigned int *hp = hist + p;

    for (int chunk = 0; chunk < nchunks; chunk++) {
        const int st = chunk & 1;
        const bool ok = mbar_wait_bounded(smem_u32(&mbar[st]), (uint32_t)((chunk >> 1) & 1));
        if (__syncthreads_or(!ok)) {
            if (tid == 0) s_abort = 1;
            break;
        }
        const int fvalid = min(fc, F - chunk * fc);
        const unsigned char *rrow = stage + (size_t)(st * NROW + pr) * fcs;
        const unsigned char *crow = stage + (size_t)(st * NROW + T + pc) * fcs;
        if (valid) {
            for (int off = (warp * NSUB + sub) * 16; off < fvalid; off += kWarps * NSUB * 16) {
                const uint4 rv = *(const uint4 *)(rrow + off);
                const uint4 cv = *(const uint4 *)(crow + off);
                const uint32_t rw[4] = {rv.x, rv.y, rv.z, rv.w};
                const uint32_t cw[4] = {cv.x, cv.y, cv.z, cv.w};
                if (off + 16 <= fvalid) {
#pragma unroll
                    for (int q = 0; q < 4; q++) {
#pragma unroll
                        for (int b = 0; b < 4; b++) {
                            const uint32_t br = (rw[q] >> (8 * b)) & 0xffu;
                            const uint32_t bc = (cw[q] >> (8 * b)) & 0xffu;
                            red_add1(hp + (br * Bc + bc) * PPS);
                        }
                    }
                } else {  // ragged end of the trajectory
                    const int n = fvalid - off;
#pragma unroll
                    for (int k = 0; k < 16; k++) {
                        if (k < n) {
                            const uint32_t br = (rw[k >> 2] >> (8 * (k & 3))) & 0xffu;
                            const uint32_t bc = (cw[k >> 2] >> (8 * (k & 3))) & 0xffu;
                            red_add1(hp + (br * Bc + bc) * PPS);
                        }
                    }
                }
            }
        }
        __syncthreads();
        if (tid == 0 && chunk + 2 < nchunks) {
            // generic-proxy reads of this stage are done (barrier above);
            // order them before the async-proxy writes that refill it
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(chunk + 2);
        }
    }

    if (s_abort) {
        // a stage never completed: record it, drain what is still in flight
        // (bounded), and leave without writing results
        if (tid == 0) {
            atomicAdd(&err[ERR_TIMEOUT], 1);
            for (int c = 0; c < nchunks && c < 2; c++) {
                (void)mbar_wait_bounded(smem_u32(&mbar[c & 1]), 0u);
            }
        }
        return;
    }

    // ---- epilogue: per pair slot, sum n ln n and occupied bins
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
            int64_t *dst = out.counts + ((int64_t)blockIdx.x * PPS + ep) * out.counts_bmax * out.counts_bmax;
            for (int bin = ej; bin < nbin; bin += kThreads / PPS) dst[bin] = hist[bin * PPS + ep];
        }
    }
    // lanes l and l+PPS*k of a warp hold the same slot: fold them first
    for (int o = 16; o >= PPS; o >>= 1) {
        snl += __shfl_down_sync(0xffffffffu, snl, o);
        occ += __shfl_down_sync(0xffffffffu, occ, o);
    }
    if (lane < PPS) {
        red_snl[warp][lane] = snl;
        red_occ[warp][lane] = occ;
    }
    __syncthreads();
    if (tid < PPS && evalid) {
        double s = 0.0;
        int o = 0;
        for (int w = 0; w < kWarps; w++) {
            s += red_snl[w][tid];
            o += red_occ[w][tid];
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
size_t smem_bytes(int bmax, int fc) {
    return hist_bytes(bmax, TileCfg<T>::PPS) + 2 * TileCfg<T>::NROW * (size_t)(fc + kStagePad) + 16;
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

int pairs_hist_config(int bmax, int *tile_dim, int *chunk_frames) {
    const int fcs[3] = {4096, 2048, 1024};
    for (int T : {4, 2, 1}) {
        for (int fc : fcs) {
            size_t need = T == 4 ? smem_bytes<4>(bmax, fc) : (T == 2 ? smem_bytes<2>(bmax, fc) : smem_bytes<1>(bmax, fc));
            if (need + 4096 <= (size_t)kSmemMax) {  // the kernel's ~3.3 KB static smem fits in the rest
                *tile_dim = T;
                *chunk_frames = fc;
                return (int)need;
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
    int T = 0, fc = 0;
    const int smem = pairs_hist_config(bmax, &T, &fc);
    if (!smem || T != tile_dim) return cudaErrorInvalidValue;
    if (n_tiles <= 0) return cudaSuccess;
    const double lnN = log((double)g.F);
    cudaError_t e;
#define PG_LAUNCH(TT)                                                                              \
    e = cudaFuncSetAttribute(pairs_hist_kernel<TT>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                             smem);                                                               \
    if (e != cudaSuccess) return e;                                                               \
    pairs_hist_kernel<TT><<<(unsigned)n_tiles, kThreads, smem, st>>>(g, bins, dof, nlogn, tiles,  \
                                                                      out, err, fc, bmax, lnN);
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
