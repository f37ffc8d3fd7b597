// Pair kernel, tensor-core one-hot form, and the form autotuner.
//
// The 2D histograms of all DOF pairs are the blocks of one Gram matrix
//   C = X^T X,  X[f, (g, b)] = 1 if DOF g is in bin b at frame f, else 0,
// whose rows/columns run over the concatenated (DOF, bin) space (R = sum of
// the DOFs' 2D bin counts). Block (g1, g2) of C is the B(g1) x B(g2)
// histogram of the pair, so the counts PARENT.cpp fills frame by frame
// (e.g. :802-804) are entries of C.
//
// A pair of CTAs (a cluster of 2, one per SM) computes one 256 x 512 tile of
// C over all frames with tcgen05.mma.cta_group::2.kind::f8f6f4 (M=256, N=256,
// K=32, two accumulators sharing the A tile): each CTA builds its 128 rows of
// A and, of each 256-column MMA, 128 rows of B as E4M3 one-hot tiles (2.0 =
// 0x40, 0.0 = 0x00) in its shared memory from the uint8 bin rows, and holds
// its 128 rows x 512 columns of FP32 accumulators in tensor memory (4 x the
// count, exact below 2^24: frames below 2^22). Against one CTA per 128 x 512
// tile (still built as PAIR = false) each SM builds 384 instead of 640 rows
// per K-block. Warp-specialised: 15 builder warps load the tile's bin rows
// two 128-frame K-blocks ahead (a 4-buffer ring) and expand each K-block into
// a ring of one-hot stages, arriving on the stage's "full" mbarrier; in the
// pair's first CTA warp 15 waits on it, issues the block's eight MMAs and
// commits them to the stage's "empty" mbarrier in both CTAs, which the
// builders wait on before rebuilding the stage; in the second CTA warp 15
// relays the stage's completion to the first. No CTA-wide barrier inside the
// K loop.
//
// Epilogue: tcgen05.ld brings each row's counts to registers; every count n>0
// of a pair (g1 < g2) adds round(2^s n ln n) (an int64 table) and 1 to the
// pair's accumulators. Integer atomics keep the result independent of the
// order tiles finish in. A finalize kernel turns (sum n ln n, occupied bins)
// into S2D and MI exactly as the histogram kernel's epilogue does.
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "../../include/parent_gb300.h"
#include "pg_internal.h"
#include "pg_sync.cuh"

namespace pg {

namespace {

constexpr int kThreads = 512;          // 16 warps: 15 load bin rows and build one-hot tiles, warp 15 issues MMAs
constexpr int kBuilderWarps = 15;
constexpr int kBuilders = kBuilderWarps * 32;
constexpr int kLoaderWarp = 15;
constexpr int kM = 128, kN = 512;      // tile of C: two 128 x 256 accumulators share one A tile
constexpr int kNH = 256;               // N of one MMA
constexpr int kKB = 128;               // frames per K-block (bytes per row per stage)
constexpr int kAStage = kM * kKB;      // 16 KB
constexpr int kMaxRowDofs = 18, kMaxColDofs = 66;  // 2D bins >= 8
constexpr int kBinSlots = kMaxRowDofs + kMaxColDofs;
constexpr int kBinBufBytes = kBinSlots * kKB;      // one K-block of the tile's bin rows

// Shared-memory layout of one CTA. PAIR: a CTA pair computes a 256 x 512
// tile with tcgen05.mma.cta_group::2 (M = 256); each CTA builds its 128 A
// rows and half of the B rows (128 of each 256-column MMA), so a CTA's stage
// holds 128 + 256 rows instead of 128 + 512.
template <bool PAIR>
struct OhCfg {
    static constexpr int kBRows = PAIR ? 256 : 512;  // B rows built by this CTA
    static constexpr int kStages = PAIR ? 3 : 2;
    // Ring of K-block bin rows, loaded two blocks ahead. A builder starts
    // block kb only when the MMAs of block kb - kStages are done, i.e. when
    // every builder has finished that block, so the builders are at most
    // kStages - 1 blocks apart; the buffer refilled for block kb + 2 was last
    // read for block kb + 2 - kBinBufs, which must lie behind the slowest
    // builder (kb - kStages + 1).
    static constexpr int kBinBufs = kStages + 2;
    static constexpr int kBStage = kBRows * kKB;
    static constexpr int kStageBytes = kAStage + kBStage;
    // byte offsets inside the dynamic shared memory
    // full[kStages] | empty[kStages] | binfull[kBinBufs] | drained
    static constexpr int kOffBar = kStages * kStageBytes;
    static constexpr int kNumBars = 2 * kStages + kBinBufs + 1;
    static constexpr int kOffTmem = kOffBar + kNumBars * 8;
    static constexpr int kOffPsSnl = (kOffTmem + 16 + 15) / 16 * 16;
    static constexpr int kOffPsOcc = kOffPsSnl + kMaxRowDofs * kMaxColDofs * 8;
    static constexpr int kOffBins = (kOffPsOcc + kMaxRowDofs * kMaxColDofs * 4 + 127) / 128 * 128;
    static constexpr int kSmemBytes = kOffBins + kBinBufs * kBinBufBytes;
    static_assert(kSmemBytes <= 227 * 1024, "one-hot kernel shared memory");
};
constexpr long long kWaitCycles = 4000000000LL;
// Frames per accumulation chunk: the FP32 accumulators hold 4 x the count of
// one chunk (exact below 2^24); at the end of every chunk but the last, the
// counts are moved into INT32 totals in global memory (one 128 x 512 slot per
// SM: one CTA of this kernel per SM at a time) and the accumulators restart.
constexpr int kChunkFrames = 1 << 20;
constexpr int kChunkKB = kChunkFrames / 128;   // K-blocks per chunk
constexpr int kDrainWarps = 4;                 // warps 0..3, one per TMEM lane quarter
constexpr size_t kDrainSlotWords = 128 * 512;
// Fixed-point scale of n ln n: the largest power of two 2^s (s <= 44) with

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
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
// arrive (release at CTA scope): the thread's earlier shared-memory writes
// are visible to whoever completes the phase's wait
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (clock64() - t0 > kWaitCycles) return false;
    }
    return true;
}

// Shared-memory matrix descriptor, no swizzle, K-major: 8-row x 16-byte core
// matrices stored contiguously (128 B); lbo = byte distance between the two
// core matrices of one K=32 step, sbo = byte distance between 8-row groups.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version for sm_100-class tensor cores
    return d;                // base offset 0, layout type 0 = no swizzle
}

// Instruction descriptor: D = F32, A = B = E4M3, both K-major, N = 256, M = 128.
constexpr uint32_t kIdesc = (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t)(kNH >> 3) << 17) |
                            ((uint32_t)(kM >> 4) << 24);
constexpr uint32_t kIdesc2 = (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t)(kNH >> 3) << 17) |
                             ((uint32_t)((2 * kM) >> 4) << 24);  // M = 256 over a CTA pair

// E4M3 one-hot of 4 bins against a bin replicated in t4: 0x40 (2.0) in every
// byte where w equals t4, 0x00 elsewhere (bins below 128). x = w ^ t4 has a
// zero byte exactly where they match and every byte below 128, so adding
// 0x7F to each byte sets its bit 7 exactly when it is nonzero, without a
// carry into the next byte; the complement's bit 7, shifted down by one, is
// 2.0 in E4M3. Four integer operations per four frames.
__device__ __forceinline__ uint32_t onehot4(uint32_t w, uint32_t t4) {
    const uint32_t a = (w ^ t4) + 0x7F7F7F7Fu;
    return (~a & 0x80808080u) >> 1;
}
// The same for bins below 64: every byte of w ^ t4 is below 64, so adding
// 0x3F sets its bit 6 exactly when it is nonzero (no carry: 63 + 63 < 128),
// and the complement's bit 6 is 2.0 in E4M3 with no shift. Three integer
// operations per four frames.
__device__ __forceinline__ uint32_t onehot4_low(uint32_t w, uint32_t t4) {
    const uint32_t a = (w ^ t4) + 0x3F3F3F3Fu;
    return ~a & 0x40404040u;
}

__device__ __forceinline__ void mma_f8(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
        "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}
// CTA pair: A and B halves from both CTAs' shared memory at the same offsets,
// the accumulator rows of each CTA in its own tensor memory
__device__ __forceinline__ void mma_f8_pair(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::2.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
        "l"(adesc), "l"(bdesc), "r"(kIdesc2), "r"(acc)
        : "memory");
}
// completion of the pair's MMAs, signalled on the barrier at this offset in both CTAs
__device__ __forceinline__ void mma_commit_pair(uint32_t bar) {
    asm volatile(
        "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(bar),
        "h"((unsigned short)3)
        : "memory");
}
__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
// shared::cluster address of the same variable in CTA `rank` of the cluster
__device__ __forceinline__ uint32_t map_to_rank(uint32_t saddr, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(saddr), "r"(rank));
    return r;
}
// arrive (release at cluster scope) on a barrier given by its cluster address
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t caddr) {
    asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(caddr) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait_cluster(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool mbar_wait_cluster_bounded(uint32_t bar, uint32_t parity) {
    const long long t0 = clock64();
    while (!mbar_try_wait_cluster(bar, parity)) {
        if (clock64() - t0 > kWaitCycles) return false;
    }
    return true;
}
__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// A tile: row tile (x128, or x256 for a CTA pair) and column tile (x512) of
// the C of system `sys` of the launch.
struct TcTile {
    int mt, nt, sys, pad;
};

// One system of a launch, as the kernel reads it (a single-system launch
// has one). rowinfo: (dof << 8) | bin for each row of the system's C; nfix:
// its fixed-point n ln n table; acc_snl/acc_occ: its D x D pair accumulators.
struct OhSys {
    const uint8_t *bins;
    int64_t ldb;
    const uint32_t *rowinfo;
    const int64_t *nfix;
    unsigned long long *acc_snl;
    unsigned int *acc_occ;
    uint32_t *drain;  // INT32 totals of trajectories longer than a chunk: [slot][512 cols][128 rows]
    int F, R, D, drain_slots;
};

// Per (row, chunk) item of the one-hot build, fixed for the whole K loop.
struct Item {
    uint32_t soff;       // offset of the item's 16 bin bytes inside a bin buffer
    uint32_t t4;         // the row's bin replicated in 4 bytes
    uint32_t dst;        // byte offset inside a stage
    int c16;             // first frame of the chunk inside a K-block
    int valid;
};

// One CTA (PAIR = false) computes the 128 x 512 tile (mt, nt) of C; a CTA
// pair (PAIR, cluster of 2) the 256 x 512 tile (mt, nt), CTA `rank` owning
// rows 256 mt + 128 rank .. +127 and, of each 256-column MMA, B columns
// 128 rank .. +127. Only the pair's rank 0 issues MMAs. Builder warps arrive
// on their own CTA's "full" barrier (CTA scope); in rank 1, warp 15 waits for
// that and relays it with one cluster-scope arrival on rank 0's "full"
// barrier (one cluster-scope release per stage instead of one per builder
// warp, whose memory barriers stalled the builders). The commit of a stage's
// MMAs arrives on the "empty" barrier of both CTAs.
// LOW: every 2D bin count of the launch is at most 64 (onehot4_low).
template <bool PAIR, bool LOW>
__global__ void __launch_bounds__(kThreads, 1)
onehot_kernel(const OhSys *__restrict__ systems, const TcTile *__restrict__ tiles, int *err) {
    using C = OhCfg<PAIR>;
    constexpr int kStages = C::kStages, kStageBytes = C::kStageBytes, kBRows = C::kBRows;
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *stages = smem;  // kStages x (A | B), 1024-B aligned
    uint64_t *full = (uint64_t *)(smem + C::kOffBar);  // stage built (one arrival per builder warp, both CTAs)
    uint64_t *empty = full + kStages;                  // stage's MMAs done (tcgen05.commit)
    uint64_t *binfull = empty + kStages;               // K-block bin rows stored (one arrival per builder warp)
    uint64_t *drained = binfull + C::kBinBufs;         // a chunk's accumulators moved to the INT32 totals
    uint32_t *tmem_slot = (uint32_t *)(smem + C::kOffTmem);
    unsigned long long *ps_snl = (unsigned long long *)(smem + C::kOffPsSnl);  // [kMaxRowDofs][kMaxColDofs]
    unsigned int *ps_occ = (unsigned int *)(smem + C::kOffPsOcc);
    __shared__ int s_r0dof, s_c0dof, s_b0dof;
    __shared__ int s_cdof[kN];  // DOF of each column of the tile (-1 past R)
    __shared__ volatile int s_abort;
    __shared__ int s_mma_issued;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t rank = PAIR ? cluster_rank() : 0u;
    const TcTile tile = tiles[PAIR ? blockIdx.x >> 1 : blockIdx.x];
    const OhSys sy = systems[tile.sys];  // both CTAs of a pair read the same tile, so the same system
    const uint8_t *__restrict__ bins = sy.bins;
    const int64_t ldb = sy.ldb;
    const uint32_t *__restrict__ rowinfo = sy.rowinfo;
    const int64_t *__restrict__ nlogn_fix = sy.nfix;
    unsigned long long *__restrict__ acc_snl = sy.acc_snl;
    unsigned int *__restrict__ acc_occ = sy.acc_occ;
    const int F = sy.F, R = sy.R, D = sy.D;
    const int r0 = PAIR ? tile.mt * 2 * kM + (int)rank * kM : tile.mt * kM;  // this CTA's A rows
    const int c0 = tile.nt * kN;
    const int b0 = PAIR ? c0 + (int)rank * (kNH / 2) : c0;  // first C column of this CTA's B rows

    if (warp == 0) {  // all 512 TMEM columns: two 128 x 256 FP32 accumulators
        if (PAIR) {
            asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                             smem_u32(tmem_slot)),
                         "r"(512)
                         : "memory");
            asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
        } else {
            asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                             smem_u32(tmem_slot)),
                         "r"(512)
                         : "memory");
            asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        }
    }
    for (int c = tid; c < kN; c += kThreads) s_cdof[c] = c0 + c < R ? (int)(rowinfo[c0 + c] >> 8) : -1;
    if (tid == 0) {
        for (int k = 0; k < kStages; k++) {
            mbar_init(smem_u32(&full[k]), (PAIR && rank == 0) ? kBuilderWarps + 1 : kBuilderWarps);
            mbar_init(smem_u32(&empty[k]), 1);
        }
        for (int k = 0; k < C::kBinBufs; k++) mbar_init(smem_u32(&binfull[k]), kBuilderWarps);
        // the drain warps of both CTAs of a pair arrive on the first CTA's barrier
        mbar_init(smem_u32(drained), (PAIR ? 2 : 1) * kDrainWarps);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_r0dof = (int)(rowinfo[r0 < R ? r0 : R - 1] >> 8);
        s_c0dof = (int)(rowinfo[c0 < R ? c0 : R - 1] >> 8);
        s_b0dof = (int)(rowinfo[b0 < R ? b0 : R - 1] >> 8);
        s_abort = 0;
        s_mma_issued = 0;
    }
    for (int i = tid; i < kMaxRowDofs * kMaxColDofs; i += kThreads) {
        ps_snl[i] = 0ull;
        ps_occ[i] = 0u;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    if (PAIR) cluster_sync_all();  // both CTAs' barriers exist before any remote arrival
    else __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    const int rdof0 = s_r0dof, bdof0 = s_b0dof;
    const int rlast = (int)(rowinfo[min(r0 + kM, R) - 1] >> 8);
    const int blast = (int)(rowinfo[min(b0 + (PAIR ? kN - kNH / 2 : kN), R) - 1] >> 8);  // last B row's DOF
    const int nkb = (F + kKB - 1) / kKB;
    unsigned char *binbuf = smem + C::kOffBins;  // [C::kBinBufs][kBinSlots][kKB]
    // INT32 totals of this SM's slot (trajectories longer than one chunk)
    const bool chunked = nkb > kChunkKB;
    uint32_t smid = 0;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
    uint32_t *totals = (chunked && sy.drain && (int)smid < sy.drain_slots) ? sy.drain + (size_t)smid * kDrainSlotWords
                                                                          : nullptr;
    if (chunked && !totals) {  // no drain area for this SM: report, count nothing
        if (tid == 0) atomicAdd(&err[ERR_TIMEOUT], 1);
    }

    if (warp == kLoaderWarp) {
        // ------------------------------------------------------- MMA issuer
        if (!PAIR || rank == 0) {
            const uint32_t sbase = smem_u32(stages);
            int kb = 0;
            for (; kb < nkb; kb++) {
                const int s = kb % kStages;
                int ok = 1;
                if (lane == 0)
                    ok = (PAIR ? mbar_wait_cluster_bounded(smem_u32(&full[s]), (uint32_t)((kb / kStages) & 1))
                               : mbar_wait_bounded(smem_u32(&full[s]), (uint32_t)((kb / kStages) & 1)))
                             ? 1
                             : 0;
                ok = __shfl_sync(0xffffffffu, ok, 0);
                if (ok && chunked && kb % kChunkKB == 0) {
                    // the previous chunk's accumulators are in the INT32 totals
                    // (both CTAs of a pair) before this chunk's MMAs restart them
                    if (lane == 0)
                        ok = (PAIR ? mbar_wait_cluster_bounded(smem_u32(drained), (uint32_t)((kb / kChunkKB - 1) & 1))
                                   : mbar_wait_bounded(smem_u32(drained), (uint32_t)((kb / kChunkKB - 1) & 1)))
                                 ? 1
                                 : 0;
                    ok = __shfl_sync(0xffffffffu, ok, 0);
                }
                if (!ok || s_abort || (chunked && !totals)) {
                    if (lane == 0) s_abort = 1;
                    break;
                }
                const int kc = kb % kChunkKB;  // K-block inside its chunk: 0 restarts the accumulators
                if (lane == 0) {
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t a0 = sbase + s * kStageBytes, bb0 = a0 + kAStage;
#pragma unroll
                    for (int kk = 0; kk < kKB / 32; kk++) {
#pragma unroll
                        for (int h = 0; h < kN / kNH; h++) {  // B rows of MMA h start kBRows/2 rows further
                            const uint64_t ad = smem_desc(a0 + kk * 256, 128, 1024);
                            const uint64_t bd = smem_desc(bb0 + h * (kBRows / 2 / 8) * 1024 + kk * 256, 128, 1024);
                            if (PAIR) mma_f8_pair(tmem + h * kNH, ad, bd, (kc | kk) != 0);
                            else mma_f8(tmem + h * kNH, ad, bd, (kc | kk) != 0);
                        }
                    }
                    if (PAIR) mma_commit_pair(smem_u32(&empty[s]));
                    else mma_commit(smem_u32(&empty[s]));
                }
                __syncwarp();
            }
            if (lane == 0) s_mma_issued = kb;
        } else if (PAIR) {
            // ------------------------------------------ rank 1: stage relay
            const uint32_t full_c0 = map_to_rank(smem_u32(&full[0]), 0u);
            for (int kb = 0; kb < nkb; kb++) {
                const int s = kb % kStages;
                int ok = 1;
                if (lane == 0) ok = mbar_wait_bounded(smem_u32(&full[s]), (uint32_t)((kb / kStages) & 1)) ? 1 : 0;
                ok = __shfl_sync(0xffffffffu, ok, 0);
                if (!ok || s_abort) {
                    if (lane == 0) s_abort = 1;
                    break;
                }
                if (lane == 0) mbar_arrive_cluster(full_c0 + (uint32_t)s * 8u);
                __syncwarp();
            }
        }
    } else {
        // ----------------------------------------------------------- builders
        // items: A rows 0..127 (1024 items), then this CTA's B rows; item i ->
        // (row group g, chunk c, row-in-group rr) with rr fastest, so 8
        // consecutive threads store one contiguous 128-B core matrix
        constexpr int kItems = (kM + kBRows) * (kKB / 16);
        constexpr int kItemsPerThread = (kItems + kBuilders - 1) / kBuilders;
        Item it[kItemsPerThread];
#pragma unroll
        for (int j = 0; j < kItemsPerThread; j++) {
            const int i = tid + j * kBuilders;
            const bool inr = i < kItems;
            const bool isA = i < kM * 8;
            const int ii = isA ? i : i - kM * 8;
            const int rr = ii & 7, c = (ii >> 3) & 7, g = ii >> 6;
            const int lrow = g * 8 + rr;  // row inside the A or B part of the stage
            // PAIR: B row lrow is column 256 (lrow / 128) + 128 rank + lrow % 128 of the tile
            const int row = isA ? r0 + lrow
                                : (PAIR ? c0 + (lrow / (kNH / 2)) * kNH + (int)rank * (kNH / 2) + lrow % (kNH / 2)
                                        : c0 + lrow);
            it[j].dst = (isA ? 0u : (uint32_t)kAStage) + (uint32_t)((g * 8 + c) * 128 + rr * 16);
            it[j].c16 = c * 16;
            it[j].valid = inr && row < R;
            const uint32_t info = it[j].valid ? rowinfo[row] : 0u;
            const int d = (int)(info >> 8);
            const int slot = isA ? d - rdof0 : kMaxRowDofs + d - bdof0;
            it[j].soff = it[j].valid ? (uint32_t)(slot * kKB + c * 16) : 0u;
            it[j].t4 = (info & 0xffu) * 0x01010101u;
            if (!inr) it[j].dst = 0xffffffffu;  // no item
        }
        // Bin rows of K-block j go to ring buffer j % kBinBufs: slot k <
        // kMaxRowDofs holds DOF rdof0 + k (rows of A), slot kMaxRowDofs + k
        // holds DOF bdof0 + k (rows of B). Every builder thread loads its share
        // of block kb + 2 into registers before building block kb and stores
        // it after; the ring is long enough that no builder still reads the
        // buffer it refills (see OhCfg::kBinBufs).
        constexpr int kLoads = kBinSlots * (kKB / 16);  // 16-byte chunks per K-block
        constexpr int kLoadsPerThread = (kLoads + kBuilders - 1) / kBuilders;
        auto load_chunk = [&](int L, int j, uint4 &v) -> bool {
            const int slot = L >> 3, c = L & 7;
            const int d = slot < kMaxRowDofs ? rdof0 + slot : bdof0 + slot - kMaxRowDofs;
            const bool ok = L < kLoads && (slot < kMaxRowDofs ? d <= rlast : d <= blast);
            if (ok) v = __ldg((const uint4 *)(bins + (int64_t)d * ldb + (int64_t)j * kKB + c * 16));
            return ok;
        };
        auto store_block = [&](int j, const uint4 *v, const bool *ok) {
            unsigned char *dst = binbuf + (j % C::kBinBufs) * kBinBufBytes;
#pragma unroll
            for (int q = 0; q < kLoadsPerThread; q++) {
                const int L = tid + q * kBuilders;
                if (ok[q]) *(uint4 *)(dst + (L >> 3) * kKB + (L & 7) * 16) = v[q];
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&binfull[j % C::kBinBufs]));
        };
        for (int j = 0; j < 2 && j < nkb; j++) {
            uint4 v[kLoadsPerThread];
            bool ok[kLoadsPerThread];
#pragma unroll
            for (int q = 0; q < kLoadsPerThread; q++) ok[q] = load_chunk(tid + q * kBuilders, j, v[q]);
            store_block(j, v, ok);
        }
        for (int kb = 0; kb < nkb; kb++) {
            const int s = kb % kStages;
            if (s_abort) break;
            uint4 pf[kLoadsPerThread];
            bool pv[kLoadsPerThread];
#pragma unroll
            for (int q = 0; q < kLoadsPerThread; q++)
                pv[q] = kb + 2 < nkb ? load_chunk(tid + q * kBuilders, kb + 2, pf[q]) : false;
            if (!mbar_wait_bounded(smem_u32(&binfull[kb % C::kBinBufs]), (uint32_t)((kb / C::kBinBufs) & 1)) ||
                (kb >= kStages &&
                 !mbar_wait_bounded(smem_u32(&empty[s]), (uint32_t)((kb / kStages - 1) & 1)))) {
                s_abort = 1;
                break;
            }
            const int nvalid = F - kb * kKB;  // frames of this block that exist (>= 1)
            const unsigned char *bb = binbuf + (kb % C::kBinBufs) * kBinBufBytes;
            unsigned char *st = stages + s * kStageBytes;
#pragma unroll
            for (int j = 0; j < kItemsPerThread; j++) {
                // every thread has an item in all but the last round
                if (j == kItemsPerThread - 1 && it[j].dst == 0xffffffffu) continue;
                uint4 o;
                {
                    // a row past the tile's end reads chunk 0 (soff 0) and is
                    // masked to zero: no branch per item
                    const uint4 w = *(const uint4 *)(bb + it[j].soff);
                    if (LOW) {
                        o.x = onehot4_low(w.x, it[j].t4);
                        o.y = onehot4_low(w.y, it[j].t4);
                        o.z = onehot4_low(w.z, it[j].t4);
                        o.w = onehot4_low(w.w, it[j].t4);
                    } else {
                        o.x = onehot4(w.x, it[j].t4);
                        o.y = onehot4(w.y, it[j].t4);
                        o.z = onehot4(w.z, it[j].t4);
                        o.w = onehot4(w.w, it[j].t4);
                    }
                    const uint32_t vm = 0u - (uint32_t)it[j].valid;
                    o.x &= vm; o.y &= vm; o.z &= vm; o.w &= vm;
                    if (nvalid < kKB) {  // last block: frames past F are not data
                        const int v = nvalid - it[j].c16;
                        uint32_t m[4];
#pragma unroll
                        for (int q = 0; q < 4; q++) {
                            const int bq = v - 4 * q;  // valid bytes in word q
                            m[q] = bq >= 4 ? 0xffffffffu : (bq <= 0 ? 0u : (0xffffffffu >> (8 * (4 - bq))));
                        }
                        o.x &= m[0]; o.y &= m[1]; o.z &= m[2]; o.w &= m[3];
                    }
                }
                *(uint4 *)(st + it[j].dst) = o;
            }
            // generic writes of the stage before the tensor core reads it
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&full[s]));
            if (kb + 2 < nkb) store_block(kb + 2, pf, pv);
            if (chunked && warp < kDrainWarps && (kb + 1) % kChunkKB == 0 && kb + 1 < nkb) {
                // end of a chunk: once its MMAs are done (the commit of this
                // block), move this warp's TMEM lane quarter into the totals
                int ok = 0;  // lane 0 waits, the warp follows it (the TMEM loads below are warp-wide)
                if (lane == 0)
                    ok = totals && mbar_wait_bounded(smem_u32(&empty[s]), (uint32_t)((kb / kStages) & 1)) ? 1 : 0;
                if (!__shfl_sync(0xffffffffu, ok, 0)) {
                    s_abort = 1;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const bool first = kb + 1 == kChunkKB;
                const int row = 32 * warp + lane;
                for (int ch = 0; ch < kN / 16; ch++) {
                    uint32_t v[16];
                    const uint32_t taddr = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(ch * 16);
                    asm volatile(
                        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                          "=r"(v[15])
                        : "r"(taddr));
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                    for (int q = 0; q < 16; q++) {
                        const uint32_t n = __float2uint_rn(__uint_as_float(v[q])) >> 2;  // 2.0 x 2.0 per frame
                        uint32_t *t = totals + (size_t)(ch * 16 + q) * 128 + row;
                        *t = first ? n : *t + n;
                    }
                }
                asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                __threadfence_block();
                __syncwarp();
                if (lane == 0) {
                    if (PAIR && rank != 0) mbar_arrive_cluster(map_to_rank(smem_u32(drained), 0u));
                    else mbar_arrive(smem_u32(drained));
                }
            }
        }
    }
    __syncthreads();

    bool aborted = s_abort != 0;
    if (!aborted && nkb > 0) {  // the commit of the final block covers every earlier MMA
        const int last = nkb - 1;
        if (!mbar_wait_bounded(smem_u32(&empty[last % kStages]), (uint32_t)((last / kStages) & 1))) s_abort = 1;
        aborted = __syncthreads_or(s_abort != 0);
    }
    if (aborted) {
        // a wait ran out: record it, let issued MMAs finish (bounded), free
        // the tensor memory and leave
        if (tid == 0) {
            atomicAdd(&err[ERR_TIMEOUT], 1);
            const int nm = s_mma_issued;
            for (int k = nm > kStages ? nm - kStages : 0; k < nm; k++)
                (void)mbar_wait_bounded(smem_u32(&empty[k % kStages]), (uint32_t)((k / kStages) & 1));
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        if (PAIR) cluster_sync_all();  // neither CTA leaves while the pair's MMAs may read its stages
        else __syncthreads();
        if (warp == 0) {
            if (PAIR)
                asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
            else
                asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
        }
        return;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

    // ---- epilogue: warp w reads TMEM lanes 32(w%4).. (tile rows) and
    // columns (w/4)*128 .. +127 (16 warps cover the 512 columns)
    const int row = 32 * (warp & 3) + lane;
    const int grow = r0 + row;
    const uint32_t rinfo = grow < R ? rowinfo[grow] : 0xffffffffu;
    const int rdof = grow < R ? (int)(rinfo >> 8) : -1;
    const int cbase = (warp >> 2) * 128;
    int cur = -1;
    unsigned long long snl = 0ull;
    unsigned int occ = 0u;
    auto flush = [&](int cdof) {
        if (cur >= 0 && (snl || occ)) {
            const int ri = rdof - s_r0dof, ci = cur - s_c0dof;
            atomicAdd(&ps_snl[ri * kMaxColDofs + ci], snl);
            atomicAdd(&ps_occ[ri * kMaxColDofs + ci], occ);
        }
        cur = cdof;
        snl = 0ull;
        occ = 0u;
    };
    for (int ch = 0; ch < 8; ch++) {
        uint32_t v[16];
        const uint32_t taddr = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(cbase + ch * 16);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
              "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (rdof < 0) continue;
#pragma unroll
        for (int q = 0; q < 16; q++) {
            const int cdof = s_cdof[cbase + ch * 16 + q];
            if (cdof < 0) break;        // past the last row of C
            if (cdof <= rdof) continue;  // only pairs g1 < g2
            if (cdof != cur) flush(cdof);
            unsigned int n = (unsigned int)__float2uint_rn(__uint_as_float(v[q])) >> 2;  // 2.0 x 2.0 per frame
            if (chunked) n += totals[(size_t)(cbase + ch * 16 + q) * 128 + row];  // earlier chunks
            if (n) {
                snl += (unsigned long long)__ldg(nlogn_fix + n);
                occ++;
            }
        }
    }
    flush(-1);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    if (PAIR) cluster_sync_all();
    else __syncthreads();
    if (warp == 0) {
        if (PAIR)
            asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
        else
            asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
    }
    // tile partials -> per-pair accumulators (integer adds: order-independent)
    for (int i = tid; i < kMaxRowDofs * kMaxColDofs; i += kThreads) {
        const unsigned int o = ps_occ[i];
        if (!o) continue;
        const int g1 = s_r0dof + i / kMaxColDofs, g2 = s_c0dof + i % kMaxColDofs;
        const int64_t pi = (int64_t)g1 * D + g2;
        atomicAdd(&acc_snl[pi], ps_snl[i]);
        atomicAdd(&acc_occ[pi], o);
    }
}

// S2D and MI of every pair from the accumulators (the histogram kernel's
// epilogue formula): S = ln N + A_i + A_j - (1/N) sum n ln n + (occ-1)/(2N).
// One system per blockIdx.z.
struct OhFin {
    SysGeom geo;
    DofArrays dof;
    const unsigned long long *acc_snl;
    const unsigned int *acc_occ;
    PairOut out;
    double lnN, fix;
};

__global__ void onehot_finalize(const OhFin *__restrict__ fins) {
    const OhFin &fn = fins[blockIdx.z];
    const SysGeom &geo = fn.geo;
    const DofArrays &dof = fn.dof;
    const unsigned long long *acc_snl = fn.acc_snl;
    const unsigned int *acc_occ = fn.acc_occ;
    const PairOut &out = fn.out;
    const double lnN = fn.lnN, fix = fn.fix;
    const int D = geo.D;
    const int g2 = blockIdx.x * blockDim.x + threadIdx.x;
    const int g1 = blockIdx.y;
    if (g1 >= D || g2 >= D || g2 <= g1) return;
    const int64_t pi = (int64_t)g1 * D + g2;
    const double N = (double)geo.F;
    const double s = (double)acc_snl[pi] / fix;
    const unsigned int o = acc_occ[pi];
    const double S2 = lnN + dof.acon[g1] + dof.acon[g2] - s / N + (o - 1.0) / (2.0 * N);
    if (out.par) out.par[par_pair_index(out.L, geo.nb, geo.na, geo.nd, g1, g2)] = S2;
    if (out.mi) {
        const double mi = dof.s1[g1] + dof.s1[g2] - S2;
        out.mi[(int64_t)g1 * D + g2] = mi;
        out.mi[(int64_t)g2 * D + g1] = mi;
    }
}




__global__ void nsmid_kernel(int *out) {
    uint32_t n;
    asm volatile("mov.u32 %0, %%nsmid;" : "=r"(n));
    *out = (int)n;
}

}  // namespace

// Number of SM ids of the current device (%nsmid: the ids need not be
// contiguous, so this bounds them), looked up once per device: the INT32
// totals of chunked one-hot runs have one slot per id.
static int device_nsmid() {
    static int cache[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && cache[dev] > 0) return cache[dev];
    int n = 0, *d = nullptr;
    if (cudaMalloc(&d, sizeof(int)) == cudaSuccess) {
        nsmid_kernel<<<1, 1>>>(d);
        if (cudaMemcpy(&n, d, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) n = 0;
        cudaFree(d);
    }
    cudaGetLastError();
    if (n <= 0) cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (dev >= 0 && dev < 64) cache[dev] = n;
    return n;
}

// Host-side geometry of one system: rows of C, its tile list and the
// scratch layout of a single-system launch.
struct OnehotPlan {
    int64_t R = 0, n_tiles = 0;
    size_t off_rowstart = 0, off_rowinfo = 0, off_tiles = 0, off_fix = 0, off_snl = 0, off_occ = 0, off_sys = 0,
           off_fin = 0, off_drain = 0, total = 0;
    int drain_slots = 0;
};

// INT32 totals: one slot per SM id when the trajectory is longer than a chunk
static int drain_slots_for(int F) { return F > kChunkFrames ? device_nsmid() : 0; }

static int bins_of(const SysGeom &g, int gd) { return g.bins[3 + dof_type(gd, g.nb, g.na)]; }
static size_t al256(size_t x) { return (x + 255) / 256 * 256; }

// rowinfo of every row of C: (dof << 8) | bin
static std::vector<uint32_t> rowinfo_of(const SysGeom &g) {
    std::vector<uint32_t> ri;
    for (int d = 0; d < g.D; d++)
        for (int b = 0; b < bins_of(g, d); b++) ri.push_back(((uint32_t)d << 8) | (uint32_t)b);
    return ri;
}

// pair: tiles of 256 rows (a CTA pair each), else 128; tiles tagged `sys`
static OnehotPlan plan(const SysGeom &g, std::vector<TcTile> *tiles, bool pair = false, int sys = 0) {
    OnehotPlan p;
    std::vector<int64_t> rs((size_t)g.D + 1, 0);
    for (int d = 0; d < g.D; d++) rs[d + 1] = rs[d] + bins_of(g, d);
    p.R = rs[g.D];
    const int64_t tm = pair ? 2 * kM : kM;
    const int64_t mts = (p.R + tm - 1) / tm, nts = (p.R + kN - 1) / kN;
    auto dof_at = [&](int64_t row) {  // last d with rs[d] <= row
        return (int)(std::upper_bound(rs.begin(), rs.end(), row) - rs.begin()) - 1;
    };
    int64_t cnt = 0;
    for (int64_t mt = 0; mt < mts; mt++) {
        const int rdof0 = dof_at(mt * tm);
        for (int64_t nt = 0; nt < nts; nt++) {
            const int64_t cend = std::min(p.R, (nt + 1) * kN) - 1;
            if (dof_at(cend) <= rdof0) continue;  // no pair g1 < g2 in this tile
            if (tiles) tiles->push_back(TcTile{(int)mt, (int)nt, sys, 0});
            cnt++;
        }
    }
    p.n_tiles = cnt;
    p.off_rowstart = 0;
    p.off_rowinfo = al256(p.off_rowstart + sizeof(int64_t) * (g.D + 1));
    p.off_tiles = al256(p.off_rowinfo + sizeof(uint32_t) * (size_t)p.R);
    p.off_fix = al256(p.off_tiles + sizeof(TcTile) * (size_t)cnt);
    p.off_snl = al256(p.off_fix + sizeof(int64_t) * ((size_t)g.F + 1));
    p.off_occ = al256(p.off_snl + sizeof(unsigned long long) * (size_t)g.D * g.D);
    p.off_sys = al256(p.off_occ + sizeof(unsigned int) * (size_t)g.D * g.D);
    p.off_fin = al256(p.off_sys + sizeof(OhSys));
    p.off_drain = al256(p.off_fin + sizeof(OhFin));
    p.drain_slots = drain_slots_for(g.F);
    p.total = al256(p.off_drain + sizeof(uint32_t) * kDrainSlotWords * (size_t)p.drain_slots);
    return p;
}

bool pairs_onehot_supported(const SysGeom &g) {
    for (int t = 0; t < 3; t++)
        if (g.bins[3 + t] < 8 || g.bins[3 + t] > 127) return false;  // per-tile DOF tables sized for >= 8 bins;
                                                                     // bin bytes below 128 for the one-hot build
    return g.F >= 1;  // longer than one chunk (2^20 frames): INT32 totals across chunks
}

size_t pairs_onehot_scratch_bytes(const SysGeom &g) { return plan(g, nullptr).total; }

// CTA pairs (tcgen05.mma.cta_group::2) unless PG_ONEHOT_PAIR=0 (one CTA per
// 128 x 512 tile). Measured at 2,994 DOFs x 100k frames, 10 bins: 38.2 ms
// against 54.7 ms.
static bool use_pairs() {
    const char *e = getenv("PG_ONEHOT_PAIR");
    return !(e && atoi(e) == 0);
}

// The pair kernel over a tile list (each tile names its system) and the
// finalize kernel over n_fin systems (largest D max_D).
// low: every 2D bin count of the launch's systems is at most 64.
static cudaError_t launch_tiles(const OhSys *d_sys, const TcTile *d_tiles, int64_t n_tiles, bool pair, bool low,
                                const OhFin *d_fin, int n_fin, int max_D, int *err, cudaStream_t st) {
    cudaError_t e;
    if (n_tiles > 0) {
        if (pair) {
            const size_t smem = (size_t)OhCfg<true>::kSmemBytes;
            auto kern = low ? onehot_kernel<true, true> : onehot_kernel<true, false>;
            if ((e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)))
                return e;
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3((unsigned)(2 * n_tiles));
            cfg.blockDim = dim3(kThreads);
            cfg.dynamicSmemBytes = smem;
            cfg.stream = st;
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = 2;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            if ((e = cudaLaunchKernelEx(&cfg, kern, d_sys, d_tiles, err))) return e;
        } else {
            const size_t smem = (size_t)OhCfg<false>::kSmemBytes;
            auto kern = low ? onehot_kernel<false, true> : onehot_kernel<false, false>;
            if ((e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem))) return e;
            kern<<<(unsigned)n_tiles, kThreads, smem, st>>>(d_sys, d_tiles, err);
        }
    }
    dim3 fg((max_D + 255) / 256, max_D, n_fin);
    onehot_finalize<<<fg, 256, 0, st>>>(d_fin);
    return cudaGetLastError();
}

// Single-system launch in two parts: the set-up (uploads of the row table,
// tiles and descriptors, which the host must wait for, and the n ln n table)
// and the run (zeroed accumulators, pair kernel, finalize), which can be
// repeated on the same inputs.
cudaError_t onehot_setup(const SysGeom &g, const uint8_t *bins, const DofArrays &dof, PairOut out, cudaStream_t st,
                         void *scratch, size_t scratch_bytes, OnehotRun *run) {
    if (!pairs_onehot_supported(g)) return cudaErrorInvalidValue;
    const bool pair = use_pairs();
    std::vector<TcTile> tiles;
    const OnehotPlan p = plan(g, &tiles, pair);
    if (scratch_bytes < p.total) return cudaErrorInvalidValue;
    char *base = (char *)scratch;
    const std::vector<uint32_t> ri = rowinfo_of(g);
    uint32_t *d_ri = (uint32_t *)(base + p.off_rowinfo);
    TcTile *d_tiles = (TcTile *)(base + p.off_tiles);
    int64_t *d_fix = (int64_t *)(base + p.off_fix);
    unsigned long long *d_snl = (unsigned long long *)(base + p.off_snl);
    unsigned int *d_occ = (unsigned int *)(base + p.off_occ);
    const double fix = nlogn_fix_scale(g.F);  // per-bin rounding error 2^-(s+1)
    const OhSys hs{bins, g.ldb, d_ri, d_fix, d_snl, d_occ,
                   p.drain_slots ? (uint32_t *)(base + p.off_drain) : nullptr, g.F, (int)p.R, g.D, p.drain_slots};
    const OhFin hf{g, dof, d_snl, d_occ, out, log((double)g.F), fix};
    cudaError_t e;
    if ((e = cudaMemcpyAsync(d_ri, ri.data(), ri.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, st))) return e;
    if ((e = cudaMemcpyAsync(d_tiles, tiles.data(), tiles.size() * sizeof(TcTile), cudaMemcpyHostToDevice, st)))
        return e;
    if ((e = cudaMemcpyAsync(base + p.off_sys, &hs, sizeof hs, cudaMemcpyHostToDevice, st))) return e;
    if ((e = cudaMemcpyAsync(base + p.off_fin, &hf, sizeof hf, cudaMemcpyHostToDevice, st))) return e;
    // the host copies must outlive the transfers
    if ((e = cudaStreamSynchronize(st))) return e;
    if ((e = launch_nlogn_fix_table((unsigned long long *)d_fix, g.F, fix, st))) return e;
    run->scratch = scratch;
    run->off_sys = p.off_sys;
    run->off_fin = p.off_fin;
    run->off_tiles = p.off_tiles;
    run->off_snl = p.off_snl;
    run->acc_bytes = p.off_sys - p.off_snl;  // the accumulators up to the descriptors
    run->n_tiles = p.n_tiles;
    run->pair = pair;
    run->low = bmax2d(g) <= 64;
    run->D = g.D;
    return cudaSuccess;
}

cudaError_t onehot_run(const OnehotRun &run, int *err, cudaStream_t st) {
    char *base = (char *)run.scratch;
    cudaError_t e = cudaMemsetAsync(base + run.off_snl, 0, run.acc_bytes, st);
    if (e != cudaSuccess) return e;
    return launch_tiles((const OhSys *)(base + run.off_sys), (const TcTile *)(base + run.off_tiles), run.n_tiles,
                        run.pair, run.low, (const OhFin *)(base + run.off_fin), 1, run.D, err, st);
}

cudaError_t launch_pairs_onehot(const SysGeom &g, const uint8_t *bins, const DofArrays &dof,
                                const double *, PairOut out, int *err, cudaStream_t st, void *scratch,
                                size_t scratch_bytes, int *launches) {
    *launches = 0;
    OnehotRun run;
    cudaError_t e = onehot_setup(g, bins, dof, out, st, scratch, scratch_bytes, &run);
    if (e != cudaSuccess) return e;
    *launches = 3;  // n ln n table, pair kernel, finalize
    return onehot_run(run, err, st);
}

// ---- many systems in one launch (pg_entropy_batch)
//
// Workspace: OhSys[n] | OhFin[n] | tiles | per system: rowinfo, n ln n table
// | the accumulators of all systems, contiguous (one memset per run).
struct OhBatchLayout {
    std::vector<size_t> off_ri, off_fix, off_snl, off_occ;
    size_t off_sys = 0, off_fin = 0, off_tiles = 0, acc_begin = 0, acc_end = 0, off_drain = 0, total = 0;
    std::vector<TcTile> tiles;
    int max_D = 1, drain_slots = 0;
};

static OhBatchLayout batch_layout(const std::vector<SysGeom> &gs, bool pair) {
    OhBatchLayout L;
    const int n = (int)gs.size();
    // tiles of the systems with the most frames (the longest tiles) first
    std::vector<int> order((size_t)n);
    for (int s = 0; s < n; s++) order[s] = s;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return gs[a].F > gs[b].F; });
    for (int s : order) plan(gs[s], &L.tiles, pair, s);
    size_t off = 0;
    L.off_sys = off;
    off = al256(off + sizeof(OhSys) * n);
    L.off_fin = off;
    off = al256(off + sizeof(OhFin) * n);
    L.off_tiles = off;
    off = al256(off + sizeof(TcTile) * std::max<size_t>(L.tiles.size(), 1));
    L.off_ri.resize(n);
    L.off_fix.resize(n);
    L.off_snl.resize(n);
    L.off_occ.resize(n);
    for (int s = 0; s < n; s++) {
        int64_t R = 0;
        for (int d = 0; d < gs[s].D; d++) R += bins_of(gs[s], d);
        L.off_ri[s] = off;
        off = al256(off + sizeof(uint32_t) * (size_t)R);
        L.off_fix[s] = off;
        off = al256(off + sizeof(int64_t) * ((size_t)gs[s].F + 1));
        L.max_D = std::max(L.max_D, gs[s].D);
    }
    L.acc_begin = off;
    for (int s = 0; s < n; s++) {
        L.off_snl[s] = off;
        off += sizeof(unsigned long long) * (size_t)gs[s].D * gs[s].D;
        L.off_occ[s] = off;
        off = (off + sizeof(unsigned int) * (size_t)gs[s].D * gs[s].D + 7) / 8 * 8;
    }
    L.acc_end = off;
    int maxF = 0;
    for (const SysGeom &g : gs) maxF = std::max(maxF, g.F);
    L.drain_slots = drain_slots_for(maxF);
    L.off_drain = al256(off);
    L.total = al256(L.off_drain + sizeof(uint32_t) * kDrainSlotWords * (size_t)L.drain_slots);
    return L;
}

size_t pairs_onehot_batch_bytes(const std::vector<SysGeom> &gs) { return batch_layout(gs, use_pairs()).total; }

int64_t pairs_onehot_batch_tiles(const std::vector<SysGeom> &gs) {
    return (int64_t)batch_layout(gs, use_pairs()).tiles.size();
}

cudaError_t prepare_pairs_onehot_batch(const std::vector<SysGeom> &gs, const std::vector<const uint8_t *> &bins,
                                       const std::vector<DofArrays> &dofs, const std::vector<PairOut> &outs,
                                       void *ws, size_t ws_bytes, cudaStream_t st) {
    const bool pair = use_pairs();
    const OhBatchLayout L = batch_layout(gs, pair);
    if (ws_bytes < L.total) return cudaErrorInvalidValue;
    const int n = (int)gs.size();
    char *base = (char *)ws;
    std::vector<OhSys> hs((size_t)n);
    std::vector<OhFin> hf((size_t)n);
    std::vector<std::vector<uint32_t>> ri((size_t)n);
    cudaError_t e;
    for (int s = 0; s < n; s++) {
        const SysGeom &g = gs[s];
        if (!pairs_onehot_supported(g)) return cudaErrorInvalidValue;
        ri[s] = rowinfo_of(g);
        const double fix = nlogn_fix_scale(g.F);
        hs[s] = OhSys{bins[s], g.ldb, (const uint32_t *)(base + L.off_ri[s]), (const int64_t *)(base + L.off_fix[s]),
                      (unsigned long long *)(base + L.off_snl[s]), (unsigned int *)(base + L.off_occ[s]),
                      L.drain_slots ? (uint32_t *)(base + L.off_drain) : nullptr, g.F, (int)ri[s].size(), g.D,
                      L.drain_slots};
        hf[s] = OhFin{g, dofs[s], hs[s].acc_snl, hs[s].acc_occ, outs[s], log((double)g.F), fix};
        if ((e = cudaMemcpyAsync(base + L.off_ri[s], ri[s].data(), ri[s].size() * sizeof(uint32_t),
                                 cudaMemcpyHostToDevice, st)))
            return e;
        if ((e = launch_nlogn_fix_table((unsigned long long *)(base + L.off_fix[s]), g.F, fix, st))) return e;
    }
    if ((e = cudaMemcpyAsync(base + L.off_sys, hs.data(), sizeof(OhSys) * n, cudaMemcpyHostToDevice, st))) return e;
    if ((e = cudaMemcpyAsync(base + L.off_fin, hf.data(), sizeof(OhFin) * n, cudaMemcpyHostToDevice, st))) return e;
    if (!L.tiles.empty() &&
        (e = cudaMemcpyAsync(base + L.off_tiles, L.tiles.data(), sizeof(TcTile) * L.tiles.size(),
                             cudaMemcpyHostToDevice, st)))
        return e;
    return cudaStreamSynchronize(st);  // the host vectors go out of scope
}

cudaError_t launch_pairs_onehot_batch(const std::vector<SysGeom> &gs, void *ws, int *err, cudaStream_t st,
                                      int *launches) {
    const bool pair = use_pairs();
    const OhBatchLayout L = batch_layout(gs, pair);
    char *base = (char *)ws;
    cudaError_t e = cudaMemsetAsync(base + L.acc_begin, 0, L.acc_end - L.acc_begin, st);
    if (e != cudaSuccess) return e;
    *launches = 2;
    int bmax = 1;
    for (const SysGeom &g : gs) bmax = std::max(bmax, bmax2d(g));
    return launch_tiles((const OhSys *)(base + L.off_sys), (const TcTile *)(base + L.off_tiles),
                        (int64_t)L.tiles.size(), pair, bmax <= 64, (const OhFin *)(base + L.off_fin), (int)gs.size(),
                        L.max_D, err, st);
}

int64_t pairs_onehot_tiles(const SysGeom &g) { return plan(g, nullptr, use_pairs()).n_tiles; }

}  // namespace pg
