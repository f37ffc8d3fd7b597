// MIST maximum spanning tree on the GPU.
//
// The reference (get_PAR_MIST.cpp:441-748) rescans every (In, Out) pair at
// each step, O(n^3) overall, and keeps the FIRST maximum in the scan order
//   blocks (In type, Out type) = BB BA BD AB AA AD DB DA DD,
//   then In insertion position, then Out DOF index      (strict '>').
// This kernel runs Prim's algorithm with one key per Out vertex, O(n^2):
//   key[v]  = best MI from any In vertex to v,
//   from[v] = the In vertex giving it; on an exact tie the In vertex of lower
//             type wins, and among equal types the earlier-inserted one
//             (it was there first), which is the reference's order restricted
//             to a fixed v.
// The step winner is the Out vertex with the largest key, ties broken by
// (type(from), type(v), position(from), v) ascending, i.e. the reference's
// scan order.
//
// One persistent CTA; thread t owns the vertices v = t, t + blockDim, ... and
// is the only thread that touches their key/from, so a step is one pass over
// the owned vertices (read the MI row of the vertex that joined last, relax,
// keep the best candidate), a warp reduction, ONE block barrier, and a
// redundant reduction of the per-warp bests by every warp (per-warp bests are
// double-buffered by step parity). The position of the vertex that joined in
// the previous step is taken from registers, every older one from shared
// memory (written before the last barrier).
//
// MI values are compared as order-preserving 64-bit integer images of the
// doubles (sign-magnitude flipped to two's-complement order, -0 folded onto
// +0), so equal doubles give equal keys and every comparison runs on the
// integer pipe; the FP64 pipe of this part is a small fraction of its
// integer rate.
#include <stdint.h>
#include <stdlib.h>

#include "pg_internal.h"

namespace pg {

namespace {

constexpr int kMaxThreads = 1024;
constexpr int kMaxWarps = kMaxThreads / 32;

// order-preserving image of a double; 0 is below every value. NaN maps to 0:
// it never beats anything, as no strict '>' with a NaN holds in the reference.
__device__ __forceinline__ unsigned long long okey(double x) {
    unsigned long long b = (unsigned long long)__double_as_longlong(x);
    if ((b & 0x7fffffffffffffffull) > 0x7ff0000000000000ull) return 0ull;  // NaN
    if (b == 0x8000000000000000ull) b = 0ull;  // -0 == +0
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double okey_value(unsigned long long k) {
    const unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    return __longlong_as_double((long long)b);
}

// A candidate: its key and a secondary word that orders equal keys,
// ~((type(from) << 62) | (type(v) << 60) | (pos(from) << 30) | v), so that the
// reference's first-in-scan-order candidate has the LARGEST (key, sec).
struct Cand {
    unsigned long long key, sec;
    int v, from;
};

__device__ __forceinline__ bool beats(const Cand &a, const Cand &b) {
    return a.key > b.key || (a.key == b.key && a.sec > b.sec);
}

__device__ __forceinline__ unsigned long long sec_of(int tf, int tv, int posf, int v) {
    return ~(((unsigned long long)tf << 62) | ((unsigned long long)tv << 60) |
             ((unsigned long long)(unsigned)posf << 30) | (unsigned long long)(unsigned)v);
}

__device__ __forceinline__ Cand shfl_cand(const Cand &c, int o) {
    Cand r;
    r.key = __shfl_xor_sync(0xffffffffu, c.key, o);
    r.sec = __shfl_xor_sync(0xffffffffu, c.sec, o);
    r.v = __shfl_xor_sync(0xffffffffu, c.v, o);
    r.from = __shfl_xor_sync(0xffffffffu, c.from, o);
    return r;
}

__device__ __forceinline__ Cand warp_best(Cand c) {
    for (int o = 16; o > 0; o >>= 1) {
        const Cand other = shfl_cand(c, o);
        if (beats(other, c)) c = other;
    }
    return c;
}

template <bool SMEM>
__device__ __forceinline__ void mist_body(int D, int nb, int na, const double *__restrict__ mi,
                                          unsigned long long *gkey, int *gfrom, int *gpos, double *edge_mi,
                                          int *edge_from, int *edge_to) {
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned long long *key = SMEM ? (unsigned long long *)smem : gkey;
    int *from = SMEM ? (int *)(smem + (size_t)D * sizeof(unsigned long long)) : gfrom;
    int *pos = SMEM ? from + D : gpos;
    __shared__ Cand wbest[2][kMaxWarps];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nthr = blockDim.x, nwarps = nthr >> 5;

    // In = {bond 0} (get_PAR_MIST.cpp:419-422)
    for (int v = tid; v < D; v += nthr) {
        key[v] = 0ull;
        from[v] = v == 0 ? -2 : -1;  // -2: in the tree, -1: no In partner yet
    }
    if (tid == 0) pos[0] = 0;
    int last_w = 0, last_pos = 0;  // the vertex that joined last and its position
    // ordering (and the initial pos) only need this barrier once: afterwards
    // every thread touches only its own vertices' key/from
    __syncthreads();

    for (int step = 0; step < D - 1; step++) {
        const int tw = dof_type(last_w, nb, na);
        const double *row = mi + (int64_t)last_w * D;
        Cand best{0ull, 0ull, -1, -1};
        for (int v0 = tid; v0 < D; v0 += 4 * nthr) {
            // the row loads of up to four owned vertices go out together
            double mv[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int v = v0 + u * nthr;
                mv[u] = v < D ? __ldg(row + v) : 0.0;
            }
#pragma unroll
            for (int u = 0; u < 4; u++) {
            const int v = v0 + u * nthr;
            if (v >= D) break;
            int f = from[v];
            if (f == -2) continue;
            const unsigned long long m = okey(mv[u]);
            unsigned long long k = key[v];
            if (m > k || (m == k && f >= 0 && tw < dof_type(f, nb, na))) {
                key[v] = m;
                from[v] = last_w;
                k = m;
                f = last_w;
            }
            const int tf = f >= 0 ? dof_type(f, nb, na) : 3;
            const int pf = f < 0 ? (1 << 30) - 1 : (f == last_w ? last_pos : pos[f]);
            const Cand c{k, sec_of(tf, dof_type(v, nb, na), pf, v), v, f};
            if (best.v < 0 || beats(c, best)) best = c;
            }
        }
        best = warp_best(best);
        if (lane == 0) wbest[step & 1][warp] = best;
        __syncthreads();
        // every warp reduces the per-warp bests (the same data, the same result)
        Cand b = lane < nwarps ? wbest[step & 1][lane] : Cand{0ull, 0ull, -1, -1};
        if (b.v < 0) b.key = 0ull, b.sec = 0ull;
        b = warp_best(b);
        const int w = b.v < 0 ? 0 : b.v;
        if (tid == 0) {
            edge_mi[step] = okey_value(b.key);
            edge_from[step] = b.v < 0 ? -1 : b.from;
            edge_to[step] = b.v;
        }
        if (b.v >= 0 && w % nthr == tid) {  // the owner of the joining vertex
            from[w] = -2;
            pos[w] = step + 1;
        }
        last_w = w;
        last_pos = step + 1;
    }
}

// ---- the same Prim steps over a cluster of kClusterCtas CTAs: CTA r owns
// the vertices [r S, (r + 1) S), S = ceil(D / kClusterCtas), with their
// key/from in its shared memory, so each step reads 1/8 of a row of the MI
// matrix per SM. Every warp sends its best candidate to a slot in every CTA
// of the cluster (distributed shared memory, slots double-buffered by step
// parity), ONE cluster barrier per step, and every warp reduces the slots to
// the same winner. All CTAs run the same D - 1 steps, so every barrier is
// met. The cluster barrier costs ~1.7 us a step, so the form pays from about
// a thousand vertices on (measured: 294 DOFs 0.52 vs 0.36 ms on one CTA;
// 2,994 DOFs 7.3 vs 9.5 ms; 7,494 DOFs 28.0 vs 40.4 ms).
constexpr int kClusterCtas = 8;
constexpr int kSlots = kClusterCtas * kMaxWarps;  // per parity
constexpr int kClusterMinD = 1024;

__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t map_to_rank(const void *p, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"((uint32_t)__cvta_generic_to_shared(p)), "r"(rank));
    return r;
}
__device__ __forceinline__ void st_cluster_cand(uint32_t addr, const Cand &c) {
    asm volatile("st.shared::cluster.u64 [%0], %1;" ::"r"(addr), "l"(c.key) : "memory");
    asm volatile("st.shared::cluster.u64 [%0], %1;" ::"r"(addr + 8), "l"(c.sec) : "memory");
    asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(addr + 16), "r"(c.v) : "memory");
    asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(addr + 20), "r"(c.from) : "memory");
}
__device__ __forceinline__ void cluster_barrier() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

size_t mist_cluster_smem(int D) {
    const size_t S = (size_t)(D + kClusterCtas - 1) / kClusterCtas;
    return S * sizeof(unsigned long long) + 2 * kSlots * sizeof(Cand) + S * sizeof(int) + (size_t)D * sizeof(int);
}

__global__ void __launch_bounds__(kMaxThreads, 1)
mist_cluster_kernel(int D, int nb, int na, const double *__restrict__ mi, double *edge_mi, int *edge_from,
                    int *edge_to) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int S = (D + kClusterCtas - 1) / kClusterCtas;
    const int rank = (int)cluster_rank();
    const int v0 = rank * S, nloc = max(0, min(D, v0 + S) - v0);
    unsigned long long *key = (unsigned long long *)smem;      // [S]
    Cand *slots = (Cand *)(key + S);                             // [2][kSlots]
    int *from = (int *)(slots + 2 * kSlots);                     // [S]
    int *pos = from + S;                                         // [D], every CTA's copy
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nthr = blockDim.x;

    // In = {bond 0} (get_PAR_MIST.cpp:419-422)
    for (int i = tid; i < nloc; i += nthr) {
        key[i] = 0ull;
        from[i] = v0 + i == 0 ? -2 : -1;
    }
    for (int i = tid; i < 2 * kSlots; i += nthr) slots[i] = Cand{0ull, 0ull, -1, -1};
    if (tid == 0) pos[0] = 0;
    cluster_barrier();  // slots initialised everywhere before any remote write
    int last_w = 0, last_pos = 0;
    for (int step = 0; step < D - 1; step++) {
        const int tw = dof_type(last_w, nb, na);
        Cand best{0ull, 0ull, -1, -1};
        for (int i = tid; i < nloc; i += nthr) {
            const int v = v0 + i;
            int f = from[i];
            if (f == -2) continue;
            const double mv = __ldg(mi + (int64_t)last_w * D + v);
            const unsigned long long m = okey(mv);
            unsigned long long k = key[i];
            if (m > k || (m == k && f >= 0 && tw < dof_type(f, nb, na))) {
                key[i] = m;
                from[i] = last_w;
                k = m;
                f = last_w;
            }
            const int tf = f >= 0 ? dof_type(f, nb, na) : 3;
            const int pf = f < 0 ? (1 << 30) - 1 : (f == last_w ? last_pos : pos[f]);
            const Cand c{k, sec_of(tf, dof_type(v, nb, na), pf, v), v, f};
            if (best.v < 0 || beats(c, best)) best = c;
        }
        best = warp_best(best);
        if (best.v < 0) best.key = 0ull, best.sec = 0ull;
        Cand *slot = slots + (step & 1) * kSlots + rank * kMaxWarps + warp;
        if (lane < kClusterCtas) st_cluster_cand(map_to_rank(slot, (uint32_t)lane), best);
        cluster_barrier();
        // every warp reduces every CTA's warp bests (the same data, the same result)
        const Cand *ps = slots + (step & 1) * kSlots;
        Cand b{0ull, 0ull, -1, -1};
        for (int j = lane; j < kSlots; j += 32) {
            const Cand x = ps[j];
            if (x.v >= 0 && (b.v < 0 || beats(x, b))) b = x;
        }
        if (b.v < 0) b.key = 0ull, b.sec = 0ull;
        b = warp_best(b);
        const int w = b.v < 0 ? 0 : b.v;
        if (rank == 0 && tid == 0) {
            edge_mi[step] = okey_value(b.key);
            edge_from[step] = b.v < 0 ? -1 : b.from;
            edge_to[step] = b.v;
        }
        if (b.v >= 0 && w >= v0 && w < v0 + nloc && (w - v0) % nthr == tid) from[w - v0] = -2;  // its owner
        if (b.v >= 0 && tid == 0) pos[w] = step + 1;  // read from step + 2 on, after the next barrier
        last_w = w;
        last_pos = step + 1;
    }
}

template <bool SMEM>
__global__ void __launch_bounds__(kMaxThreads, 1)
mist_kernel(int D, int nb, int na, const double *__restrict__ mi, unsigned long long *gkey, int *gfrom,
            int *pos, double *edge_mi, int *edge_from, int *edge_to) {
    mist_body<SMEM>(D, nb, na, mi, gkey, gfrom, pos, edge_mi, edge_from, edge_to);
}

// One CTA per system of a batch.
template <bool SMEM>
__global__ void __launch_bounds__(kMaxThreads, 1) mist_batch_kernel(const MistDesc *__restrict__ sys) {
    const MistDesc &d = sys[blockIdx.x];
    unsigned long long *gkey = (unsigned long long *)d.scratch;
    int *gfrom = (int *)(gkey + d.D);
    int *pos = gfrom + d.D;
    mist_body<SMEM>(d.D, d.nb, d.na, d.mi, gkey, gfrom, pos, d.edge_mi, d.edge_from, d.edge_to);
}

// Threads per CTA for D vertices: one vertex per thread up to 1,024 (whole
// warps, at least 64), 1,024 threads above.
int mist_threads(int D) {
    int t = (D + 31) / 32 * 32;
    return t < 64 ? 64 : (t > kMaxThreads ? kMaxThreads : t);
}

// Dense symmetric MI matrix from a .par body on the device, get_mutual
// (util.cpp:47-81): MI = S1[lower] + S1[higher] - S2D.
__global__ void mi_from_par_kernel(int n_dih, const double *par, ParLayout L, double *mi) {
    const int nb = n_dih + 2, na = n_dih + 1, nd = n_dih, D = nb + na + nd;
    const int64_t total = (int64_t)D * D;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(idx / D), c = (int)(idx % D);
        if (r == c) { mi[idx] = 0.0; continue; }
        const int g1 = r < c ? r : c, g2 = r < c ? c : r;
        const int t1 = dof_type(g1, nb, na), t2 = dof_type(g2, nb, na);
        const int64_t o1 = t1 == TB ? L.s1b + g1 : (t1 == TA ? L.s1a + g1 - nb : L.s1d + g1 - nb - na);
        const int64_t o2 = t2 == TB ? L.s1b + g2 : (t2 == TA ? L.s1a + g2 - nb : L.s1d + g2 - nb - na);
        mi[idx] = par[o1] + par[o2] - par[par_pair_index(L, nb, na, nd, g1, g2)];
    }
}

}  // namespace

size_t mist_scratch_bytes(int D) { return (size_t)D * (sizeof(double) + 2 * sizeof(int)) + 256; }

// Prim over a cluster of 8 CTAs (kernel above) from kClusterMinD vertices up,
// one CTA below; PG_MIST_CLUSTER=0 keeps one CTA.
static bool mist_cluster_enabled() {
    const char *e = getenv("PG_MIST_CLUSTER");
    return !(e && atoi(e) == 0);
}

cudaError_t launch_mist_impl(int D, int nb, int na, const double *mi, void *scratch,
                             double *edge_mi, int *edge_from, int *edge_to, cudaStream_t st) {
    if (D >= kClusterMinD && mist_cluster_enabled()) {
        const size_t smem = mist_cluster_smem(D);
        if (smem <= 200 * 1024) {
            auto kern = mist_cluster_kernel;
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(kClusterCtas);
            cfg.blockDim = dim3(mist_threads((D + kClusterCtas - 1) / kClusterCtas));
            cfg.dynamicSmemBytes = smem;
            cfg.stream = st;
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = kClusterCtas;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            cfg.attrs = at;
            cfg.numAttrs = 1;
            e = cudaLaunchKernelEx(&cfg, kern, D, nb, na, mi, edge_mi, edge_from, edge_to);
            if (e != cudaSuccess) return e;
            return cudaGetLastError();
        }
    }
    unsigned long long *gkey = (unsigned long long *)scratch;
    int *gfrom = (int *)(gkey + D);
    int *pos = gfrom + D;
    const size_t smem = (size_t)D * (sizeof(unsigned long long) + 2 * sizeof(int));
    const int nthr = mist_threads(D);
    if (smem <= 200 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(mist_kernel<true>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        mist_kernel<true><<<1, nthr, smem, st>>>(D, nb, na, mi, gkey, gfrom, pos, edge_mi, edge_from, edge_to);
    } else {
        mist_kernel<false><<<1, nthr, 0, st>>>(D, nb, na, mi, gkey, gfrom, pos, edge_mi, edge_from, edge_to);
    }
    return cudaGetLastError();
}

cudaError_t launch_mist_batch(const MistDesc *sys, int n_sys, int max_D, cudaStream_t st) {
    if (n_sys <= 0) return cudaSuccess;
    const size_t smem = (size_t)max_D * (sizeof(unsigned long long) + 2 * sizeof(int));
    const int nthr = mist_threads(max_D);
    if (smem <= 200 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(mist_batch_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        mist_batch_kernel<true><<<n_sys, nthr, smem, st>>>(sys);
    } else {
        mist_batch_kernel<false><<<n_sys, nthr, 0, st>>>(sys);
    }
    return cudaGetLastError();
}

cudaError_t launch_mi_from_par(int n_dih, const double *par, ParLayout L, double *mi,
                               cudaStream_t st) {
    const int D = 3 * n_dih + 3;
    int64_t total = (int64_t)D * D;
    int blocks = (int)((total + 255) / 256);
    if (blocks > 152 * 32) blocks = 152 * 32;
    mi_from_par_kernel<<<blocks, 256, 0, st>>>(n_dih, par, L, mi);
    return cudaGetLastError();
}

}  // namespace pg
