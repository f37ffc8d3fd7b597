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
// scan order. One persistent CTA of 1024 threads keeps key/from in shared
// memory and reads one MI row (the vertex that just joined) per step.
//
// MI values are compared as order-preserving 64-bit integer images of the
// doubles (sign-magnitude flipped to two's-complement order, -0 folded onto
// +0), so equal doubles give equal keys and every comparison runs on the
// integer pipe; the FP64 pipe of this part is a small fraction of its
// integer rate.
#include <stdint.h>

#include "pg_internal.h"

namespace pg {

namespace {

constexpr int kThreads = 1024;
constexpr int kWarps = kThreads / 32;

struct Cand {
    unsigned long long key;
    int v;  // -1: none
};

// order-preserving image of a (non-NaN) double; 0 is below every value
__device__ __forceinline__ unsigned long long okey(double x) {
    unsigned long long b = (unsigned long long)__double_as_longlong(x);
    if (b == 0x8000000000000000ull) b = 0ull;  // -0 == +0
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double okey_value(unsigned long long k) {
    const unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    return __longlong_as_double((long long)b);
}

__device__ __forceinline__ int type_of(int g, int nb, int na) { return dof_type(g, nb, na); }

// true if candidate a comes before candidate b in the reference's order
__device__ __forceinline__ bool better(const Cand &a, const Cand &b, const int *from,
                                       const int *pos, int nb, int na) {
    if (a.v < 0) return false;
    if (b.v < 0) return true;
    if (a.key > b.key) return true;
    if (a.key < b.key) return false;
    const int fa = from[a.v], fb = from[b.v];
    const int tfa = fa >= 0 ? type_of(fa, nb, na) : 3, tfb = fb >= 0 ? type_of(fb, nb, na) : 3;
    if (tfa != tfb) return tfa < tfb;
    const int tva = type_of(a.v, nb, na), tvb = type_of(b.v, nb, na);
    if (tva != tvb) return tva < tvb;
    const int pa = fa >= 0 ? pos[fa] : 0x7fffffff, pb = fb >= 0 ? pos[fb] : 0x7fffffff;
    if (pa != pb) return pa < pb;
    return a.v < b.v;
}

template <bool SMEM>
__device__ __forceinline__ void mist_body(int D, int nb, int na, const double *__restrict__ mi,
                                          unsigned long long *gkey, int *gfrom, int *pos, double *edge_mi,
                                          int *edge_from, int *edge_to) {
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned long long *key = SMEM ? (unsigned long long *)smem : gkey;
    int *from = SMEM ? (int *)(smem + (size_t)D * sizeof(unsigned long long)) : gfrom;
    __shared__ Cand wbest[kWarps];
    __shared__ int s_win;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    // In = {bond 0} (get_PAR_MIST.cpp:419-422)
    for (int v = tid; v < D; v += kThreads) {
        key[v] = 0ull;
        from[v] = v == 0 ? -2 : -1;  // -2: in the tree, -1: no In partner yet
    }
    if (tid == 0) {
        pos[0] = 0;
        s_win = 0;
    }
    __syncthreads();

    for (int step = 0; step < D; step++) {
        // relax keys with the row of the vertex that joined last
        const int w = s_win;
        const int tw = type_of(w, nb, na);
        const double *row = mi + (int64_t)w * D;
        for (int v = tid; v < D; v += kThreads) {
            const int f = from[v];
            if (f == -2) continue;
            const unsigned long long m = okey(__ldg(row + v));
            const unsigned long long k = key[v];
            if (m > k || (m == k && f >= 0 && tw < type_of(f, nb, na))) {
                key[v] = m;
                from[v] = w;
            }
        }
        if (step == D - 1) break;
        __syncthreads();
        // argmax in the reference's order
        Cand best{0ull, -1};
        for (int v = tid; v < D; v += kThreads) {
            if (from[v] == -2) continue;
            const Cand c{key[v], v};
            if (better(c, best, from, pos, nb, na)) best = c;
        }
        for (int o = 16; o > 0; o >>= 1) {
            Cand other;
            other.key = __shfl_xor_sync(0xffffffffu, best.key, o);
            other.v = __shfl_xor_sync(0xffffffffu, best.v, o);
            if (better(other, best, from, pos, nb, na)) best = other;
        }
        if (lane == 0) wbest[warp] = best;
        __syncthreads();
        if (warp == 0) {
            Cand b = wbest[lane];
            for (int o = 16; o > 0; o >>= 1) {
                Cand other;
                other.key = __shfl_xor_sync(0xffffffffu, b.key, o);
                other.v = __shfl_xor_sync(0xffffffffu, b.v, o);
                if (better(other, b, from, pos, nb, na)) b = other;
            }
            if (lane == 0) {
                const int v = b.v < 0 ? 0 : b.v;
                edge_mi[step] = okey_value(b.key);
                edge_from[step] = b.v < 0 ? -1 : from[v];
                edge_to[step] = b.v;
                if (b.v >= 0) {
                    pos[v] = step + 1;
                    from[v] = -2;
                }
                s_win = v;
            }
        }
        __syncthreads();
    }
}

template <bool SMEM>
__global__ void __launch_bounds__(kThreads, 1)
mist_kernel(int D, int nb, int na, const double *__restrict__ mi, unsigned long long *gkey, int *gfrom,
            int *pos, double *edge_mi, int *edge_from, int *edge_to) {
    mist_body<SMEM>(D, nb, na, mi, gkey, gfrom, pos, edge_mi, edge_from, edge_to);
}

// One CTA per system of a batch.
template <bool SMEM>
__global__ void __launch_bounds__(kThreads, 1) mist_batch_kernel(const MistDesc *__restrict__ sys) {
    const MistDesc &d = sys[blockIdx.x];
    unsigned long long *gkey = (unsigned long long *)d.scratch;
    int *gfrom = (int *)(gkey + d.D);
    int *pos = gfrom + d.D;
    mist_body<SMEM>(d.D, d.nb, d.na, d.mi, gkey, gfrom, pos, d.edge_mi, d.edge_from, d.edge_to);
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

cudaError_t launch_mist_impl(int D, int nb, int na, const double *mi, void *scratch,
                             double *edge_mi, int *edge_from, int *edge_to, cudaStream_t st) {
    unsigned long long *gkey = (unsigned long long *)scratch;
    int *gfrom = (int *)(gkey + D);
    int *pos = gfrom + D;
    const size_t smem = (size_t)D * (sizeof(unsigned long long) + sizeof(int));
    if (smem <= 200 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(mist_kernel<true>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        mist_kernel<true><<<1, kThreads, smem, st>>>(D, nb, na, mi, gkey, gfrom, pos, edge_mi,
                                                     edge_from, edge_to);
    } else {
        mist_kernel<false><<<1, kThreads, 0, st>>>(D, nb, na, mi, gkey, gfrom, pos, edge_mi,
                                                   edge_from, edge_to);
    }
    return cudaGetLastError();
}

cudaError_t launch_mist_batch(const MistDesc *sys, int n_sys, int max_D, cudaStream_t st) {
    if (n_sys <= 0) return cudaSuccess;
    const size_t smem = (size_t)max_D * (sizeof(double) + sizeof(int));
    if (smem <= 200 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(mist_batch_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        mist_batch_kernel<true><<<n_sys, kThreads, smem, st>>>(sys);
    } else {
        mist_batch_kernel<false><<<n_sys, kThreads, 0, st>>>(sys);
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
