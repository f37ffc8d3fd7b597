// .bat ingest on the device: frame-major records -> DOF-major columns.
//
// Replaces PARENT's per-frame scatter of read_BAT_frame's values into the
// DOF-major `bonds/angles/dihedrals` arrays (PARENT.cpp:443-473; the record
// layout is read_BAT_frame's, io_binary.cpp:281-368). The host reads the
// file's frame records in large chunks into pinned buffers and copies them to
// the device unchanged; this kernel transposes a chunk through shared memory:
// a 32 x 32 tile of (frame, value) is read along the values of a record and
// written along the frames of a column, so both sides stay coalesced.
//
// A record holds 11 floats (time, precision, box), the 6 root externals and
// then b0 b1 a0 (b a d) x nDih, each value 4 or 8 bytes. Value u (counted
// from b0) lands in
//   u = 0, 1        -> bond u
//   u = 2           -> angle 0
//   u = 3 + 3k + r  -> bond k+2 (r = 0), angle k+1 (r = 1), dihedral k (r = 2)
// of the column block bonds | angles | dihedrals (column stride ld elements).
// Double values sit on 4-byte boundaries only (the 44-byte float block), so
// they are loaded as two 32-bit words.
#include <stdint.h>

#include <type_traits>

#include <cuda_runtime.h>

namespace pg {

namespace {

__device__ __forceinline__ int64_t column_of(int u, int nb, int na) {
    if (u < 2) return u;
    if (u == 2) return nb;
    const int k = (u - 3) / 3, r = (u - 3) - 3 * k;
    return r == 0 ? k + 2 : (r == 1 ? (int64_t)nb + k + 1 : (int64_t)nb + na + k);
}

template <int ES>
__global__ void __launch_bounds__(256) bat_transpose_kernel(const uint8_t *__restrict__ raw, int nf, int64_t rec,
                                                            int off0, int nvals, int nb, int na,
                                                            uint8_t *__restrict__ cols, int64_t ld, int64_t f0) {
    using Word = typename std::conditional<ES == 4, uint32_t, unsigned long long>::type;
    __shared__ Word tile[32][33];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int u0 = blockIdx.x * 32, i0 = blockIdx.y * 32;
#pragma unroll
    for (int r = ty; r < 32; r += 8) {
        const int i = i0 + r, u = u0 + tx;
        if (i < nf && u < nvals) {
            const uint32_t *p = (const uint32_t *)(raw + (int64_t)i * rec + off0 + (int64_t)u * ES);
            if constexpr (ES == 4) {
                tile[r][tx] = __ldg(p);
            } else {
                tile[r][tx] = (unsigned long long)__ldg(p) | ((unsigned long long)__ldg(p + 1) << 32);
            }
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = ty; r < 32; r += 8) {
        const int u = u0 + r, i = i0 + tx;
        if (u < nvals && i < nf) ((Word *)cols)[column_of(u, nb, na) * ld + f0 + i] = tile[tx][r];
    }
}

// dst[i] = src[i] for n 16-byte words; src is host memory the GPU can read
// directly (pinned, or pageable where the platform maps it): the SMs pull it
// over the host link, which on Grace-attached parts outruns a copy engine
// (210 vs 120-210 GB/s measured, and unaffected by kernels running meanwhile)
__global__ void __launch_bounds__(512) host_pull_kernel(const uint4 *__restrict__ src, uint4 *__restrict__ dst,
                                                        size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

}  // namespace

// Copies `bytes` from host memory to the device with a pull kernel when the
// GPU can read `src` directly and both addresses and the size are 16-byte
// multiples; with a copy-engine copy otherwise. *pulled says which.
bool host_readable(const void *src) {
    bool readable = false;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, src) == cudaSuccess) {
        if (at.type == cudaMemoryTypeHost && at.devicePointer == src) readable = true;
        if (at.type == cudaMemoryTypeUnregistered) {
            int dev = 0, pma = 0;
            cudaGetDevice(&dev);
            readable = cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, dev) == cudaSuccess && pma;
        }
    }
    cudaGetLastError();
    return readable;
}

cudaError_t h2d_copy(void *dst, const void *src, size_t bytes, cudaStream_t st, bool *pulled) {
    *pulled = false;
    if (bytes == 0) return cudaSuccess;
    const bool aligned = (((uintptr_t)dst | (uintptr_t)src | bytes) & 15) == 0;
    const bool readable = aligned && host_readable(src);
    if (!readable) return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    host_pull_kernel<<<4 * sms, 512, 0, st>>>((const uint4 *)src, (uint4 *)dst, bytes / 16);
    *pulled = true;
    return cudaGetLastError();
}

// raw: nf records of rec bytes on the device; values start at byte off0 of a
// record, es (4 or 8) bytes each, 3 + 3 nDih of them. Writes frames
// [f0, f0 + nf) of every column of `cols` (ld elements apart).
cudaError_t launch_bat_transpose(const uint8_t *raw, int nf, int64_t rec, int off0, int es, int n_dih,
                                 uint8_t *cols, int64_t ld, int64_t f0, cudaStream_t st) {
    if (nf <= 0) return cudaSuccess;
    if ((es != 4 && es != 8) || rec % 4 != 0 || off0 % 4 != 0 || n_dih < 0) return cudaErrorInvalidValue;
    const int nvals = 3 + 3 * n_dih, nb = n_dih + 2, na = n_dih + 1;
    const dim3 block(32, 8), grid((nvals + 31) / 32, (nf + 31) / 32);
    if (grid.y > 65535u) return cudaErrorInvalidValue;
    if (es == 4)
        bat_transpose_kernel<4><<<grid, block, 0, st>>>(raw, nf, rec, off0, nvals, nb, na, cols, ld, f0);
    else
        bat_transpose_kernel<8><<<grid, block, 0, st>>>(raw, nf, rec, off0, nvals, nb, na, cols, ld, f0);
    return cudaGetLastError();
}

}  // namespace pg
