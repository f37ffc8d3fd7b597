// Cartesian -> BAT conversion on the device.
//
// Replaces BAT_builder's per-frame conversion (BAT_trajectory.cpp:114-125):
// coordinates scaled by 10 (nm -> Angstrom, stored back as float),
// convert_to_BAT (:219-300), convert_dihedrals_to_phaseangles (:303-310) and
// shift_dihedrals_0_2pi_range (:209-214), writing the DOF-major columns that
// pg_entropy reads (the values BAT_builder would write to the .bat, in its
// precision) without a .bat file in between.
//
// Three kernels per chunk of frames:
//   1. cart_transpose_kernel: frame-major (frame, atom, xyz) floats -> one
//      row per (atom, coordinate), frames contiguous, scaled by 10 as the
//      reference does (float * 10.0 in double, rounded back to float);
//   2. bat_convert_kernel: one thread per frame, a block row per group of
//      dihedrals: the difference vectors in float, everything after in FP64
//      in the reference's operation order (this file is compiled without
//      FMA contraction), bond, angle and raw dihedral per dihedral, the two
//      root bonds and the root angle in the first block row;
//   3. bat_phase_kernel: one thread per frame, in dihedral order: subtract the
//      parent dihedral in place (a parent later in the list is still raw when
//      it is read, as in the reference's in-place loop), then the shift into
//      [0, 2 pi).
// sqrt and the IEEE divisions are correctly rounded on both sides, so bonds
// are bit-identical to the reference; acos and atan2 come from CUDA's libm
// and may differ from the host's in the last place.
#include <math.h>
#include <stdint.h>

#include <cuda_runtime.h>

namespace pg {

namespace {

constexpr int kConvThreads = 128;
constexpr int kDihPerRow = 32;   // dihedrals per block row of the conversion grid
constexpr int kPhaseThreads = 128;

__global__ void __launch_bounds__(256) cart_transpose_kernel(const float *__restrict__ aos, int nf, int ncols,
                                                             float *__restrict__ soa, int64_t lds) {
    __shared__ float tile[32][33];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int c0 = blockIdx.x * 32, f0 = blockIdx.y * 32;
#pragma unroll
    for (int r = ty; r < 32; r += 8) {
        const int f = f0 + r, c = c0 + tx;
        if (f < nf && c < ncols) tile[r][tx] = __double2float_rn((double)__ldg(aos + (int64_t)f * ncols + c) * 10.0);
    }
    __syncthreads();
#pragma unroll
    for (int r = ty; r < 32; r += 8) {
        const int c = c0 + r, f = f0 + tx;
        if (c < ncols && f < nf) soa[(int64_t)c * lds + f] = tile[tx][r];
    }
}

struct Vec3 {
    double x, y, z;
};

// x[a1] - x[a0] per coordinate in float (the reference's operands are float)
__device__ __forceinline__ Vec3 diff(const float *__restrict__ soa, int64_t lds, int f, int a1, int a0) {
    const float *p1 = soa + (int64_t)(3 * a1) * lds + f, *p0 = soa + (int64_t)(3 * a0) * lds + f;
    Vec3 v;
    v.x = (double)__fsub_rn(__ldg(p1), __ldg(p0));
    v.y = (double)__fsub_rn(__ldg(p1 + lds), __ldg(p0 + lds));
    v.z = (double)__fsub_rn(__ldg(p1 + 2 * lds), __ldg(p0 + 2 * lds));
    return v;
}

__device__ __forceinline__ void put(void *col, int prec, int64_t idx, double v) {
    if (prec) ((double *)col)[idx] = v;
    else ((float *)col)[idx] = __double2float_rn(v);
}

// atoms: per dihedral the four atoms (0-based). Writes bonds/angles columns
// (typed, frames f0 + f) and the raw dihedral into dtmp (FP64, ldt apart).
__global__ void __launch_bounds__(kConvThreads) bat_convert_kernel(const float *__restrict__ soa, int64_t lds, int nf,
                                                                   int nd, const int4 *__restrict__ atoms,
                                                                   void *bonds, void *angles, int64_t ld, int64_t f0,
                                                                   int prec, double *__restrict__ dtmp, int64_t ldt) {
    const int f = blockIdx.x * kConvThreads + threadIdx.x;
    if (f >= nf) return;
    const int i0 = blockIdx.y * kDihPerRow, i1 = min(nd, i0 + kDihPerRow);
    if (blockIdx.y == 0) {  // root bonds and angle (:229-265)
        const int4 r = __ldg(atoms);
        const Vec3 b2 = diff(soa, lds, f, r.y, r.x), b3 = diff(soa, lds, f, r.z, r.y);
        const double rb0 = sqrt(b2.x * b2.x + b2.y * b2.y + b2.z * b2.z);
        const double rb1 = sqrt(b3.x * b3.x + b3.y * b3.y + b3.z * b3.z);
        const double ra = acos((b2.x * b3.x + b2.y * b3.y + b2.z * b3.z) / rb0 / rb1);
        put(bonds, prec, f0 + f, rb0);
        put(bonds, prec, ld + f0 + f, rb1);
        put(angles, prec, f0 + f, ra);
    }
    for (int i = i0; i < i1; i++) {  // :270-298
        const int4 a = __ldg(atoms + i);
        const Vec3 b1 = diff(soa, lds, f, a.y, a.x), b2 = diff(soa, lds, f, a.z, a.y), b3 = diff(soa, lds, f, a.w, a.z);
        const double bl = sqrt(b3.x * b3.x + b3.y * b3.y + b3.z * b3.z);
        const double prev = sqrt(b2.x * b2.x + b2.y * b2.y + b2.z * b2.z);
        const double ang = acos((b2.x * b3.x + b2.y * b3.y + b2.z * b3.z) / bl / prev);
        const double A0 = b1.y * b2.z - b1.z * b2.y, A1 = b1.z * b2.x - b1.x * b2.z, A2 = b1.x * b2.y - b1.y * b2.x;
        const double B0 = b2.y * b3.z - b2.z * b3.y, B1 = b2.z * b3.x - b2.x * b3.z, B2 = b2.x * b3.y - b2.y * b3.x;
        const double num = (A2 * B0 - A0 * B2) * b2.y / prev - (A2 * B1 - A1 * B2) * b2.x / prev -
                           (A1 * B0 - A0 * B1) * b2.z / prev;
        const double den = A0 * B0 + A1 * B1 + A2 * B2;
        put(bonds, prec, (int64_t)(i + 2) * ld + f0 + f, bl);
        put(angles, prec, (int64_t)(i + 1) * ld + f0 + f, ang);
        dtmp[(int64_t)i * ldt + f] = atan2(num, den);
    }
}

// parent: per dihedral the parent dihedral (0-based) or -1.
__global__ void __launch_bounds__(kPhaseThreads) bat_phase_kernel(double *__restrict__ dtmp, int64_t ldt, int nf,
                                                                  int nd, const int *__restrict__ parent,
                                                                  void *dih, int64_t ld, int64_t f0, int prec,
                                                                  double pi) {
    const int f = blockIdx.x * kPhaseThreads + threadIdx.x;
    if (f >= nf) return;
    for (int i = 0; i < nd; i++) {  // :303-310, in place and in order
        const int p = __ldg(parent + i);
        if (p >= 0) dtmp[(int64_t)i * ldt + f] -= dtmp[(int64_t)p * ldt + f];
    }
    for (int i = 0; i < nd; i++) {  // :209-214
        const double d = dtmp[(int64_t)i * ldt + f];
        const double t = d + 2 * pi;
        const double s = t - (double)((int)(t / (2 * pi)) * 2) * pi;
        put(dih, prec, (int64_t)i * ld + f0 + f, s);
    }
}

}  // namespace

cudaError_t launch_cart_transpose(const float *aos, int nf, int n_atoms, float *soa, int64_t lds, cudaStream_t st) {
    if (nf <= 0) return cudaSuccess;
    const int ncols = 3 * n_atoms;
    const dim3 block(32, 8), grid((ncols + 31) / 32, (nf + 31) / 32);
    if (grid.y > 65535u) return cudaErrorInvalidValue;
    cart_transpose_kernel<<<grid, block, 0, st>>>(aos, nf, ncols, soa, lds);
    return cudaGetLastError();
}

cudaError_t launch_bat_convert(const float *soa, int64_t lds, int nf, int nd, const int4 *atoms, void *bonds,
                               void *angles, int64_t ld, int64_t f0, int prec, double *dtmp, int64_t ldt,
                               cudaStream_t st) {
    if (nf <= 0 || nd <= 0) return cudaSuccess;
    const dim3 grid((nf + kConvThreads - 1) / kConvThreads, (nd + kDihPerRow - 1) / kDihPerRow);
    if (grid.y > 65535u) return cudaErrorInvalidValue;
    bat_convert_kernel<<<grid, kConvThreads, 0, st>>>(soa, lds, nf, nd, atoms, bonds, angles, ld, f0, prec, dtmp, ldt);
    return cudaGetLastError();
}

cudaError_t launch_bat_phase(double *dtmp, int64_t ldt, int nf, int nd, const int *parent, void *dih, int64_t ld,
                             int64_t f0, int prec, cudaStream_t st) {
    if (nf <= 0 || nd <= 0) return cudaSuccess;
    bat_phase_kernel<<<(nf + kPhaseThreads - 1) / kPhaseThreads, kPhaseThreads, 0, st>>>(
        dtmp, ldt, nf, nd, parent, dih, ld, f0, prec, acos(-1.0));  // pi as the reference defines it (:51)
    return cudaGetLastError();
}

}  // namespace pg
