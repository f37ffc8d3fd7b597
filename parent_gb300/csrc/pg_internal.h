// Internal declarations shared by the parent_gb300 CUDA translation units and
// the host orchestration (pg_api.cu). Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <vector>

namespace pg {

// DOF type codes (reference util.h:33-35).
enum { TB = 0, TA = 1, TD = 2 };

// Device-side error words, zeroed before each run and read back after it.
enum {
    ERR_BIN_RANGE = 0,    // a bin index fell outside [0, B) (reference: UB)
    ERR_NEG_BOND = 1,     // a bond value < 0 (reference aborts, PARENT.cpp:522-525)
    ERR_MODFIT_RANGE = 2, // a dihedral outside the modfit histogram (PARENT.cpp:571, UB)
    ERR_TIMEOUT = 3,      // a bounded mbarrier / flag wait ran out
    ERR_WORDS = 4
};

// Geometry of one system (one trajectory).
struct SysGeom {
    int n_dih, nb, na, nd, D;  // D = nb + na + nd
    int F;                     // frames
    int64_t ldb;               // bytes between DOF rows of the uint8 bin matrix (bins_ld(F))
    int bins[6];               // b1D a1D d1D b2D a2D d2D
    int codes;                 // 1: a second matrix follows the bin matrix, holding
                               // each 2D bin b as the row code (b >> 1) | (b & 1) << 7
    int ilv;                   // 1: both matrices are frame-group interleaved (ilv_index)
                               // instead of DOF rows ldb bytes apart
};

// Frame-group interleaved bin layout (SysGeom::ilv), read by the streamed
// 32-slot histogram kernel. Frames go in groups of 16 and DOFs in blocks of
// 8; block k holds, for every group in frame order, the 16 bytes of each of
// its 8 DOFs (128 bytes per group): DOF g, frame f at
//   ((g / 8) * G + f / 16) * 128 + (g % 8) * 16 + f % 16,  G = ilv_groups(F).
// A tile's 8 column DOFs (a block) are then one 128-byte line per group and
// its 4 row DOFs half of one, and consecutive groups of a DOF are 128 bytes
// apart, so a warp streams its groups at small constant offsets. D is padded
// to a multiple of 8.
__host__ __device__ inline int64_t ilv_dp(int D) { return ((int64_t)D + 7) / 8 * 8; }
__host__ __device__ inline int64_t ilv_groups(int F) { return ((int64_t)F + 15) / 16; }
__host__ __device__ inline int64_t ilv_bytes(int D, int F) { return ilv_groups(F) * ilv_dp(D) * 16; }
// byte offset of DOF g's first group
__host__ __device__ inline int64_t ilv_dof_base(int F, int g) {
    return (int64_t)(g >> 3) * ilv_groups(F) * 128 + (g & 7) * 16;
}
// byte offset of (DOF g, frame f) from that base
__host__ __device__ inline int64_t ilv_frame_off(int f) { return ((int64_t)(f >> 4) << 7) + (f & 15); }
__host__ __device__ inline int64_t ilv_index(int F, int g, int f) { return ilv_dof_base(F, g) + ilv_frame_off(f); }

// Bytes of the bin matrix (and the row-code matrix after it, if any).
inline size_t bins_bytes(const SysGeom &g) {
    const size_t one = g.ilv ? (size_t)ilv_bytes(g.D, g.F) : (size_t)g.D * (size_t)g.ldb;
    return one * (g.codes ? 2 : 1);
}

// Stores 2D bin b of DOF d, frame f in every matrix of g's layout.
__host__ __device__ inline void store_bin(uint8_t *bins, const SysGeom &g, int d, int f, int b) {
    const int64_t at = g.ilv ? ilv_index(g.F, d, f) : (int64_t)d * g.ldb + f;
    bins[at] = (uint8_t)b;
    // row codes for the 16-bit 32-slot layouts: (b >> 1) | (b & 1) << 7
    if (g.codes) bins[(g.ilv ? ilv_bytes(g.D, g.F) : (int64_t)g.D * g.ldb) + at] = (uint8_t)((b >> 1) | ((b & 1) << 7));
}

// Stores the 2D bins b[0..N) of DOF d, frames f0..f0+N-1 (N = 2 or 4, f0 a
// multiple of N: the run lies in one DOF row or one 16-frame group, on an
// N-byte boundary) with one store per matrix.
template <int N>
__device__ inline void store_bin_run(uint8_t *bins, const SysGeom &g, int d, int f0, const int *b) {
    const int64_t at = g.ilv ? ilv_index(g.F, d, f0) : (int64_t)d * g.ldb + f0;
    uint32_t w = 0, c = 0;
#pragma unroll
    for (int k = 0; k < N; k++) {
        w |= (uint32_t)b[k] << (8 * k);
        c |= (uint32_t)((b[k] >> 1) | ((b[k] & 1) << 7)) << (8 * k);
    }
    uint8_t *cm = bins + (g.ilv ? ilv_bytes(g.D, g.F) : (int64_t)g.D * g.ldb);
    if (N == 4) {
        *(uint32_t *)(bins + at) = w;
        if (g.codes) *(uint32_t *)(cm + at) = c;
    } else {
        *(uint16_t *)(bins + at) = (uint16_t)w;
        if (g.codes) *(uint16_t *)(cm + at) = (uint16_t)c;
    }
}

// largest 2D bin count of a geometry's DOF types
inline int bmax2d(const SysGeom &g) {
    const int a = g.bins[3] > g.bins[4] ? g.bins[3] : g.bins[4];
    return a > g.bins[5] ? a : g.bins[5];
}

__host__ __device__ inline int dof_type(int g, int nb, int na) {
    return g < nb ? TB : (g < nb + na ? TA : TD);
}

// Per-DOF arrays produced by the preprocessing kernel (structure of arrays,
// each D long, all in one device allocation).
struct DofArrays {
    double *mn, *mx, *shift; // extrema after padding/clamps; dihedral modFit
    double *s1;              // 1D entropy (PARENT.cpp:650-757)
    double *acon;            // ln(binsize_2D) + (1/N) sum_k m(k) ln J(k), the
                             // per-DOF constant of the 2D entropy decomposition
    int *b2;                 // 2D bin count of the DOF's type
    int *m2;                 // largest marginal count over the DOF's 2D bins
};

// One system's DofArrays in one allocation of dof_bytes(D) bytes at base
inline size_t dof_bytes(int D) { return (size_t)D * (5 * sizeof(double) + 2 * sizeof(int)) + 64; }
inline DofArrays dof_at(void *base, int D) {
    DofArrays d;
    double *b = (double *)base;
    d.mn = b;
    d.mx = b + D;
    d.shift = b + 2 * (size_t)D;
    d.s1 = b + 3 * (size_t)D;
    d.acon = b + 4 * (size_t)D;
    d.b2 = (int *)(b + 5 * (size_t)D);
    d.m2 = d.b2 + D;
    return d;
}

// Offsets of the nine .par body blocks inside one contiguous double buffer.
struct ParLayout {
    int64_t s1b, s1a, s1d, bb, ba, bd, aa, ad, dd, total;
};
ParLayout par_layout(int n_dih);

// Where the pair (g1 < g2) lands in the .par body (PARENT.cpp:896-898,
// 1107-1112; reader util.cpp:55,67,76).
__host__ __device__ inline int64_t par_pair_index(const ParLayout &L, int nb, int na, int nd,
                                                  int g1, int g2) {
    const int t1 = dof_type(g1, nb, na), t2 = dof_type(g2, nb, na);
    const int i1 = g1 - (t1 == TB ? 0 : (t1 == TA ? nb : nb + na));
    const int i2 = g2 - (t2 == TB ? 0 : (t2 == TA ? nb : nb + na));
    if (t1 == t2) {
        const int n = t1 == TB ? nb : (t1 == TA ? na : nd);
        const int64_t base = t1 == TB ? L.bb : (t1 == TA ? L.aa : L.dd);
        return base + (int64_t)(n - i1) * (n - i1 - 1) / 2 + i1 - i2;
    }
    if (t1 == TB && t2 == TA) return L.ba + (int64_t)i1 * na + i2;
    if (t1 == TB) return L.bd + (int64_t)i1 * nd + i2;
    return L.ad + (int64_t)i1 * nd + i2;
}

// A pair tile: row DOFs [row0, row0+nrow), column DOFs [col0, col0+ncol);
// pair (r, c) is valid when r < c.
struct PairTile {
    int row0, col0;
    int nrow, ncol;
};

// ---------------------------------------------------------------- launchers
// All launchers enqueue on `st` and return cudaGetLastError().

// nlogn[n] = n ln n for n in [0, nmax] (FP64).
cudaError_t launch_nlogn_table(double *nlogn, int nmax, cudaStream_t st);
// nfix[n] = round(n ln n * fix) for n in [0, nmax], fix = nlogn_fix_scale(F)
// for some F >= nmax (fixed point, so sums are exact integer additions).
cudaError_t launch_nlogn_fix_table(unsigned long long *nfix, int nmax, double fix, cudaStream_t st);

// Extrema + modfit + binning + 1D entropies + 2D decomposition constants for
// DOFs [g_first, g_first + g_count) (g_count < 0: through the last DOF).
// cols[t] = device base of the type-t block (columns ld elements apart).
cudaError_t launch_prep(const SysGeom &g, const void *const cols[3], int64_t ld, int double_prec,
                        DofArrays dof, uint8_t *bins, int *err, cudaStream_t st, int g_first = 0,
                        int g_count = -1);
// One system's preprocessing inputs and outputs, for batched launches.
struct PrepDesc {
    SysGeom geo;
    const void *cols[3];
    int64_t ld;
    int prec;
    DofArrays dof;
    uint8_t *bins;
};
// Preprocessing of many systems in one launch: CTA k handles DOF map[k].y of
// system map[k].x; all systems have the input precision double_prec and the
// bin counts of bins_of.
cudaError_t launch_prep_batch(const SysGeom &bins_of, const PrepDesc *sys, const int2 *map, int n_cta,
                              int double_prec, int *err, cudaStream_t st);

// Shared-memory histogram pair kernel with fused entropy/MI epilogue.
// If counts != nullptr the raw 2D histograms of each tile's first pair slots
// are dumped (debug export) instead of the .par/MI outputs.
struct PairOut {
    double *par;        // .par body on device
    double *mi;         // D x D dense MI (may be nullptr)
    ParLayout L;
    int64_t *counts;    // debug dump, per tile: 16 pair slots x Bmax^2 (nullptr normally)
    int counts_bmax;
};
// One system of a batch, as the batched kernels read it.
struct SysDesc {
    SysGeom geo;
    const uint8_t *bins;
    DofArrays dof;
    PairOut out;
    double lnN;
};

// Row pitch of the uint8 bin matrix: a multiple of 4096 with at least 4096
// bytes past the last frame, so a pair kernel's last chunk (any chunk size up
// to 4096 frames) stays inside its row.
inline int64_t bins_ld(int F) { return ((int64_t)F + 4095) / 4096 * 4096 + 4096; }

// 2^s with s as large as possible (<= 44) such that F ln F * 2^s stays below
// 1.6e19: sums of n ln n over a histogram of F frames, rounded to multiples
// of 2^-s, then fit in 64-bit unsigned integers.
inline double nlogn_fix_scale(int F) {
    const double top = (double)F * log((double)F > 1 ? (double)F : 2.0) + 1.0;
    int s = (int)floor(log2(1.6e19 / top));
    if (s > 44) s = 44;
    return ldexp(1.0, s);
}
cudaError_t launch_pairs_hist_batch(int bmax, const SysDesc *sys, const PairTile *tiles, const int *tile_sys,
                                    int64_t n_tiles, const unsigned long long *nfix, double fix, int *err,
                                    int tile_dim, cudaStream_t st);
cudaError_t launch_pairs_hist(const SysGeom &g, const uint8_t *bins, const DofArrays &dof,
                              const unsigned long long *nfix, double fix, const PairTile *tiles, int64_t n_tiles,
                              int tile_dim, PairOut out, int *err, cudaStream_t st);
// smem bytes the histogram kernel needs for a given max 2D bin count, or 0 if
// it cannot run; sets *tile_dim (4, 2 or 1 DOFs per tile side) and the
// staging geometry (frames per chunk, stages).
int pairs_hist_config(int bmax, int *tile_dim, int *chunk_frames, int *stages);

// 32-slot histogram pair kernel (2D bins <= 50): conflict-free counters over
// 4 x 8-DOF tiles, persistent grid of pairs_hist32_grid(n) CTAs. Geometries
// with the interleaved bin layout (SysGeom::ilv) run the streamed form (rows
// loaded straight from global memory), the others the TMA-ring form. Up to 35
// bins 32-bit counters; 36-50 bins 16-bit counters, which need the row-code
// matrix (SysGeom::codes), and tiles that could overflow a 16-bit counter move
// counts into a per-CTA overflow area in `scratch`
// (pairs_hist32_scratch_bytes, zeroed by the launcher) every 32,768 frames.
bool pairs_hist32_supported(int bmax);
bool pairs_hist32_wide(int bmax);  // 32-bit counters fit (2D bins <= 35)
int pairs_hist32_grid(int64_t n_tiles);
size_t pairs_hist32_scratch_bytes(int bmax, int grid);
cudaError_t launch_pairs_hist32(const SysGeom &g, const uint8_t *bins, const DofArrays &dof,
                                const unsigned long long *nfix, double fix, const PairTile *tiles, int64_t n_tiles,
                                PairOut out, int *err, void *scratch, size_t scratch_bytes, cudaStream_t st);
cudaError_t launch_pairs_hist32_batch(int bmax, bool codes, bool ilv, const SysDesc *sys, const PairTile *tiles,
                                      const int *tile_sys, int64_t n_tiles, const unsigned long long *nfix,
                                      double fix, int *err, void *scratch, size_t scratch_bytes, cudaStream_t st);

// Cartesian -> BAT conversion (pg_batconv.cu): coordinates of a chunk of
// frames to one row per (atom, xyz) scaled by 10; bonds/angles/raw dihedrals;
// phase angles and the [0, 2 pi) shift. Columns ld elements apart, frames f0..
cudaError_t launch_cart_transpose(const float *aos, int nf, int n_atoms, float *soa, int64_t lds, cudaStream_t st);
cudaError_t launch_bat_convert(const float *soa, int64_t lds, int nf, int nd, const int4 *atoms, void *bonds,
                               void *angles, int64_t ld, int64_t f0, int prec, double *dtmp, int64_t ldt,
                               cudaStream_t st);
cudaError_t launch_bat_phase(double *dtmp, int64_t ldt, int nf, int nd, const int *parent, void *dih, int64_t ld,
                             int64_t f0, int prec, cudaStream_t st);

// Host -> device copy by SM loads where the GPU can read the host memory
// (pg_ingest.cu), else by the copy engine.
cudaError_t h2d_copy(void *dst, const void *src, size_t bytes, cudaStream_t st, bool *pulled);
// Host memory this GPU's kernels can read directly: pinned, or pageable where
// the device has pageable memory access (a Grace-attached part).
bool host_readable(const void *src);

// A kernel whose bounded mbarrier wait nothing completes (sets err[ERR_TIMEOUT]).
cudaError_t launch_wait_timeout_probe(long long limit_cycles, int *err, cudaStream_t st);

// MIE text on the device (pg_mie.cu): the six pair blocks of the 2D lines,
// rows of each block in order (row0[q] .. row0[q+1]), lines numbered from
// line0[q]; every line first goes to a 96-byte slot, then the rows are packed.
constexpr int kMieSlot = 96;
struct MieArgs {
    const double *blk[6];          // .par body block of the pair type
    const double *s1r[6], *s1c[6]; // 1D entropies of the row / column DOF type
    int n1[6], n2[6], same[6];
    int64_t line0[6];
    int row0[7];
    int rows;
    char name[6][20];              // "bond-bond " ... "dihedral-dihedral "
    int name_len[6];
    char *slots;
    uint8_t *lens;
    long long *row_len, *row_off;  // rows, rows + 1
    char *text;
    int *fb_count;                 // lines left to the host formatter
    int64_t *fb_list;
    int fb_cap;
};
cudaError_t launch_mie_format(const MieArgs &a, cudaStream_t st);
cudaError_t launch_mie_offsets(const MieArgs &a, cudaStream_t st);   // row_len, row_off (total at [rows])
cudaError_t launch_mie_compact(const MieArgs &a, cudaStream_t st);   // slots -> text

// tcgen05 one-hot pair kernel (same outputs as the histogram kernel).
cudaError_t launch_pairs_onehot(const SysGeom &g, const uint8_t *bins, const DofArrays &dof,
                                const double *nlogn, PairOut out, int *err, cudaStream_t st,
                                void *scratch, size_t scratch_bytes, int *launches);
size_t pairs_onehot_scratch_bytes(const SysGeom &g);
bool pairs_onehot_supported(const SysGeom &g);
// launch_pairs_onehot in two parts: the set-up (synchronous uploads, the
// n ln n table) and the run (accumulators zeroed, pair kernel, finalize),
// which can be repeated on the same inputs (the autotuner's probes time it).
struct OnehotRun {
    void *scratch = nullptr;
    size_t off_sys = 0, off_fin = 0, off_tiles = 0, off_snl = 0, acc_bytes = 0;
    int64_t n_tiles = 0;
    bool pair = true;
    bool low = false;  // every 2D bin count at most 64
    int D = 0;
};
cudaError_t onehot_setup(const SysGeom &g, const uint8_t *bins, const DofArrays &dof, PairOut out, cudaStream_t st,
                         void *scratch, size_t scratch_bytes, OnehotRun *run);
cudaError_t onehot_run(const OnehotRun &run, int *err, cudaStream_t st);
// Many systems in one one-hot launch (each tile names its system; tiles of
// the longest trajectories first): workspace size, tile count, the set-up
// of the descriptors and tables that depend only on the geometries
// (synchronous, outside any graph capture), and the launch itself (zeroes
// the accumulators, pair kernel, one finalize launch over all systems;
// capturable).
size_t pairs_onehot_batch_bytes(const std::vector<SysGeom> &gs);
int64_t pairs_onehot_batch_tiles(const std::vector<SysGeom> &gs);
cudaError_t prepare_pairs_onehot_batch(const std::vector<SysGeom> &gs, const std::vector<const uint8_t *> &bins,
                                       const std::vector<DofArrays> &dofs, const std::vector<PairOut> &outs,
                                       void *ws, size_t ws_bytes, cudaStream_t st);
cudaError_t launch_pairs_onehot_batch(const std::vector<SysGeom> &gs, void *ws, int *err, cudaStream_t st,
                                      int *launches);

// One system of a batched MIST launch (one CTA each); scratch holds
// key[D] | from[D] | pos[D] (mist_scratch_bytes(D)).
struct MistDesc {
    int D, nb, na;
    const double *mi;
    void *scratch;
    double *edge_mi;
    int *edge_from, *edge_to;
};
cudaError_t launch_mist_batch(const MistDesc *sys, int n_sys, int max_D, cudaStream_t st);

// MI matrix from a .par body already on the device (get_mutual semantics).
cudaError_t launch_mi_from_par(int n_dih, const double *par, ParLayout L, double *mi,
                               cudaStream_t st);

std::vector<PairTile> build_tiles32(int D);
// tile count of the one-hot form for a geometry (CTA-pair tiles unless
// PG_ONEHOT_PAIR=0)
int64_t pairs_onehot_tiles(const SysGeom &g);

// Histogram layouts: the 16-slot kernel (two lanes per pair), the 32-slot
// kernel fed by a TMA ring, and the streamed 32-slot kernel (rows loaded
// straight from the frame-group interleaved bin matrix).
enum { HIST16 = 0, HIST32_RING = 1, HIST32_STREAM = 2 };
int hist_layout(const SysGeom &g);
// SysGeom::codes / SysGeom::ilv of a histogram layout at a bin count
int layout_codes(int layout, int bmax);
int layout_ilv(int layout);
// The autotuner (pg_autotune.cu): predicted pair-kernel seconds of a form on
// this GPU (< 0 if unknown), and the form PG_FORM_AUTO takes for one system
// and for a batch run in one launch.
double predict_pair_seconds(const SysGeom &g, int form);
int autotune_form(const SysGeom &g);
int autotune_batch_form(const std::vector<SysGeom> &gs);

}  // namespace pg
