/*
 * parent_gb300 — C ABI of the GB300 (sm_103a) engine for PARENT's hot path:
 * all-pairs 2D-histogram entropies / mutual information over the bond, angle
 * and dihedral degrees of freedom (DOFs) of a BAT trajectory, and the MIST
 * maximum spanning tree over the resulting MI matrix.
 *
 * The reference (markusfleck/PARENT) exposes this path as processes and files:
 *   PARENT.x in.bat out.par b1D a1D d1D b2D a2D d2D   (src/PARENT/PARENT.cpp:190-244)
 *   get_PAR_MIST.x in.par out.txt                     (src/process_output/get_PAR_MIST.cpp:74-77)
 *   get_PAR_MIE.x in.par, get_PAR_info.x in.par       (src/process_output/get_PAR_MIE.cpp:91, get_PAR_info.cpp:46)
 * and the io library src/util/io/io_binary.h:42-52. Each entry point below
 * names the reference code it replaces. The CLIs in parent_gb300/cli/ are
 * drop-ins for those programs and are built on this ABI.
 *
 * Conventions (mirroring the reference's int-return io library,
 * io_binary.cpp:101,199,602,643): every function returns a pg_status; 0 is
 * success. No C++ exception crosses this boundary. The caller owns every host
 * buffer it passes; the library owns device memory it allocates. One context
 * per host thread; calls on one context are serialised on its CUDA stream.
 *
 * DOF numbering: nBonds = nDih + 2, nAngles = nDih + 1 (PARENT.cpp:298-299).
 * Global DOF index g: bonds [0, nB), angles [nB, nB+nA), dihedrals after.
 */
#ifndef PARENT_GB300_H
#define PARENT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define PG_API __attribute__((visibility("default")))
#else
#define PG_API
#endif

typedef enum pg_status {
    PG_OK = 0,
    PG_ERR_ARG = 1,     /* bad argument (reference: usage message + MPI_Abort) */
    PG_ERR_IO = 2,      /* open/read/write failure (reference: fstream failbit) */
    PG_ERR_FORMAT = 3,  /* corrupted header (io_binary.cpp:127-145, :477-519, :558-591) */
    PG_ERR_DATA = 4,    /* value outside the reference's valid domain: negative bond
                           (PARENT.cpp:522-525) or a bin index outside [0,B) */
    PG_ERR_CUDA = 5,    /* CUDA runtime error */
    PG_ERR_NOMEM = 6,   /* allocation failure (reference: "ERROR ALLOCATNG MEMORY") */
    PG_ERR_TIMEOUT = 7, /* a bounded device-side wait ran out (status read back, context kept) */
    PG_ERR_UNSUPPORTED = 8
} pg_status;

/* Which pair-count kernel computes the 2D histograms. */
typedef enum pg_form {
    PG_FORM_AUTO = 0,   /* autotuner picks per (bins, frames, DOFs) */
    PG_FORM_HIST = 1,   /* shared-memory histogram kernel (TMA-staged bins, smem atomics) */
    PG_FORM_ONEHOT = 2  /* tcgen05 one-hot GEMM kernel (FP8 0/1 operands, FP32 TMEM accumulate) */
} pg_form;

typedef struct pg_ctx pg_ctx;

/* Trajectory columns, DOF-major: column k of a block starts at base + k*ld
 * elements and holds n_frames values. double_prec=1 -> double, 0 -> float
 * (FP32 values are promoted to double before any arithmetic, as
 * read_BAT_frame does, io_binary.cpp:322-364). on_device=1 -> pointers are
 * device pointers on the context's device. */
typedef struct pg_bat_view {
    int n_dihedrals;
    int n_frames;
    int double_prec;
    int on_device;
    int64_t ld; /* elements between consecutive DOF columns (>= n_frames) */
    const void *bonds;
    const void *angles;
    const void *dihedrals;
} pg_bat_view;

/* Entropy results in the exact .par body layout (write_PAR_body,
 * io_binary.cpp:606-631): same-type blocks bb/aa/dd store pair #(P-1-k) at
 * element k, i.e. reverse lexicographic order (PARENT.cpp:1107-1112);
 * ba/bd/ad are row-major with the bond (resp. angle) index slow.
 * Pointers owned by the caller, to host memory or to device memory of the
 * context's GPU (the copies take their direction from the pointers); sizes
 * nB, nA, nD, nB(nB-1)/2, nB*nA, nB*nD, nA(nA-1)/2, nA*nD, nD(nD-1)/2
 * doubles. */
typedef struct pg_par_body {
    double *s1_b, *s1_a, *s1_d;
    double *bb, *ba, *bd, *aa, *ad, *dd;
} pg_par_body;

/* One MIST edge as get_PAR_MIST.cpp:667 prints it: In type, Out type
 * (0=b,1=a,2=d), 1-based In/Out DOF indices within their type, MI, and the
 * number of DOFs still outside the tree before this edge's Out DOF joined. */
typedef struct pg_mist_edge {
    int type_in, type_out;
    int index_in, index_out;
    double mi;
    int left;
    int pad_;
} pg_mist_edge;

/* ---------------------------------------------------------------- context */

/* Creates a context on CUDA device `device` with its own stream.
 * Replaces the MPI_Init_thread/rank set-up of PARENT.cpp:131-145. */
PG_API int pg_create(pg_ctx **out, int device);
PG_API void pg_destroy(pg_ctx *ctx);
/* Message of the last failing call on this context ("" if none). */
PG_API const char *pg_last_error(const pg_ctx *ctx);
/* Message of the last failing call that had no context (pg_create, file I/O). */
PG_API const char *pg_last_global_error(void);

/* --------------------------------------------------------- entropy engine */

/* The PARENT.x computation (PARENT.cpp:443-1493 minus the file I/O): per-DOF
 * extrema and dihedral shift, 1D entropies, every pair's 2D entropy, written
 * into `out` in .par body layout. bins = {b1D, a1D, d1D, b2D, a2D, d2D}
 * (the CLI order of PARENT.cpp:211-234); every bin count >= 1, 2D bin counts
 * <= PG_MAX_BINS_2D. The MI matrix stays resident on the device for pg_mist.
 * `out` may be NULL (results kept on the device only). */
#define PG_MAX_BINS_2D 218
PG_API int pg_entropy(pg_ctx *ctx, const pg_bat_view *traj, const int bins[6], int form,
                      pg_par_body *out);

/* Uploads the columns of a host view ahead of the pg_entropy call that will
 * read them: the copy engine moves them into a standby device buffer while
 * the current call's kernels run, and the next pg_entropy (or
 * pg_entropy_shard) of the same view (every field equal) uses them instead of
 * uploading; a call with another view drops the prefetch. Returns once the
 * copies are queued; the host columns must stay unchanged (and, for the
 * copies to run asynchronously, in pinned memory) until that call. Replaces
 * nothing in the reference: the master's per-run read of the next .bat
 * (PARENT.cpp:443-473) is the step it overlaps. */
PG_API int pg_prefetch(pg_ctx *ctx, const pg_bat_view *traj);

/* pg_entropy of `traj` that, once traj's own columns are on the device,
 * queues the upload of `next` (a host view, or NULL) on the copy engine, so
 * it runs while this call's kernels do; the following call on `next`
 * (pg_entropy or pg_entropy_ahead) takes the uploaded columns. The way to
 * overlap a loop over trajectories: call i passes trajectory i + 1 as next.
 * The host columns of `next` must stay unchanged until that call. */
PG_API int pg_entropy_ahead(pg_ctx *ctx, const pg_bat_view *traj, const int bins[6], int form,
                            pg_par_body *out, const pg_bat_view *next);

/* MIST (get_PAR_MIST.cpp:272-766). If body != NULL the MI values are formed
 * from it exactly as get_mutual (util.cpp:47-81) does; if body == NULL the MI
 * matrix resident from the last pg_entropy on this context is used.
 * edges: nB+nA+nD-1 entries; totals[10] in get_PAR_MIST.cpp:756-765 order. */
PG_API int pg_mist(pg_ctx *ctx, int n_dihedrals, const pg_par_body *body, pg_mist_edge *edges,
                   double totals[10]);

/* MIST that allocates nothing. It has no counterpart in the reference; it
 * exists for callers that cannot call cudaMalloc, such as a host program that
 * owns the whole device memory budget in its own pre-allocated pool, or one
 * that cannot accept the device-wide synchronisation an allocation or free
 * may cause while its other streams run.
 * mi: caller's device buffer, dense symmetric D x D FP64 MI matrix (D =
 * 3*n_dihedrals+3, global DOF order bonds|angles|dihedrals, diagonal unused);
 * edge_mi / edge_from / edge_to: caller's device buffers of D-1 entries,
 * filled with step k's MI, In DOF and Out DOF (global indices), in the order
 * pg_mist produces them. stream: a cudaStream_t (NULL = default stream); the
 * call only enqueues, results are ready when the stream reaches them.
 * D must not exceed PG_NOALLOC_MAX_DOFS (PG_ERR_UNSUPPORTED otherwise). The
 * per-DOF scratch of the one-CTA kernel, when it runs on more DOFs than its
 * shared memory holds (above 12,800 DOFs with PG_MIST_CLUSTER=0), is one
 * static device array per GPU (16 bytes x PG_NOALLOC_MAX_DOFS, held until
 * exit) shared by every call: such calls that overlap on the GPU race on it
 * and must be serialised by the caller. The other kernels keep their
 * per-DOF arrays in shared memory. Every call looks up that array's address
 * with the current device (after a device reset too); the first call on a
 * device may also load the library's device code, so make it before any
 * stream capture. */
#define PG_NOALLOC_MAX_DOFS 16384
PG_API int pg_mist_noalloc(int n_dihedrals, const double *mi, double *edge_mi, int *edge_from,
                           int *edge_to, void *stream);

/* One shard of the pair work of one trajectory, for splitting a system over
 * several GPUs (the reference splits DOF blocks over MPI ranks,
 * PARENT.cpp:333-414, 775-1119). The histogram form's tile list is cut into
 * n_shards contiguous ranges of equal tile count; every shard preprocesses all
 * DOFs, computes the 2D entropies of its own pairs and writes them into `out`
 * (.par body layout) with zeros everywhere else; shard 0 also writes the 1D
 * entropies. The element-wise sum of the n_shards bodies (any order: every
 * entry is non-zero in at most one shard, so the FP64 sum is exact) is the
 * pg_entropy body. MIST then runs on the merged body (pg_mist with body). */
PG_API int pg_entropy_shard(pg_ctx *ctx, const pg_bat_view *traj, const int bins[6], int form, int shard,
                            int n_shards, pg_par_body *out);
/* Which .par body entries shard `shard` of `n_shards` writes (1) for a system
 * of n_dihedrals and these bin counts: mask[total body length], body order.
 * Host only; no context or GPU needed. */
PG_API int pg_shard_mask(int n_dihedrals, const int bins[6], int shard, int n_shards, uint8_t *mask);

/* Many independent trajectories in one run (no reference counterpart: the
 * reference handles one trajectory per PARENT.x / get_PAR_MIST.x process).
 * Every system gets the PARENT.x computation and its MIST tree; the pair
 * histograms of all systems run in ONE launch over the concatenated tile
 * list, the trees in one launch (one CTA per system), and the whole device
 * sequence is captured once into a CUDA graph that later calls with the same
 * geometry replay. outs (n_sys bodies), edges (n_sys arrays of D_s-1) and
 * totals (10 per system) may each be NULL. One form for the whole batch:
 * PG_FORM_HIST, PG_FORM_ONEHOT (every system's tensor-core tiles in one
 * launch, tiles naming their system; PG_ERR_UNSUPPORTED if a system's bins
 * or frames are outside the one-hot form's range), or PG_FORM_AUTO (the
 * one-hot form where the autotuner picks it for every system). */
PG_API int pg_entropy_batch(pg_ctx *ctx, int n_sys, const pg_bat_view *trajs, const int bins[6], int form,
                            pg_par_body *outs, pg_mist_edge *const *edges, double *totals);

/* Device milliseconds of the kernels of the last pg_entropy / pg_mist call,
 * measured with CUDA events on the context's stream:
 * ms[0] = preprocessing (extrema, modfit, binning, 1D), ms[1] = pair kernel,
 * ms[2] = MIST kernel, ms[3] = host<->device copies, ms[4] = whole call. */
PG_API int pg_last_timings(const pg_ctx *ctx, double ms[5]);
/* The autotuner's prediction (no reference counterpart) of the pair-kernel
 * milliseconds of a system of n_dihedrals / n_frames at these bins in a form
 * (PG_FORM_HIST with the histogram layout the library picks, PG_FORM_ONEHOT,
 * or PG_FORM_AUTO: the form the autotuner picks). The model is ceil(tiles /
 * concurrent tiles) x (t0 + t1 F) plus the form's per-call set-up, with t0,
 * t1 and the set-up measured on this GPU by short probe launches the first
 * time a kernel variant is needed (random bins, one full wave, F = 4,096 and
 * 32,768). PG_ERR_UNSUPPORTED if the form cannot run the geometry. */
PG_API int pg_predict_pair_ms(pg_ctx *ctx, int n_dihedrals, int n_frames, const int bins[6], int form,
                              double *ms);
/* Kernel launches issued by this context since creation. */
PG_API int64_t pg_launch_count(const pg_ctx *ctx);
/* Form used by the last pg_entropy (PG_FORM_HIST or PG_FORM_ONEHOT). */
PG_API int pg_last_form(const pg_ctx *ctx);
/* The context's CUDA stream (a cudaStream_t), for event timing by callers. */
PG_API void *pg_stream(const pg_ctx *ctx);

/* Debug/parity export: runs the same preprocessing and pair-histogram kernel
 * as pg_entropy for n_pairs explicit pairs (g1[k] < g2[k], global DOF
 * indices) and copies their 2D counts (row-major, B(g1) x B(g2), int64) to
 * counts + k*stride. The reference never exposes counts; this replaces
 * nothing and exists so counts can be compared bit-exactly. */
PG_API int pg_pair_counts(pg_ctx *ctx, const pg_bat_view *traj, const int bins[6], int form,
                          int n_pairs, const int *g1, const int *g2, int64_t *counts,
                          int64_t stride);

/* Per-DOF preprocessing results of the last pg_entropy (host arrays of D):
 * min, max (after padding/clamps, PARENT.cpp:526-533,551-559,624-634) and
 * the dihedral shift modFit (PARENT.cpp:609; 0 for bonds/angles). */
PG_API int pg_dof_stats(pg_ctx *ctx, double *mn, double *mx, double *shift);

/* Cartesian -> BAT on the device, as BAT_builder converts an .xtc frame by
 * frame (BAT_trajectory.cpp:114-125: coordinates x10 into Angstrom,
 * convert_to_BAT :219-300, phase angles :303-310, shift into [0, 2 pi)
 * :209-214). xyz: n_frames x (n_dihedrals + 3) x 3 floats in nm, frame-major
 * as read_xtc returns them (host memory, or device memory when
 * xyz_on_device = 1); dih: n_dihedrals x 6 ints as in the .bat header
 * (atoms 1-based, [4] the type, [5] the parent dihedral 1-based or -1).
 * *out receives a device view of the BAT columns (FP64 for double_prec = 1,
 * else FP32, the values a .bat of that precision holds), owned by the
 * context and valid until the next conversion or pg_destroy; pass it to
 * pg_entropy. Bonds are bit-identical to BAT_builder's; angles and dihedrals
 * use CUDA's acos/atan2 and can differ in the last place. */
PG_API int pg_bat_from_cartesian(pg_ctx *ctx, const float *xyz, int xyz_on_device, int n_frames, int n_dihedrals,
                                 const int *dih, int double_prec, pg_bat_view *out);

/* ------------------------------------------------------------ file formats */

/* Opaque .bat contents: header (atoms, dihedral table, masses) and DOF-major
 * FP64 or FP32 columns in pinned host memory. Replaces read_BAT_header +
 * read_BAT_frame (io_binary.cpp:107-200, :281-368) and PARENT's frame-major
 * to DOF-major scatter (PARENT.cpp:443-473). */
typedef struct pg_bat pg_bat;
PG_API int pg_bat_read(const char *path, pg_bat **out);
/* Same file, same checks and messages, but the columns end up in device
 * memory on `device` (owned by the pg_bat, freed by pg_bat_free): the frame
 * records are read in large chunks by several threads into pinned buffers,
 * copied up unchanged and transposed by a kernel while the next chunk is
 * read. The view (pg_bat_view_of) then has on_device = 1 and ld = n_frames
 * rounded up to 32. */
PG_API int pg_bat_read_device(const char *path, int device, pg_bat **out);
PG_API void pg_bat_free(pg_bat *bat);
PG_API int pg_bat_view_of(const pg_bat *bat, pg_bat_view *view);
PG_API int pg_bat_n_dihedrals(const pg_bat *bat);
/* The header's dihedral table (nDih x 6 ints: atoms 1-based, type, parent
 * dihedral 1-based or -1; read_BAT_header, io_binary.cpp:178-191), e.g. for
 * pg_bat_from_cartesian on new coordinates of the same system. */
PG_API int pg_bat_dihedral_table(const pg_bat *bat, int *dih);
PG_API int pg_bat_n_frames(const pg_bat *bat);

/* Writes a .bat (version 3) from DOF-major host columns with a synthetic
 * linear-chain header (write_BAT_header / write_BAT_frame,
 * io_binary.cpp:43-102, :203-278). Used for synthetic trajectories. */
PG_API int pg_bat_write_synthetic(const char *path, const pg_bat_view *traj);

/* Writes a .par: header from `bat` (write_PAR_header, io_binary.cpp:371-442,
 * version 4) and body (write_PAR_body, :606-631). Byte-compatible with the
 * reference's read_PAR_header/read_PAR_body. */
PG_API int pg_par_write(const char *path, const pg_bat *bat, const int bins[6],
                        const pg_par_body *body);

/* Opaque .par contents (read_PAR_header + read_PAR_body, io_binary.cpp:446-673). */
typedef struct pg_par pg_par;
PG_API int pg_par_read(const char *path, pg_par **out);
PG_API void pg_par_free(pg_par *par);
PG_API int pg_par_n_dihedrals(const pg_par *par);
PG_API int pg_par_body_of(const pg_par *par, pg_par_body *body);
PG_API int pg_par_bins(const pg_par *par, int bins[6]);

/* Text outputs, byte-identical to the reference programs' stdout/file:
 * get_PAR_MIE.cpp:109-199 (MIE), get_PAR_MIST.cpp:667-765 (MIST),
 * get_PAR_info.cpp:64-79 (topology). path NULL -> stdout. */
PG_API int pg_write_mie_text(const char *path, int n_dihedrals, const pg_par_body *body);
/* The same text, byte for byte, with the ~n^2/2 pair lines formatted on the
 * context's GPU (one thread per line, %.12g in exact 128-bit integer
 * arithmetic) and streamed back in order; the 1D lines and the totals (summed
 * in the reference's line order) stay on the host. */
PG_API int pg_write_mie_text_device(pg_ctx *ctx, const char *path, int n_dihedrals, const pg_par_body *body);
/* printf("%.12g") of v into out (>= 32 bytes, NUL-terminated) by the exact
 * formatter the device text writer uses (the C library's where that
 * formatter's range ends); returns the length. Exported for verification. */
PG_API int pg_format_g12(double v, char *out);
PG_API int pg_write_mist_text(const char *path, int n_dihedrals, const pg_mist_edge *edges,
                              const double totals[10]);
PG_API int pg_write_info_text(const char *path, const pg_par *par);

/* ------------------------------------------------------ synthetic workload */

/* Seeded synthetic linear-chain trajectory (n_atoms atoms -> nDih = n_atoms-3)
 * written DOF-major into caller buffers (host: pg_synth_host, device:
 * pg_synth_device on ctx's device). Bonds ~ Normal(0.15, 0.005), angles ~
 * von Mises(1.91, 40) clipped inside (0, pi), dihedrals ~ mixture of 1-3
 * von Mises modes wrapped to [0, 2pi), correlated through n_latents AR(1)
 * latents (phi = 0.95) mixed with Normal(0, 0.3) weights.
 * frac_bimodal_dih / frac_bimodal_bond: fraction of dihedrals (bonds) whose
 * mode follows a two-state Markov chain with switch probability p_switch. */
typedef struct pg_synth_spec {
    int n_atoms;
    int n_frames;
    int double_prec;
    int n_latents;
    uint64_t seed;
    double frac_bimodal_dih;
    double frac_bimodal_bond;
    double p_switch;
} pg_synth_spec;
PG_API int pg_synth_host(const pg_synth_spec *spec, void *bonds, void *angles, void *dihedrals,
                         int64_t ld, int n_threads);
PG_API int pg_synth_device(pg_ctx *ctx, const pg_synth_spec *spec, void *bonds, void *angles,
                           void *dihedrals, int64_t ld);

/* Roofline probe (no reference counterpart): rate of warp-wide shared-memory
 * reductions with every lane on its own bank, over all SMs of the context's
 * device. It is the peak the histogram pair kernel is measured against. */
PG_API int pg_probe_smem_red_rate(pg_ctx *ctx, double *reductions_per_s);

/* Failure detection check: runs a kernel whose bounded mbarrier wait (the
 * helper every pair kernel uses) is completed by nobody, with a limit of
 * limit_ms. Returns PG_ERR_TIMEOUT, recorded on the device and read back as
 * for a real timeout; the context stays usable. */
PG_API int pg_check_wait_timeout(pg_ctx *ctx, double limit_ms);

/* ------------------------------------------------------ device memory */

/* Device allocations owned by the caller through the library (so callers
 * need no CUDA runtime of their own). */
PG_API int pg_device_alloc(pg_ctx *ctx, size_t bytes, void **ptr);
PG_API int pg_device_free(pg_ctx *ctx, void *ptr);
PG_API int pg_memcpy(pg_ctx *ctx, void *dst, const void *src, size_t bytes, int kind /* 1 H2D, 2 D2H, 3 D2D */);
PG_API int pg_host_alloc_pinned(size_t bytes, void **ptr);
PG_API int pg_host_free_pinned(void *ptr);
PG_API int pg_synchronize(pg_ctx *ctx);

#ifdef __cplusplus
}
#endif
#endif
