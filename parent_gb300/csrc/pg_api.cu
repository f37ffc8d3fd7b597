// C ABI implementation: context, device buffers, and the orchestration of the
// preprocessing, pair and MIST kernels (host code; kernels live in the other
// translation units).
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <functional>
#include <string>
#include <vector>

#include "../../include/parent_gb300.h"
#include "pg_internal.h"

namespace pg {

size_t prep_smem_bytes(const SysGeom &g);
size_t mist_scratch_bytes(int D);
cudaError_t launch_mist_impl(int D, int nb, int na, const double *mi, void *scratch,
                             double *edge_mi, int *edge_from, int *edge_to, cudaStream_t st);
bool synth_spec_ok(const pg_synth_spec *sp);
size_t synth_scratch_bytes(const pg_synth_spec *sp, size_t *lat_bytes, size_t *sw_bytes,
                           std::vector<float> &lat, std::vector<int> &sw, std::vector<int> &sw_off);
cudaError_t launch_synth_dev(const pg_synth_spec *sp, void *b, void *a, void *d, int64_t ld,
                             const float *lat, const int *sw, const int *sw_off, cudaStream_t st);
void set_global_error(const char *msg);
double probe_smem_red_rate(int n_sm, cudaStream_t st, int *launches);

ParLayout par_layout(int n_dih) {
    const int64_t nb = n_dih + 2, na = n_dih + 1, nd = n_dih;
    ParLayout L;
    L.s1b = 0;
    L.s1a = L.s1b + nb;
    L.s1d = L.s1a + na;
    L.bb = L.s1d + nd;
    L.ba = L.bb + nb * (nb - 1) / 2;
    L.bd = L.ba + nb * na;
    L.aa = L.bd + nb * nd;
    L.ad = L.aa + na * (na - 1) / 2;
    L.dd = L.ad + na * nd;
    L.total = L.dd + nd * (nd - 1) / 2;
    return L;
}

// Tiles of T x T DOFs over the upper triangle of the DOF x DOF grid, in
// super-blocks of 16 x 16 tiles so that CTAs resident at the same time share
// their bin rows in L2.
std::vector<PairTile> build_tiles(int D, int T) {
    const int nblk = (D + T - 1) / T, S = 16, nsb = (nblk + S - 1) / S;
    std::vector<PairTile> t;
    t.reserve((size_t)nblk * (nblk + 1) / 2);
    for (int sc = 0; sc < nsb; sc++)
        for (int sr = 0; sr <= sc; sr++)
            for (int cb = sc * S; cb < std::min(nblk, (sc + 1) * S); cb++)
                for (int rb = sr * S; rb < std::min(nblk, (sr + 1) * S) && rb <= cb; rb++)
                    t.push_back(PairTile{rb * T, cb * T, std::min(T, D - rb * T), std::min(T, D - cb * T)});
    return t;
}

}  // namespace pg

using namespace pg;

namespace {

thread_local std::string g_global_err;

}  // namespace

void pg::set_global_error(const char *msg) { g_global_err = msg; }

namespace {

struct DevBuf {
    void *p = nullptr;
    size_t n = 0;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= n && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        size_t b = std::max<size_t>(bytes, 256);
        cudaError_t e = cudaMalloc(&p, b);
        if (e == cudaSuccess) n = b;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

}  // namespace

struct pg_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[6] = {};
    std::string err;
    DevBuf cols, bins, dofbuf, par, mi, nlogn, tiles, errw, scratch, counts, edges, mistscr;
    int nlogn_max = -1;
    DevBuf nfix;          // fixed-point n ln n table of the histogram kernel
    int nfix_max = -1;
    double nfix_scale = 0.0;
    std::vector<PairTile> tiles_host;
    int tiles_D = -1, tiles_T = -1;
    int64_t launches = 0;
    double timings[5] = {0, 0, 0, 0, 0};
    int last_form = 0;
    bool resident = false;  // MI matrix of the last pg_entropy is valid
    SysGeom geo{};
    // batched runs: one arena for every system's device data, descriptors,
    // and the CUDA graph of the last batch geometry
    DevBuf batch, batchmeta, ohbatch;
    cudaGraphExec_t graph = nullptr;
    std::vector<int64_t> graph_key;
    // host trajectories: uploads run on their own stream, one event per DOF group
    cudaStream_t copy = nullptr;
    // pg_prefetch: the host columns of the next call, uploaded by the copy
    // engine into a standby buffer while the current call computes; the next
    // pg_entropy of the same view swaps it in instead of uploading
    DevBuf cols_pf;
    pg_bat_view pf_view{};
    bool pf_pending = false;
    cudaEvent_t pf_done = nullptr;
    // pg_entropy_ahead: the view whose upload the running call queues once
    // its own columns are in place
    pg_bat_view ahead_view{};
    bool ahead_set = false;
    static constexpr int kMaxGroups = 64;
    cudaEvent_t gev[kMaxGroups] = {};
    // ... and the pair launches of consecutive groups alternate between two
    // streams, so one launch's last wave overlaps the next launch's first
    cudaStream_t pst[2] = {};
    cudaEvent_t pev[kMaxGroups] = {}, pend[2] = {};
    // Cartesian -> BAT: output columns (valid until the next conversion or
    // pg_destroy), per-chunk staging, coordinate rows, FP64 dihedrals, table
    DevBuf bc_out, bc_stage, bc_soa, bc_tmp, bc_tab;
    // MIE text: body, line slots and lengths, row offsets, text, host fallbacks
    DevBuf mie_body, mie_slots, mie_lens, mie_rows, mie_text, mie_fb;
    // pinned host staging for small results (MIST edges, 1D entropies)
    void *hstage = nullptr;
    size_t hstage_n = 0;
    cudaError_t ensure_hstage(size_t bytes) {
        if (bytes <= hstage_n && hstage) return cudaSuccess;
        if (hstage) cudaFreeHost(hstage);
        hstage = nullptr;
        hstage_n = 0;
        const size_t b = std::max<size_t>(bytes, 4096);
        cudaError_t e = cudaHostAlloc(&hstage, b, cudaHostAllocDefault);
        if (e == cudaSuccess) hstage_n = b;
        return e;
    }
};

static int fail(pg_ctx *c, int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (c) c->err = buf; else g_global_err = buf;
    return code;
}

// A failing runtime call also leaves its error as the thread's "last error";
// it is cleared here so that no later launch check reports it again.
#define CK(call)                                                                                     \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess) {                                                                     \
            cudaGetLastError();                                                                      \
            return fail(ctx, e_ == cudaErrorMemoryAllocation ? PG_ERR_NOMEM : PG_ERR_CUDA, "%s: %s", \
                        #call, cudaGetErrorString(e_));                                              \
        }                                                                                            \
    } while (0)

static DofArrays dof_arrays(pg_ctx *ctx, int D) { return dof_at(ctx->dofbuf.p, D); }

static size_t elem_size(int prec) { return prec ? 8 : 4; }

// Validation and the geometry of a trajectory (ctx->geo).
static void set_bin_layout(SysGeom &g, int form);

// form: the form the caller asked for (PG_FORM_AUTO/HIST/ONEHOT); it decides
// the bin-matrix layout the preprocessing writes (set_bin_layout).
static int setup_geometry(pg_ctx *ctx, const pg_bat_view *tv, const int bins[6], int form) {
    if (!tv || !bins) return fail(ctx, PG_ERR_ARG, "null trajectory or bins");
    if (tv->n_dihedrals < 0 || tv->n_frames < 1)
        return fail(ctx, PG_ERR_ARG, "n_dihedrals (%d) < 0 or n_frames (%d) < 1", tv->n_dihedrals, tv->n_frames);
    if (tv->double_prec != 0 && tv->double_prec != 1)
        return fail(ctx, PG_ERR_ARG, "double_prec must be 0 or 1");
    if (tv->ld < tv->n_frames) return fail(ctx, PG_ERR_ARG, "ld < n_frames");
    if (!tv->bonds || !tv->angles || (tv->n_dihedrals > 0 && !tv->dihedrals))
        return fail(ctx, PG_ERR_ARG, "null column pointer");
    for (int k = 0; k < 6; k++) {
        if (bins[k] < 1) return fail(ctx, PG_ERR_ARG, "bin count %d (index %d) < 1", bins[k], k);
        if (k < 3 && bins[k] > 16384) return fail(ctx, PG_ERR_UNSUPPORTED, "1D bin count %d > 16384", bins[k]);
        if (k >= 3 && bins[k] > PG_MAX_BINS_2D)
            return fail(ctx, PG_ERR_UNSUPPORTED, "2D bin count %d > %d", bins[k], PG_MAX_BINS_2D);
    }
    CK(cudaSetDevice(ctx->device));
    SysGeom &g = ctx->geo;
    g.n_dih = tv->n_dihedrals;
    g.nb = g.n_dih + 2;
    g.na = g.n_dih + 1;
    g.nd = g.n_dih;
    g.D = g.nb + g.na + g.nd;
    g.F = tv->n_frames;
    g.ldb = bins_ld(g.F);
    for (int k = 0; k < 6; k++) g.bins[k] = bins[k];
    set_bin_layout(g, form);
    ctx->resident = false;
    return PG_OK;
}

// Shared front half of pg_entropy / pg_pair_counts: validation, upload,
static bool same_view(const pg_bat_view &a, const pg_bat_view &b) {
    return a.n_dihedrals == b.n_dihedrals && a.n_frames == b.n_frames && a.double_prec == b.double_prec &&
           a.on_device == b.on_device && a.ld == b.ld && a.bonds == b.bonds && a.angles == b.angles &&
           a.dihedrals == b.dihedrals;
}

// If pg_prefetch uploaded this host view, its standby buffer becomes the
// column buffer (ctx->cols, columns DOF-major, n_frames apart) once the
// upload is done on `st`; returns whether it did. A prefetch of another view
// is dropped (after its upload ends, so the buffer can be reused).
static cudaError_t take_prefetch(pg_ctx *ctx, const pg_bat_view *tv, cudaStream_t st, bool *taken) {
    *taken = false;
    if (!ctx->pf_pending) return cudaSuccess;
    ctx->pf_pending = false;
    if (!same_view(ctx->pf_view, *tv)) return cudaEventSynchronize(ctx->pf_done);
    std::swap(ctx->cols, ctx->cols_pf);
    *taken = true;
    return cudaStreamWaitEvent(st, ctx->pf_done, 0);
}

// Queues the upload of a host view's columns into the standby buffer on the
// copy stream (copy engine), after the work already on `after` (the stream
// carrying the current call's own upload), for the next call of that view.
static int queue_prefetch(pg_ctx *ctx, const pg_bat_view *traj, cudaStream_t after) {
    if (!traj || traj->on_device) return fail(ctx, PG_ERR_ARG, "prefetch needs a host view");
    if (traj->n_dihedrals < 0 || traj->n_frames < 1 || traj->ld < traj->n_frames)
        return fail(ctx, PG_ERR_ARG, "bad view");
    if (!traj->bonds || !traj->angles || (traj->n_dihedrals > 0 && !traj->dihedrals))
        return fail(ctx, PG_ERR_ARG, "null column pointer");
    if (ctx->pf_pending) CK(cudaEventSynchronize(ctx->pf_done));  // one prefetch at a time
    ctx->pf_pending = false;
    if (!ctx->pf_done) CK(cudaEventCreateWithFlags(&ctx->pf_done, cudaEventDisableTiming));
    const int nd = traj->n_dihedrals, nb = nd + 2, na = nd + 1;
    const size_t es = elem_size(traj->double_prec), F = (size_t)traj->n_frames;
    const size_t blk[3] = {(size_t)nb * F * es, (size_t)na * F * es, (size_t)nd * F * es};
    CK(ctx->cols_pf.ensure(blk[0] + blk[1] + blk[2] + 256));
    // the standby buffer's last reader (an earlier call's kernels) is done,
    // and the current call's own upload goes first
    CK(cudaEventRecord(ctx->ev[5], after));
    CK(cudaStreamWaitEvent(ctx->copy, ctx->ev[5], 0));
    char *dst = (char *)ctx->cols_pf.p;
    const void *src[3] = {traj->bonds, traj->angles, traj->dihedrals};
    const int cnt[3] = {nb, na, nd};
    for (int t = 0; t < 3; t++) {
        if (cnt[t] > 0) {
            // the copy engine, so the upload runs beside the SMs' work
            if ((size_t)traj->ld == F)
                CK(cudaMemcpyAsync(dst, src[t], blk[t], cudaMemcpyHostToDevice, ctx->copy));
            else
                CK(cudaMemcpy2DAsync(dst, F * es, src[t], (size_t)traj->ld * es, F * es, cnt[t],
                                     cudaMemcpyHostToDevice, ctx->copy));
        }
        dst += blk[t];
    }
    CK(cudaEventRecord(ctx->pf_done, ctx->copy));
    ctx->pf_view = *traj;
    ctx->pf_pending = true;
    return PG_OK;
}

// The pending pg_entropy_ahead upload, queued after `after`'s work. It only
// saves time, so a failure to queue it (no memory for the standby buffer,
// say) drops it and leaves the current call alone: the next call uploads.
static int queue_ahead(pg_ctx *ctx, cudaStream_t after) {
    if (!ctx->ahead_set) return PG_OK;
    ctx->ahead_set = false;
    if (queue_prefetch(ctx, &ctx->ahead_view, after) != PG_OK) {
        ctx->pf_pending = false;
        ctx->err.clear();
        cudaGetLastError();
    }
    return PG_OK;
}

// preprocessing. Leaves bins, dof arrays and the nlogn table on the device.
static int run_prep(pg_ctx *ctx, const pg_bat_view *tv, const int bins[6], int form) {
    int rc0 = setup_geometry(ctx, tv, bins, form);
    if (rc0) return rc0;
    const SysGeom &g = ctx->geo;
    const int D = g.D;
    cudaStream_t st = ctx->stream;

    CK(cudaEventRecord(ctx->ev[0], st));
    // columns
    const void *cols[3];
    int64_t ld = tv->ld;
    if (tv->on_device) {
        cols[0] = tv->bonds;
        cols[1] = tv->angles;
        cols[2] = tv->dihedrals ? tv->dihedrals : tv->angles;
    } else {
        const size_t es = elem_size(tv->double_prec);
        ld = tv->n_frames;
        const size_t blk[3] = {(size_t)g.nb * ld * es, (size_t)g.na * ld * es, (size_t)g.nd * ld * es};
        bool pre = false;
        CK(take_prefetch(ctx, tv, st, &pre));
        CK(ctx->cols.ensure(blk[0] + blk[1] + blk[2] + 256));
        char *dst = (char *)ctx->cols.p;
        const void *src[3] = {tv->bonds, tv->angles, tv->dihedrals};
        const int cnt[3] = {g.nb, g.na, g.nd};
        for (int t = 0; t < 3; t++) {
            cols[t] = dst;
            if (cnt[t] > 0 && !pre) {
                if (tv->ld == tv->n_frames) {
                    bool pulled = false;
                    CK(h2d_copy(dst, src[t], blk[t], st, &pulled));
                    if (pulled) ctx->launches++;
                } else {
                    CK(cudaMemcpy2DAsync(dst, ld * es, src[t], tv->ld * es, ld * es, cnt[t],
                                         cudaMemcpyHostToDevice, st));
                }
            }
            dst += blk[t];
        }
        if (g.nd == 0) cols[2] = cols[1];
    }
    CK(cudaEventRecord(ctx->ev[1], st));
    {
        // pg_entropy_ahead: the next call's columns follow on the copy engine
        const int rca = queue_ahead(ctx, st);
        if (rca) return rca;
    }

    CK(ctx->bins.ensure(bins_bytes(g)));
    CK(ctx->dofbuf.ensure(dof_bytes(D)));
    CK(ctx->errw.ensure(ERR_WORDS * sizeof(int)));
    CK(cudaMemsetAsync(ctx->errw.p, 0, ERR_WORDS * sizeof(int), st));
    if (ctx->nlogn_max < g.F) {
        CK(ctx->nlogn.ensure(((size_t)g.F + 1) * sizeof(double)));
        CK(launch_nlogn_table((double *)ctx->nlogn.p, g.F, st));
        ctx->launches++;
        ctx->nlogn_max = g.F;
    }
    if (prep_smem_bytes(g) > 200 * 1024) return fail(ctx, PG_ERR_UNSUPPORTED, "1D bin counts too large");
    CK(launch_prep(g, cols, ld, tv->double_prec, dof_arrays(ctx, D), (uint8_t *)ctx->bins.p,
                   (int *)ctx->errw.p, st));
    ctx->launches++;
    CK(cudaEventRecord(ctx->ev[2], st));
    return PG_OK;
}

// Enqueues the copies of a device .par body (layout L) into the caller's
// blocks (host memory, or device memory of this context's GPU: the copy
// direction comes from the pointers); every non-empty block needs a
// destination.
static int body_to_host(pg_ctx *ctx, const double *par, const ParLayout &L, const pg_par_body *out, int sys) {
    double *dst[9] = {out->s1_b, out->s1_a, out->s1_d, out->bb, out->ba, out->bd, out->aa, out->ad, out->dd};
    const int64_t off[10] = {L.s1b, L.s1a, L.s1d, L.bb, L.ba, L.bd, L.aa, L.ad, L.dd, L.total};
    for (int k = 0; k < 9; k++) {
        const int64_t n = off[k + 1] - off[k];
        if (n <= 0) continue;
        if (!dst[k]) {
            if (sys >= 0) return fail(ctx, PG_ERR_ARG, "system %d: null output block %d", sys, k);
            return fail(ctx, PG_ERR_ARG, "null output block %d", k);
        }
        CK(cudaMemcpyAsync(dst[k], par + off[k], (size_t)n * sizeof(double), cudaMemcpyDefault, ctx->stream));
    }
    return PG_OK;
}

static int check_err_words(pg_ctx *ctx) {
    int h[ERR_WORDS];
    CK(cudaMemcpyAsync(h, ctx->errw.p, sizeof h, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (h[ERR_NEG_BOND]) return fail(ctx, PG_ERR_DATA, "ERROR: %d bond(s) smaller than 0.0", h[ERR_NEG_BOND]);
    if (h[ERR_MODFIT_RANGE])
        return fail(ctx, PG_ERR_DATA, "%d dihedral value(s) outside [0, 2pi+5e-9) (shift histogram)", h[ERR_MODFIT_RANGE]);
    if (h[ERR_BIN_RANGE]) return fail(ctx, PG_ERR_DATA, "%d bin index(es) outside [0, B)", h[ERR_BIN_RANGE]);
    if (h[ERR_TIMEOUT]) return fail(ctx, PG_ERR_TIMEOUT, "a device-side wait timed out (%d CTA(s))", h[ERR_TIMEOUT]);
    return PG_OK;
}

static int bmax_of(const SysGeom &g) {
    return std::max(g.bins[3], std::max(g.bins[4], g.bins[5]));
}

// Fixed-point n ln n table covering counts up to F. A table built for a
// larger F is reused: its scale is no larger, so sums still fit 64 bits.
static int ensure_fix_table(pg_ctx *ctx, int F) {
    if (ctx->nfix_max >= F) return PG_OK;
    const double fix = nlogn_fix_scale(F);
    CK(ctx->nfix.ensure(((size_t)F + 1) * sizeof(unsigned long long)));
    CK(launch_nlogn_fix_table((unsigned long long *)ctx->nfix.p, F, fix, ctx->stream));
    ctx->launches++;
    ctx->nfix_max = F;
    ctx->nfix_scale = fix;
    return PG_OK;
}

static bool use_hist32(const SysGeom &g) { return hist_layout(g) != HIST16; }

// The bin matrices the preprocessing writes for a form: the 16-bit 32-slot
// layouts stage their row DOFs from the row-code matrix; the streamed layout
// reads both matrices frame-group interleaved; the one-hot form and the
// 16-slot kernel read plain DOF rows.
static void set_bin_layout(SysGeom &g, int form) {
    int chosen = form == PG_FORM_AUTO ? autotune_form(g) : form;
    if (chosen == PG_FORM_ONEHOT && !pairs_onehot_supported(g)) chosen = PG_FORM_HIST;
    const bool hist = chosen != PG_FORM_ONEHOT;
    const int layout = hist ? hist_layout(g) : HIST16;
    g.codes = layout_codes(layout, bmax_of(g));
    g.ilv = layout_ilv(layout);
}

// Launches the 32-slot kernel over the cached full tile list (explicit ==
// nullptr) or over n_explicit given tiles; the per-CTA accumulators live in
// ctx->scratch.
static int run_hist32(pg_ctx *ctx, const SysGeom &g, const DofArrays &dof, const PairOut &po,
                      const PairTile *explicit_tiles, int64_t n_explicit) {
    cudaStream_t st = ctx->stream;
    const PairTile *tiles;
    int64_t n;
    DevBuf ex;
    if (explicit_tiles) {
        CK(ex.ensure(sizeof(PairTile) * (size_t)std::max<int64_t>(n_explicit, 1)));
        CK(cudaMemcpyAsync(ex.p, explicit_tiles, sizeof(PairTile) * n_explicit, cudaMemcpyHostToDevice, st));
        tiles = (const PairTile *)ex.p;
        n = n_explicit;
    } else {
        if (ctx->tiles_D != g.D || ctx->tiles_T != 32) {
            ctx->tiles_host = build_tiles32(g.D);
            CK(ctx->tiles.ensure(ctx->tiles_host.size() * sizeof(PairTile)));
            CK(cudaMemcpyAsync(ctx->tiles.p, ctx->tiles_host.data(), ctx->tiles_host.size() * sizeof(PairTile),
                               cudaMemcpyHostToDevice, st));
            CK(cudaStreamSynchronize(st));
            ctx->tiles_D = g.D;
            ctx->tiles_T = 32;
        }
        tiles = (const PairTile *)ctx->tiles.p;
        n = (int64_t)ctx->tiles_host.size();
    }
    const size_t sb = pairs_hist32_scratch_bytes(bmax_of(g), pairs_hist32_grid(n));
    CK(ctx->scratch.ensure(sb));
    int rc = ensure_fix_table(ctx, g.F);
    if (rc) return rc;
    CK(launch_pairs_hist32(g, (const uint8_t *)ctx->bins.p, dof, (const unsigned long long *)ctx->nfix.p,
                           ctx->nfix_scale, tiles, n, po, (int *)ctx->errw.p, ctx->scratch.p, sb, st));
    ctx->launches++;
    if (explicit_tiles) {
        CK(cudaStreamSynchronize(st));  // the private tile buffer is released on return
    }
    return PG_OK;
}

static int mist_edges_to_user(pg_ctx *ctx, int n_dihedrals, const double *hmi, const int *hf, const int *ht,
                              const double *s1, pg_mist_edge *edges, double totals[10]);

// Tile list of the histogram layout a geometry uses, and the contiguous range
// [b, e) of it that shard `shard` of `n_shards` owns (balanced by tile count;
// tiles carry equal work apart from the diagonal and ragged edges).
static std::vector<PairTile> layout_tiles(const SysGeom &g, int *T_out) {
    int T = 0, fc = 0, nst = 0;
    const bool h32 = use_hist32(g);
    if (!h32 && !pairs_hist_config(bmax_of(g), &T, &fc, &nst)) return {};
    *T_out = h32 ? 32 : T;
    return h32 ? build_tiles32(g.D) : build_tiles(g.D, T);
}
// The contiguous tile range [b, e) of shard `shard`: cut where the running
// work passes shard / n_shards of the total, a tile's work being its pair
// slots with r < c (the counting, which dominates) plus two for streaming its
// bin rows, so shards of diagonal and ragged-edge tiles take more tiles.
static void shard_range(const std::vector<PairTile> &tl, int shard, int n_shards, int64_t *b, int64_t *e) {
    std::vector<double> cum(tl.size() + 1, 0.0);
    for (size_t k = 0; k < tl.size(); k++) {
        const PairTile &t = tl[k];
        int pairs = 0;
        for (int r = 0; r < t.nrow; r++)
            for (int c = 0; c < t.ncol; c++) pairs += t.row0 + r < t.col0 + c;
        cum[k + 1] = cum[k] + pairs + 2.0;
    }
    const double W = cum.back();
    auto cut = [&](int s) -> int64_t {
        if (s <= 0) return 0;
        if (s >= n_shards) return (int64_t)tl.size();
        const double target = W * s / n_shards;
        return (int64_t)(std::lower_bound(cum.begin(), cum.end(), target) - cum.begin());
    };
    *b = cut(shard);
    *e = std::max(*b, cut(shard + 1));
}

// Entropies of a HOST trajectory, the upload optionally overlapped: the DOFs
// are split into K groups on column super-block boundaries of the tile list;
// a second stream uploads group after group, and on the context's stream
// group k's preprocessing and the pair tiles whose column block lies in group
// k (their row DOFs are in groups <= k) start as soon as group k has arrived.
// The pair launches of consecutive groups go to two streams in turn (each
// waits for its group's preprocessing), so the last wave of one persistent
// launch overlaps the first CTAs of the next. K = 1 by default (see below).
// Same kernels and results as the device-resident path; histogram form
// (geometry already set by setup_geometry).
static int run_streamed(pg_ctx *ctx, const pg_bat_view *tv, pg_par_body *out) {
    const SysGeom &g = ctx->geo;
    const int D = g.D;
    cudaStream_t st = ctx->stream, cs = ctx->copy;
    const size_t es = elem_size(tv->double_prec);
    const int64_t F = g.F;
    const bool h32 = use_hist32(g);
    int T = 0, fc = 0, nst = 0;
    if (!h32 && !pairs_hist_config(bmax_of(g), &T, &fc, &nst)) return fail(ctx, PG_ERR_UNSUPPORTED, "2D bins too large");
    if (prep_smem_bytes(g) > 200 * 1024) return fail(ctx, PG_ERR_UNSUPPORTED, "1D bin counts too large");
    const ParLayout L = par_layout(g.n_dih);
    CK(ctx->cols.ensure((size_t)D * F * es + 256));
    CK(ctx->bins.ensure(bins_bytes(g)));
    CK(ctx->dofbuf.ensure(dof_bytes(D)));
    CK(ctx->errw.ensure(ERR_WORDS * sizeof(int)));
    CK(ctx->par.ensure((size_t)L.total * sizeof(double)));
    CK(ctx->mi.ensure((size_t)D * D * sizeof(double)));
    const int layout = h32 ? 32 : T;
    if (ctx->tiles_D != D || ctx->tiles_T != layout) {
        ctx->tiles_host = h32 ? build_tiles32(D) : build_tiles(D, T);
        CK(ctx->tiles.ensure(ctx->tiles_host.size() * sizeof(PairTile)));
        CK(cudaMemcpyAsync(ctx->tiles.p, ctx->tiles_host.data(), ctx->tiles_host.size() * sizeof(PairTile),
                           cudaMemcpyHostToDevice, st));
        CK(cudaStreamSynchronize(st));
        ctx->tiles_D = D;
        ctx->tiles_T = layout;
    }
    // groups of whole column super-blocks (16 tiles wide); both tile lists
    // run over column super-blocks in order, so a group's tiles are one range
    const int sbw = 16 * (h32 ? 8 : T);
    const int nsb = (D + sbw - 1) / sbw;
    // Upload groups, PG_STREAM_GROUPS = 1..64, default 1: the whole upload
    // first, by SM loads. Measured at 7,494 DOFs x 500k frames (15 GB): the
    // columns arrive in ~71 ms that way, while copy-engine uploads that
    // overlap the pair kernels ran at 26-80 GB/s and each group's
    // preprocessing waited for SMs the persistent pair kernels held: 16
    // groups took 3.64-3.72 s against 3.58 s for one (copy engine) and 3.45 s
    // with the columns already resident.
    int K = 1;
    if (const char *e = getenv("PG_STREAM_GROUPS")) K = std::max(1, std::min(pg_ctx::kMaxGroups, atoi(e)));
    K = std::min(K, nsb);
    std::vector<int> G((size_t)K + 1);
    std::vector<int64_t> cut((size_t)K + 1);
    for (int k = 0; k <= K; k++) G[k] = std::min(D, (int)((int64_t)k * nsb / K) * sbw);
    {
        const std::vector<PairTile> &tl = ctx->tiles_host;
        int64_t i = 0;
        for (int k = 0; k <= K; k++) {
            while (i < (int64_t)tl.size() && tl[i].col0 < G[k]) i++;
            cut[k] = k == K ? (int64_t)tl.size() : i;
        }
    }
    const size_t sb32 = h32 ? pairs_hist32_scratch_bytes(bmax_of(g), pairs_hist32_grid((int64_t)ctx->tiles_host.size()))
                            : 0;
    // one scratch area (tile counter, overflow counts) per pair stream
    if (h32) CK(ctx->scratch.ensure(2 * sb32));

    CK(cudaEventRecord(ctx->ev[0], st));
    CK(cudaStreamWaitEvent(cs, ctx->ev[0], 0));  // earlier kernels reading the columns are done
    bool pre = false;  // the columns were uploaded ahead by pg_prefetch
    CK(take_prefetch(ctx, tv, cs, &pre));
    CK(ctx->cols.ensure((size_t)D * F * es + 256));
    char *cols = (char *)ctx->cols.p;
    const int lo[3] = {0, g.nb, g.nb + g.na}, cnt[3] = {g.nb, g.na, g.nd};
    const void *src[3] = {tv->bonds, tv->angles, tv->dihedrals};
    for (int k = 0; k < K; k++) {
        for (int t = 0; t < 3 && !pre; t++) {
            const int a = std::max(G[k], lo[t]), b = std::min(G[k + 1], lo[t] + cnt[t]);
            if (a >= b) continue;
            const char *from = (const char *)src[t] + (size_t)(a - lo[t]) * tv->ld * es;
            if (tv->ld == F && K == 1) {  // nothing to overlap: SM loads, the fastest route
                bool pulled = false;
                CK(h2d_copy(cols + (size_t)a * F * es, from, (size_t)(b - a) * F * es, cs, &pulled));
                if (pulled) ctx->launches++;
            } else if (tv->ld == F) {  // contiguous rows: one linear copy (2D copies ran at 20-80 GB/s)
                CK(cudaMemcpyAsync(cols + (size_t)a * F * es, from, (size_t)(b - a) * F * es, cudaMemcpyHostToDevice,
                                   cs));
            } else
                CK(cudaMemcpy2DAsync(cols + (size_t)a * F * es, (size_t)F * es, from, (size_t)tv->ld * es,
                                     (size_t)F * es, (size_t)(b - a), cudaMemcpyHostToDevice, cs));
        }
        CK(cudaEventRecord(ctx->gev[k], cs));
    }
    CK(cudaEventRecord(ctx->ev[4], cs));
    {
        // pg_entropy_ahead: the next call's columns follow on the copy engine
        const int rca = queue_ahead(ctx, cs);
        if (rca) return rca;
    }

    CK(cudaMemsetAsync(ctx->errw.p, 0, ERR_WORDS * sizeof(int), st));
    int rc = ensure_fix_table(ctx, g.F);
    if (rc) return rc;
    const void *colp[3] = {cols, cols + (size_t)g.nb * F * es,
                           g.nd ? cols + (size_t)(g.nb + g.na) * F * es : cols + (size_t)g.nb * F * es};
    const DofArrays dof = dof_arrays(ctx, D);
    PairOut po;
    po.par = (double *)ctx->par.p;
    po.mi = (double *)ctx->mi.p;
    po.L = L;
    po.counts = nullptr;
    po.counts_bmax = 0;
    const PairTile *tiles = (const PairTile *)ctx->tiles.p;
    if (!ctx->pst[0]) {
        for (int k = 0; k < 2; k++) {
            CK(cudaStreamCreateWithFlags(&ctx->pst[k], cudaStreamNonBlocking));
            CK(cudaEventCreateWithFlags(&ctx->pend[k], cudaEventDisableTiming));
        }
        for (auto &e : ctx->pev) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    for (int k = 0; k < K; k++) {
        CK(cudaStreamWaitEvent(st, ctx->gev[k], 0));
        CK(launch_prep(g, colp, F, tv->double_prec, dof, (uint8_t *)ctx->bins.p, (int *)ctx->errw.p, st, G[k],
                       G[k + 1] - G[k]));
        ctx->launches++;
        // group k's pair tiles need the bins of groups 0..k: every prep so far
        CK(cudaEventRecord(ctx->pev[k], st));
        const int64_t n = cut[k + 1] - cut[k];
        if (n <= 0) continue;
        cudaStream_t ps = ctx->pst[k & 1];
        CK(cudaStreamWaitEvent(ps, ctx->pev[k], 0));
        if (h32)
            CK(launch_pairs_hist32(g, (const uint8_t *)ctx->bins.p, dof, (const unsigned long long *)ctx->nfix.p,
                                   ctx->nfix_scale, tiles + cut[k], n, po, (int *)ctx->errw.p,
                                   (char *)ctx->scratch.p + (k & 1) * sb32, sb32, ps));
        else
            CK(launch_pairs_hist(g, (const uint8_t *)ctx->bins.p, dof, (const unsigned long long *)ctx->nfix.p,
                                 ctx->nfix_scale, tiles + cut[k], n, T, po, (int *)ctx->errw.p, ps));
        ctx->launches++;
    }
    for (int k = 0; k < 2; k++) {
        CK(cudaEventRecord(ctx->pend[k], ctx->pst[k]));
        CK(cudaStreamWaitEvent(st, ctx->pend[k], 0));
    }
    CK(cudaMemcpyAsync((double *)ctx->par.p + L.s1b, dof.s1, (size_t)D * sizeof(double), cudaMemcpyDeviceToDevice,
                       st));
    CK(cudaEventRecord(ctx->ev[1], st));
    if (out) {
        const int rcb = body_to_host(ctx, (const double *)ctx->par.p, L, out, -1);
        if (rcb) return rcb;
    }
    CK(cudaEventRecord(ctx->ev[2], st));
    rc = check_err_words(ctx);
    float up = 0.f, dev = 0.f, down = 0.f;
    cudaEventElapsedTime(&up, ctx->ev[0], ctx->ev[4]);
    cudaEventElapsedTime(&dev, ctx->ev[0], ctx->ev[1]);
    cudaEventElapsedTime(&down, ctx->ev[1], ctx->ev[2]);
    ctx->timings[0] = 0.0;   // preprocessing runs interleaved with the pair launches
    ctx->timings[1] = dev;   // first upload group to the last pair launch
    ctx->timings[3] = up + down;
    ctx->timings[4] = dev + down;
    if (rc) return rc;
    ctx->last_form = PG_FORM_HIST;
    ctx->resident = true;
    return PG_OK;
}

extern "C" {

PG_API const char *pg_last_global_error(void) { return g_global_err.c_str(); }

PG_API int pg_create(pg_ctx **out, int device) {
    if (!out) return fail(nullptr, PG_ERR_ARG, "null out");
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0)
        return fail(nullptr, PG_ERR_CUDA, "no CUDA device: %s", cudaGetErrorString(e));
    if (device < 0 || device >= n) return fail(nullptr, PG_ERR_ARG, "device %d out of range", device);
    e = cudaSetDevice(device);
    if (e != cudaSuccess) return fail(nullptr, PG_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
    pg_ctx *c = new pg_ctx;
    c->device = device;
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->copy, cudaStreamNonBlocking);
    for (int k = 0; k < 6 && e == cudaSuccess; k++) e = cudaEventCreate(&c->ev[k]);
    for (int k = 0; k < pg_ctx::kMaxGroups && e == cudaSuccess; k++)
        e = cudaEventCreateWithFlags(&c->gev[k], cudaEventDisableTiming);
    if (e != cudaSuccess) {
        delete c;
        return fail(nullptr, PG_ERR_CUDA, "stream/event creation: %s", cudaGetErrorString(e));
    }
    *out = c;
    return PG_OK;
}

PG_API void pg_destroy(pg_ctx *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (ctx->pf_pending) cudaEventSynchronize(ctx->pf_done);
    for (DevBuf *b : {&ctx->cols, &ctx->cols_pf, &ctx->bins, &ctx->dofbuf, &ctx->par, &ctx->mi, &ctx->nlogn, &ctx->nfix,
                      &ctx->tiles, &ctx->errw, &ctx->scratch, &ctx->counts, &ctx->edges, &ctx->mistscr,
                      &ctx->bc_out, &ctx->bc_stage, &ctx->bc_soa, &ctx->bc_tmp, &ctx->bc_tab, &ctx->mie_body,
                      &ctx->mie_slots, &ctx->mie_lens, &ctx->mie_rows, &ctx->mie_text, &ctx->mie_fb})
        b->release();
    if (ctx->graph) cudaGraphExecDestroy(ctx->graph);
    ctx->batch.release();
    ctx->batchmeta.release();
    if (ctx->copy) cudaStreamSynchronize(ctx->copy);
    for (auto &e : ctx->ev)
        if (e) cudaEventDestroy(e);
    if (ctx->pf_done) cudaEventDestroy(ctx->pf_done);
    for (auto &e : ctx->gev)
        if (e) cudaEventDestroy(e);
    cudaStreamDestroy(ctx->stream);
    if (ctx->copy) cudaStreamDestroy(ctx->copy);
    for (int k = 0; k < 2; k++) {
        if (ctx->pst[k]) cudaStreamDestroy(ctx->pst[k]);
        if (ctx->pend[k]) cudaEventDestroy(ctx->pend[k]);
    }
    for (auto &e : ctx->pev)
        if (e) cudaEventDestroy(e);
    if (ctx->hstage) cudaFreeHost(ctx->hstage);
    delete ctx;
}

PG_API const char *pg_last_error(const pg_ctx *ctx) { return ctx ? ctx->err.c_str() : g_global_err.c_str(); }

}  // extern "C"

namespace pg {
int mie_lines_device(pg_ctx *ctx, int nd, const pg_par_body *b, const std::function<bool(const char *, size_t)> &sink);
}

// The 2D lines of the MIE text (get_PAR_MIE.cpp:109-199) formatted on the
// device, handed to `sink` in order in pieces of at most 64 MB. Lines with a
// value outside the device formatter's exact range are formatted here.
int pg::mie_lines_device(pg_ctx *ctx, int nd, const pg_par_body *b,
                         const std::function<bool(const char *, size_t)> &sink) {
    if (!ctx || !b || nd < 0) return fail(ctx, PG_ERR_ARG, "mie: bad arguments");
    ctx->err.clear();
    cudaGetLastError();  // an error left by an earlier failed call of this thread is not this call's
    CK(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const int nb = nd + 2, na = nd + 1;
    const ParLayout L = par_layout(nd);
    const double *hb[9] = {b->s1_b, b->s1_a, b->s1_d, b->bb, b->ba, b->bd, b->aa, b->ad, b->dd};
    const int64_t off[9] = {L.s1b, L.s1a, L.s1d, L.bb, L.ba, L.bd, L.aa, L.ad, L.dd};
    const int64_t len9[9] = {L.s1a - L.s1b, L.s1d - L.s1a, L.bb - L.s1d, L.ba - L.bb, L.bd - L.ba,
                             L.aa - L.bd, L.ad - L.aa, L.dd - L.ad, L.total - L.dd};
    CK(ctx->mie_body.ensure((size_t)L.total * sizeof(double) + 64));
    double *db = (double *)ctx->mie_body.p;
    for (int k = 0; k < 9; k++)
        if (len9[k] > 0) CK(cudaMemcpyAsync(db + off[k], hb[k], (size_t)len9[k] * sizeof(double), cudaMemcpyHostToDevice, st));
    MieArgs a{};
    static const char *nm[6] = {"bond-bond ", "bond-angle ", "bond-dihedral ", "angle-angle ", "angle-dihedral ",
                                "dihedral-dihedral "};
    const int n1[6] = {nb, nb, nb, na, na, nd}, n2[6] = {nb, na, nd, na, nd, nd}, same[6] = {1, 0, 0, 1, 0, 1};
    const int64_t boff[6] = {L.bb, L.ba, L.bd, L.aa, L.ad, L.dd};
    const int64_t s1o[3] = {L.s1b, L.s1a, L.s1d};
    const int rt[6] = {0, 0, 0, 1, 1, 2}, ct[6] = {0, 1, 2, 1, 2, 2};
    int64_t lines = 0;
    int rows = 0;
    for (int q = 0; q < 6; q++) {
        a.blk[q] = db + boff[q];
        a.s1r[q] = db + s1o[rt[q]];
        a.s1c[q] = db + s1o[ct[q]];
        a.n1[q] = n1[q];
        a.n2[q] = n2[q];
        a.same[q] = same[q];
        a.line0[q] = lines;
        a.row0[q] = rows;
        const int64_t nl = same[q] ? (int64_t)n1[q] * (n1[q] - 1) / 2 : (int64_t)n1[q] * n2[q];
        if (nl > 0) rows += same[q] ? n1[q] - 1 : n1[q];
        lines += nl;
        a.name_len[q] = (int)strlen(nm[q]);
        memcpy(a.name[q], nm[q], (size_t)a.name_len[q]);
    }
    a.row0[6] = rows;
    a.rows = rows;
    if (lines == 0) return PG_OK;
    constexpr int kFbCap = 1 << 16;
    CK(ctx->mie_slots.ensure((size_t)lines * kMieSlot));
    CK(ctx->mie_lens.ensure((size_t)lines));
    CK(ctx->mie_rows.ensure((size_t)(2 * (int64_t)rows + 1) * sizeof(long long)));
    CK(ctx->mie_fb.ensure(sizeof(int64_t) * (kFbCap + 1)));
    a.slots = (char *)ctx->mie_slots.p;
    a.lens = (uint8_t *)ctx->mie_lens.p;
    a.row_len = (long long *)ctx->mie_rows.p;
    a.row_off = a.row_len + rows;
    a.fb_count = (int *)ctx->mie_fb.p;
    a.fb_list = (int64_t *)ctx->mie_fb.p + 1;
    a.fb_cap = kFbCap;
    CK(cudaMemsetAsync(a.fb_count, 0, sizeof(int), st));
    CK(launch_mie_format(a, st));
    ctx->launches++;
    int nfb = 0;
    CK(cudaMemcpyAsync(&nfb, a.fb_count, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (nfb > kFbCap) return fail(ctx, PG_ERR_UNSUPPORTED, "mie: %d values outside the device formatter's range", nfb);
    if (nfb > 0) {  // the C library formats these lines; they go into their slots
        std::vector<int64_t> fl((size_t)nfb);
        CK(cudaMemcpy(fl.data(), a.fb_list, sizeof(int64_t) * nfb, cudaMemcpyDeviceToHost));
        const double *hs1[3] = {b->s1_b, b->s1_a, b->s1_d};
        const double *hblk[6] = {b->bb, b->ba, b->bd, b->aa, b->ad, b->dd};
        for (int64_t Lg : fl) {
            int q = 5;
            while (q > 0 && Lg < a.line0[q]) q--;
            const int64_t Lq = Lg - a.line0[q];
            int i, j;
            double s2;
            if (same[q]) {  // row i starts at i (n-1) - i (i-1) / 2
                const int64_t n = n1[q];
                int lo = 0, hi = n1[q] - 2;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) / 2;
                    if ((int64_t)mid * (n - 1) - (int64_t)mid * (mid - 1) / 2 <= Lq) lo = mid; else hi = mid - 1;
                }
                i = lo;
                j = i + 1 + (int)(Lq - ((int64_t)i * (n - 1) - (int64_t)i * (i - 1) / 2));
                s2 = hblk[q][n * (n - 1) / 2 - 1 - Lq];
            } else {
                i = (int)(Lq / n2[q]);
                j = (int)(Lq % n2[q]);
                s2 = hblk[q][Lq];
            }
            const double mu = hs1[rt[q]][i] + hs1[ct[q]][j] - s2;
            char line[kMieSlot + 64];
            const int k = snprintf(line, sizeof line, "%s%d  %d   %.12g   %.12g\n", nm[q], i + 1, j + 1, s2, mu);
            if (k <= 0 || k > kMieSlot) return fail(ctx, PG_ERR_UNSUPPORTED, "mie: line too long");
            const uint8_t lk = (uint8_t)k;
            CK(cudaMemcpy(a.slots + Lg * kMieSlot, line, (size_t)k, cudaMemcpyHostToDevice));
            CK(cudaMemcpy(a.lens + Lg, &lk, 1, cudaMemcpyHostToDevice));
        }
    }
    CK(launch_mie_offsets(a, st));
    long long total = 0;
    CK(cudaMemcpyAsync(&total, a.row_off + rows, sizeof(long long), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    CK(ctx->mie_text.ensure((size_t)total + 64));
    a.text = (char *)ctx->mie_text.p;
    CK(launch_mie_compact(a, st));
    ctx->launches += 3;
    // to the host in pieces, the next piece copied while the sink writes one
    constexpr size_t kPiece = (size_t)64 << 20;
    char *pin[2] = {nullptr, nullptr};
    cudaEvent_t done[2] = {nullptr, nullptr};
    int rc = PG_OK;
    for (int k = 0; k < 2 && rc == PG_OK; k++) {
        if (cudaHostAlloc(&pin[k], kPiece, cudaHostAllocDefault) != cudaSuccess ||
            cudaEventCreateWithFlags(&done[k], cudaEventDisableTiming) != cudaSuccess)
            rc = fail(ctx, PG_ERR_NOMEM, "mie: pinned staging");
    }
    const size_t T = (size_t)total, np = (T + kPiece - 1) / kPiece;
    for (size_t k = 0; k < np && rc == PG_OK; k++) {
        const int s = (int)(k & 1);
        if (k == 0) {
            cudaMemcpyAsync(pin[0], a.text, std::min(kPiece, T), cudaMemcpyDeviceToHost, st);
            cudaEventRecord(done[0], st);
        }
        if (k + 1 < np) {
            const size_t o = (k + 1) * kPiece;
            cudaMemcpyAsync(pin[s ^ 1], a.text + o, std::min(kPiece, T - o), cudaMemcpyDeviceToHost, st);
            cudaEventRecord(done[s ^ 1], st);
        }
        if (cudaEventSynchronize(done[s]) != cudaSuccess) {
            rc = fail(ctx, PG_ERR_CUDA, "mie: copy");
            break;
        }
        if (!sink(pin[s], std::min(kPiece, T - k * kPiece))) rc = fail(ctx, PG_ERR_IO, "mie: write failed");
    }
    cudaStreamSynchronize(st);
    for (int k = 0; k < 2; k++) {
        if (pin[k]) cudaFreeHost(pin[k]);
        if (done[k]) cudaEventDestroy(done[k]);
    }
    return rc;
}

extern "C" {

PG_API int pg_bat_from_cartesian(pg_ctx *ctx, const float *xyz, int xyz_on_device, int n_frames, int n_dihedrals,
                                 const int *dih, int double_prec, pg_bat_view *out) {
    if (!ctx) return fail(nullptr, PG_ERR_ARG, "null context");
    ctx->err.clear();
    cudaGetLastError();  // an error left by an earlier failed call of this thread is not this call's
    if (!xyz || !dih || !out) return fail(ctx, PG_ERR_ARG, "null argument");
    if (n_dihedrals < 1 || n_frames < 1) return fail(ctx, PG_ERR_ARG, "n_dihedrals (%d) or n_frames (%d) < 1",
                                                     n_dihedrals, n_frames);
    if (double_prec != 0 && double_prec != 1) return fail(ctx, PG_ERR_ARG, "double_prec must be 0 or 1");
    const int nd = n_dihedrals, na = nd + 3;  // BAT_trajectory.cpp:80-83: natoms == nDih + 3
    std::vector<int4> atoms((size_t)nd);
    std::vector<int> parent((size_t)nd);
    for (int i = 0; i < nd; i++) {
        const int *r = dih + 6 * (size_t)i;
        for (int k = 0; k < 4; k++)
            if (r[k] < 1 || r[k] > na) return fail(ctx, PG_ERR_ARG, "dihedral %d: atom %d outside 1..%d", i + 1, r[k], na);
        if (r[5] != -1 && (r[5] < 1 || r[5] > nd))
            return fail(ctx, PG_ERR_ARG, "dihedral %d: parent %d outside 1..%d", i + 1, r[5], nd);
        atoms[i] = make_int4(r[0] - 1, r[1] - 1, r[2] - 1, r[3] - 1);
        parent[i] = r[5] == -1 ? -1 : r[5] - 1;
    }
    CK(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const int64_t F = n_frames, ld = (F + 31) / 32 * 32;
    const size_t es = double_prec ? 8 : 4;
    const int64_t fc = std::min<int64_t>(F, 65536);  // frames per chunk
    const int64_t lds = (fc + 31) / 32 * 32;
    CK(ctx->bc_out.ensure((size_t)(3 * (int64_t)nd + 3) * ld * es));
    CK(ctx->bc_soa.ensure((size_t)3 * na * lds * sizeof(float)));
    if (!double_prec) CK(ctx->bc_tmp.ensure((size_t)nd * lds * sizeof(double)));
    // host coordinates the GPU can read go straight into the transpose (one
    // read over the host link), the others through a staging copy
    const bool stage = !xyz_on_device && !host_readable(xyz);
    if (stage) CK(ctx->bc_stage.ensure((size_t)fc * na * 3 * sizeof(float)));
    CK(ctx->bc_tab.ensure((size_t)nd * (sizeof(int4) + sizeof(int))));
    int4 *d_atoms = (int4 *)ctx->bc_tab.p;
    int *d_parent = (int *)(d_atoms + nd);
    CK(cudaMemcpyAsync(d_atoms, atoms.data(), sizeof(int4) * nd, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(d_parent, parent.data(), sizeof(int) * nd, cudaMemcpyHostToDevice, st));
    char *o = (char *)ctx->bc_out.p;
    void *bonds = o, *angles = o + (size_t)(nd + 2) * ld * es, *dihs = o + (size_t)(2 * nd + 3) * ld * es;
    CK(cudaEventRecord(ctx->ev[0], st));
    for (int64_t f0 = 0; f0 < F; f0 += fc) {
        const int n = (int)std::min<int64_t>(fc, F - f0);
        const float *src = xyz + (size_t)f0 * na * 3;
        if (stage) {
            CK(cudaMemcpyAsync(ctx->bc_stage.p, src, (size_t)n * na * 3 * sizeof(float), cudaMemcpyHostToDevice, st));
            src = (const float *)ctx->bc_stage.p;
        }
        CK(launch_cart_transpose(src, n, na, (float *)ctx->bc_soa.p, lds, st));
        double *tmp = double_prec ? (double *)dihs + f0 : (double *)ctx->bc_tmp.p;
        const int64_t ldt = double_prec ? ld : lds;
        CK(launch_bat_convert((const float *)ctx->bc_soa.p, lds, n, nd, d_atoms, bonds, angles, ld, f0, double_prec,
                              tmp, ldt, st));
        CK(launch_bat_phase(tmp, ldt, n, nd, d_parent, dihs, ld, f0, double_prec, st));
        ctx->launches += 3;
    }
    CK(cudaEventRecord(ctx->ev[1], st));
    CK(cudaStreamSynchronize(st));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]));
    ctx->timings[4] = ms;
    out->n_dihedrals = nd;
    out->n_frames = n_frames;
    out->double_prec = double_prec;
    out->on_device = 1;
    out->ld = ld;
    out->bonds = bonds;
    out->angles = angles;
    out->dihedrals = dihs;
    return PG_OK;
}

PG_API int pg_prefetch(pg_ctx *ctx, const pg_bat_view *traj) {
    if (!ctx) return fail(nullptr, PG_ERR_ARG, "null context");
    ctx->err.clear();
    cudaGetLastError();  // an error left by an earlier failed call of this thread is not this call's
    CK(cudaSetDevice(ctx->device));
    return queue_prefetch(ctx, traj, ctx->stream);
}

PG_API int pg_entropy(pg_ctx *ctx, const pg_bat_view *traj, const int bins[6], int form,
                      pg_par_body *out) {
    if (!ctx) return fail(nullptr, PG_ERR_ARG, "null context");
    ctx->err.clear();
    cudaGetLastError();  // an error left by an earlier failed call of this thread is not this call's
    if (form < PG_FORM_AUTO || form > PG_FORM_ONEHOT) return fail(ctx, PG_ERR_ARG, "unknown form %d", form);
    if (traj && !traj->on_device && form != PG_FORM_ONEHOT) {
        int rc0 = setup_geometry(ctx, traj, bins, form);
        if (rc0) return rc0;
        const int f = form == PG_FORM_AUTO ? autotune_form(ctx->geo) : form;
        if (f != PG_FORM_ONEHOT || !pairs_onehot_supported(ctx->geo)) return run_streamed(ctx, traj, out);
    }
    int rc = run_prep(ctx, traj, bins, form);
    if (rc) return rc;
    const SysGeom &g = ctx->geo;
    cudaStream_t st = ctx->stream;
    const ParLayout L = par_layout(g.n_dih);
    CK(ctx->par.ensure((size_t)L.total * sizeof(double)));
    CK(ctx->mi.ensure((size_t)g.D * g.D * sizeof(double)));
    DofArrays dof = dof_arrays(ctx, g.D);
    // 1D entropies into the .par body (bonds, angles, dihedrals are contiguous
    // in both the DOF arrays and the body)
    CK(cudaMemcpyAsync((double *)ctx->par.p + L.s1b, dof.s1, (size_t)g.D * sizeof(double),
                       cudaMemcpyDeviceToDevice, st));

    int chosen = form == PG_FORM_AUTO ? autotune_form(g) : form;
    if (chosen == PG_FORM_ONEHOT && !pairs_onehot_supported(g)) {
        if (form == PG_FORM_ONEHOT)
            return fail(ctx, PG_ERR_UNSUPPORTED, "one-hot tensor-core form unsupported for this geometry");
        chosen = PG_FORM_HIST;
    }
    PairOut po;
    po.par = (double *)ctx->par.p;
    po.mi = (double *)ctx->mi.p;
    po.L = L;
    po.counts = nullptr;
    po.counts_bmax = 0;
    if (chosen == PG_FORM_HIST && use_hist32(g)) {
        int rc2 = run_hist32(ctx, g, dof, po, nullptr, 0);
        if (rc2) return rc2;
    } else if (chosen == PG_FORM_HIST) {
        int T = 0, fc = 0, nst = 0;
        if (!pairs_hist_config(bmax_of(g), &T, &fc, &nst)) return fail(ctx, PG_ERR_UNSUPPORTED, "2D bins too large");
        if (ctx->tiles_D != g.D || ctx->tiles_T != T) {
            ctx->tiles_host = build_tiles(g.D, T);
            CK(ctx->tiles.ensure(ctx->tiles_host.size() * sizeof(PairTile)));
            CK(cudaMemcpyAsync(ctx->tiles.p, ctx->tiles_host.data(), ctx->tiles_host.size() * sizeof(PairTile),
                               cudaMemcpyHostToDevice, st));
            CK(cudaStreamSynchronize(st));  // host vector may be rebuilt later
            ctx->tiles_D = g.D;
            ctx->tiles_T = T;
        }
        int rc3 = ensure_fix_table(ctx, g.F);
        if (rc3) return rc3;
        CK(launch_pairs_hist(g, (const uint8_t *)ctx->bins.p, dof, (const unsigned long long *)ctx->nfix.p,
                             ctx->nfix_scale,
                             (const PairTile *)ctx->tiles.p, (int64_t)ctx->tiles_host.size(), T, po,
                             (int *)ctx->errw.p, st));
        ctx->launches++;
    } else {
        const size_t sb = pairs_onehot_scratch_bytes(g);
        CK(ctx->scratch.ensure(sb));
        int nl = 0;
        CK(launch_pairs_onehot(g, (const uint8_t *)ctx->bins.p, dof, (const double *)ctx->nlogn.p, po,
                               (int *)ctx->errw.p, st, ctx->scratch.p, sb, &nl));
        ctx->launches += nl;
    }
    ctx->last_form = chosen;
    CK(cudaEventRecord(ctx->ev[3], st));
    if (out) {
        const int rcb = body_to_host(ctx, (const double *)ctx->par.p, L, out, -1);
        if (rcb) return rcb;
    }
    CK(cudaEventRecord(ctx->ev[4], st));
    rc = check_err_words(ctx);
    float ms[4];
    cudaEventElapsedTime(&ms[0], ctx->ev[0], ctx->ev[1]);
    cudaEventElapsedTime(&ms[1], ctx->ev[1], ctx->ev[2]);
    cudaEventElapsedTime(&ms[2], ctx->ev[2], ctx->ev[3]);
    cudaEventElapsedTime(&ms[3], ctx->ev[3], ctx->ev[4]);
    ctx->timings[0] = ms[1];
    ctx->timings[1] = ms[2];
    ctx->timings[3] = ms[0] + ms[3];
    ctx->timings[4] = ms[0] + ms[1] + ms[2] + ms[3];
    if (rc) return rc;
    ctx->resident = true;
    return PG_OK;
}

PG_API int pg_shard_mask(int n_dihedrals, const int bins[6], int shard, int n_shards, uint8_t *mask) {
    if (n_dihedrals < 0 || !bins || !mask || n_shards < 1 || shard < 0 || shard >= n_shards)
        return fail(nullptr, PG_ERR_ARG, "invalid shard arguments");
    SysGeom g{};
    g.n_dih = n_dihedrals;
    g.nb = n_dihedrals + 2;
    g.na = n_dihedrals + 1;
    g.nd = n_dihedrals;
    g.D = g.nb + g.na + g.nd;
    for (int k = 0; k < 6; k++) {
        if (bins[k] < 1 || (k >= 3 && bins[k] > PG_MAX_BINS_2D)) return fail(nullptr, PG_ERR_ARG, "bad bin count");
        g.bins[k] = bins[k];
    }
    int T = 0;
    const std::vector<PairTile> tl = layout_tiles(g, &T);
    const ParLayout L = par_layout(g.n_dih);
    memset(mask, 0, (size_t)L.total);
    if (shard == 0) memset(mask, 1, (size_t)g.D);  // the 1D entropies (body offsets 0 .. D-1)
    int64_t b = 0, e = 0;
    shard_range(tl, shard, n_shards, &b, &e);
    for (int64_t k = b; k < e; k++) {
        const PairTile &t = tl[k];
        for (int r = 0; r < t.nrow; r++)
            for (int c = 0; c < t.ncol; c++) {
                const int g1 = t.row0 + r, g2 = t.col0 + c;
                if (g1 < g2) mask[par_pair_index(L, g.nb, g.na, g.nd, g1, g2)] = 1;
            }
    }
    return PG_OK;
}

PG_API int pg_entropy_ahead(pg_ctx *ctx, const pg_bat_view *traj, const int bins[6], int form,
                            pg_par_body *out, const pg_bat_view *next) {
    if (!ctx) return fail(nullptr, PG_ERR_ARG, "null context");
    ctx->ahead_set = false;
    if (next) {
        if (next->on_device) return fail(ctx, PG_ERR_ARG, "next must be a host view");
        ctx->ahead_view = *next;
        ctx->ahead_set = true;
    }
    int rc = pg_entropy(ctx, traj, bins, form, out);
    // a path that uploaded nothing (device columns) queues it now
    if (rc == PG_OK && ctx->ahead_set) rc = queue_ahead(ctx, ctx->stream);
    ctx->ahead_set = false;
    return rc;
}

PG_API int pg_entropy_shard(pg_ctx *ctx, const pg_bat_view *traj, const int bins[6], int form, int shard,
                            int n_shards, pg_par_body *out) {
    if (!ctx) return fail(nullptr, PG_ERR_ARG, "null context");
    ctx->err.clear();
    cudaGetLastError();  // an error left by an earlier failed call of this thread is not this call's
    if (n_shards < 1 || shard < 0 || shard >= n_shards) return fail(ctx, PG_ERR_ARG, "shard %d of %d", shard, n_shards);
    if (form == PG_FORM_ONEHOT) return fail(ctx, PG_ERR_UNSUPPORTED, "shards use the histogram form");
    if (form != PG_FORM_AUTO && form != PG_FORM_HIST) return fail(ctx, PG_ERR_ARG, "unknown form %d", form);
    int rc = run_prep(ctx, traj, bins, PG_FORM_HIST);  // every shard bins all D columns (O(D F))
    if (rc) return rc;
    const SysGeom &g = ctx->geo;
    cudaStream_t st = ctx->stream;
    const ParLayout L = par_layout(g.n_dih);
    CK(ctx->par.ensure((size_t)L.total * sizeof(double)));
    CK(cudaMemsetAsync(ctx->par.p, 0, (size_t)L.total * sizeof(double), st));
    DofArrays dof = dof_arrays(ctx, g.D);
    if (shard == 0)
        CK(cudaMemcpyAsync((double *)ctx->par.p + L.s1b, dof.s1, (size_t)g.D * sizeof(double),
                           cudaMemcpyDeviceToDevice, st));
    int T = 0;
    const std::vector<PairTile> tl = layout_tiles(g, &T);
    if (tl.empty() && g.D > 1) return fail(ctx, PG_ERR_UNSUPPORTED, "2D bins too large");
    int64_t b = 0, e = 0;
    shard_range(tl, shard, n_shards, &b, &e);
    PairOut po;
    po.par = (double *)ctx->par.p;
    po.mi = nullptr;  // a shard's MI matrix is partial: MIST runs on the merged body
    po.L = L;
    po.counts = nullptr;
    po.counts_bmax = 0;
    if (e > b) {
        DevBuf tbuf;
        CK(tbuf.ensure(sizeof(PairTile) * (size_t)(e - b)));
        CK(cudaMemcpyAsync(tbuf.p, tl.data() + b, sizeof(PairTile) * (size_t)(e - b), cudaMemcpyHostToDevice, st));
        rc = ensure_fix_table(ctx, g.F);
        if (rc) return rc;
        if (T == 32) {
            const size_t sb = pairs_hist32_scratch_bytes(bmax_of(g), pairs_hist32_grid(e - b));
            CK(ctx->scratch.ensure(sb));
            CK(launch_pairs_hist32(g, (const uint8_t *)ctx->bins.p, dof, (const unsigned long long *)ctx->nfix.p,
                                   ctx->nfix_scale, (const PairTile *)tbuf.p, e - b, po, (int *)ctx->errw.p,
                                   ctx->scratch.p, sb, st));
        } else {
            CK(launch_pairs_hist(g, (const uint8_t *)ctx->bins.p, dof, (const unsigned long long *)ctx->nfix.p,
                                 ctx->nfix_scale, (const PairTile *)tbuf.p, e - b, T, po, (int *)ctx->errw.p, st));
        }
        ctx->launches++;
        CK(cudaStreamSynchronize(st));  // the private tile buffer is released on return
    }
    if (out) {
        const int rcb = body_to_host(ctx, (const double *)ctx->par.p, L, out, -1);
        if (rcb) return rcb;
    }
    rc = check_err_words(ctx);
    if (rc) return rc;
    ctx->last_form = PG_FORM_HIST;
    ctx->resident = false;
    return PG_OK;
}

PG_API int pg_pair_counts(pg_ctx *ctx, const pg_bat_view *traj, const int bins[6], int form,
                          int n_pairs, const int *g1, const int *g2, int64_t *counts, int64_t stride) {
    if (!ctx) return fail(nullptr, PG_ERR_ARG, "null context");
    ctx->err.clear();
    cudaGetLastError();  // an error left by an earlier failed call of this thread is not this call's
    if (n_pairs < 0 || (n_pairs > 0 && (!g1 || !g2 || !counts))) return fail(ctx, PG_ERR_ARG, "bad pair list");
    if (form == PG_FORM_ONEHOT) return fail(ctx, PG_ERR_UNSUPPORTED, "count export uses the histogram form");
    int rc = run_prep(ctx, traj, bins, PG_FORM_HIST);
    if (rc) return rc;
    const SysGeom &g = ctx->geo;
    std::vector<PairTile> t((size_t)n_pairs);
    for (int k = 0; k < n_pairs; k++) {
        if (g1[k] < 0 || g2[k] >= g.D || g1[k] >= g2[k])
            return fail(ctx, PG_ERR_ARG, "pair %d: need 0 <= g1 < g2 < D", k);
        t[k] = PairTile{g1[k], g2[k], 1, 1};
        const int b1 = g.bins[3 + dof_type(g1[k], g.nb, g.na)], b2 = g.bins[3 + dof_type(g2[k], g.nb, g.na)];
        if (stride < (int64_t)b1 * b2) return fail(ctx, PG_ERR_ARG, "stride < B1*B2");
    }
    if (n_pairs == 0) return PG_OK;
    const int bm = bmax_of(g);
    cudaStream_t st = ctx->stream;
    PairOut po;
    po.par = nullptr;
    po.mi = nullptr;
    po.L = par_layout(g.n_dih);
    po.counts_bmax = bm;
    int pps;
    cudaError_t e = cudaSuccess;
    DevBuf tiles;  // private: keep the cached full tile list intact
    if (use_hist32(g)) {
        pps = 32;
        CK(ctx->counts.ensure((size_t)n_pairs * pps * bm * bm * sizeof(int64_t)));
        po.counts = (int64_t *)ctx->counts.p;
        int rc2 = run_hist32(ctx, g, dof_arrays(ctx, g.D), po, t.data(), n_pairs);
        if (rc2) return rc2;
    } else {
        int T = 0, fc = 0, nst = 0;
        if (!pairs_hist_config(bm, &T, &fc, &nst)) return fail(ctx, PG_ERR_UNSUPPORTED, "2D bins too large");
        pps = T * T;
        CK(tiles.ensure(t.size() * sizeof(PairTile)));
        CK(ctx->counts.ensure((size_t)n_pairs * pps * bm * bm * sizeof(int64_t)));
        CK(cudaMemcpyAsync(tiles.p, t.data(), t.size() * sizeof(PairTile), cudaMemcpyHostToDevice, st));
        po.counts = (int64_t *)ctx->counts.p;
        int rc3 = ensure_fix_table(ctx, g.F);
        if (rc3) return rc3;
        e = launch_pairs_hist(g, (const uint8_t *)ctx->bins.p, dof_arrays(ctx, g.D),
                              (const unsigned long long *)ctx->nfix.p, ctx->nfix_scale, (const PairTile *)tiles.p,
                              n_pairs, T, po, (int *)ctx->errw.p, st);
        ctx->launches++;
    }
    if (e == cudaSuccess) {
        for (int k = 0; k < n_pairs && e == cudaSuccess; k++) {
            const int b1 = g.bins[3 + dof_type(g1[k], g.nb, g.na)], b2 = g.bins[3 + dof_type(g2[k], g.nb, g.na)];
            e = cudaMemcpyAsync(counts + (int64_t)k * stride, (int64_t *)ctx->counts.p + (int64_t)k * pps * bm * bm,
                                (size_t)b1 * b2 * sizeof(int64_t), cudaMemcpyDeviceToHost, st);
        }
    }
    cudaStreamSynchronize(st);
    tiles.release();
    if (e != cudaSuccess) return fail(ctx, PG_ERR_CUDA, "pair count export: %s", cudaGetErrorString(e));
    return check_err_words(ctx);
}

PG_API int pg_dof_stats(pg_ctx *ctx, double *mn, double *mx, double *shift) {
    if (!ctx || !mn || !mx || !shift) return fail(ctx, PG_ERR_ARG, "null argument");
    if (!ctx->dofbuf.p || ctx->geo.D == 0) return fail(ctx, PG_ERR_ARG, "no preprocessing results");
    DofArrays d = dof_arrays(ctx, ctx->geo.D);
    const size_t b = (size_t)ctx->geo.D * sizeof(double);
    CK(cudaMemcpyAsync(mn, d.mn, b, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(mx, d.mx, b, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(shift, d.shift, b, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return PG_OK;
}

PG_API int pg_mist(pg_ctx *ctx, int n_dihedrals, const pg_par_body *body, pg_mist_edge *edges,
                   double totals[10]) {
    if (!ctx) return fail(nullptr, PG_ERR_ARG, "null context");
    ctx->err.clear();
    cudaGetLastError();  // an error left by an earlier failed call of this thread is not this call's
    if (!edges || !totals) return fail(ctx, PG_ERR_ARG, "null edges/totals");
    if (n_dihedrals < 0) return fail(ctx, PG_ERR_ARG, "n_dihedrals < 0");
    CK(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const int nb = n_dihedrals + 2, na = n_dihedrals + 1, nd = n_dihedrals, D = nb + na + nd;
    const ParLayout L = par_layout(n_dihedrals);
    std::vector<double> s1((size_t)D);
    // results come back through one pinned buffer: s1 | edge MI | from | to
    CK(ctx->ensure_hstage((size_t)D * (2 * sizeof(double) + 2 * sizeof(int)) + 64));
    double *h_s1 = (double *)ctx->hstage, *hmi = h_s1 + D;
    int *hf = (int *)(hmi + D), *ht = hf + D;
    CK(cudaEventRecord(ctx->ev[0], st));
    if (body) {
        const double *src[9] = {body->s1_b, body->s1_a, body->s1_d, body->bb, body->ba, body->bd, body->aa, body->ad, body->dd};
        const int64_t off[10] = {L.s1b, L.s1a, L.s1d, L.bb, L.ba, L.bd, L.aa, L.ad, L.dd, L.total};
        CK(ctx->par.ensure((size_t)L.total * sizeof(double)));
        CK(ctx->mi.ensure((size_t)D * D * sizeof(double)));
        for (int k = 0; k < 9; k++) {
            const int64_t n = off[k + 1] - off[k];
            if (n <= 0) continue;
            if (!src[k]) return fail(ctx, PG_ERR_ARG, "null body block %d", k);
            // host or device blocks: the copy direction comes from the pointers
            CK(cudaMemcpyAsync((double *)ctx->par.p + off[k], src[k], (size_t)n * sizeof(double), cudaMemcpyDefault,
                               st));
        }
        CK(launch_mi_from_par(n_dihedrals, (const double *)ctx->par.p, L, (double *)ctx->mi.p, st));
        ctx->launches++;
        ctx->resident = false;
    } else {
        if (!ctx->resident || ctx->geo.n_dih != n_dihedrals)
            return fail(ctx, PG_ERR_ARG, "no resident MI matrix for %d dihedrals", n_dihedrals);
    }
    CK(ctx->edges.ensure((size_t)D * (sizeof(double) + 2 * sizeof(int)) + 256));
    CK(ctx->mistscr.ensure(mist_scratch_bytes(D)));
    double *emi = (double *)ctx->edges.p;
    int *efrom = (int *)(emi + D), *eto = efrom + D;
    CK(cudaEventRecord(ctx->ev[1], st));
    CK(launch_mist_impl(D, nb, na, (const double *)ctx->mi.p, ctx->mistscr.p, emi, efrom, eto, st));
    ctx->launches++;
    CK(cudaEventRecord(ctx->ev[2], st));
    // the 1D entropies (s1_b | s1_a | s1_d lead the body layout)
    CK(cudaMemcpyAsync(h_s1, body ? (const double *)ctx->par.p + L.s1b : dof_arrays(ctx, D).s1,
                       (size_t)D * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (D > 1) {
        CK(cudaMemcpyAsync(hmi, emi, (size_t)(D - 1) * sizeof(double), cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(hf, efrom, (size_t)(D - 1) * sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(ht, eto, (size_t)(D - 1) * sizeof(int), cudaMemcpyDeviceToHost, st));
    }
    CK(cudaEventRecord(ctx->ev[3], st));
    CK(cudaStreamSynchronize(st));
    memcpy(s1.data(), h_s1, (size_t)D * sizeof(double));
    float ms[3];
    cudaEventElapsedTime(&ms[0], ctx->ev[0], ctx->ev[1]);
    cudaEventElapsedTime(&ms[1], ctx->ev[1], ctx->ev[2]);
    cudaEventElapsedTime(&ms[2], ctx->ev[2], ctx->ev[3]);
    ctx->timings[2] = ms[1];
    return mist_edges_to_user(ctx, n_dihedrals, hmi, hf, ht, s1.data(), edges, totals);
}

}  // extern "C"

// Device edge triples (MI, In DOF, Out DOF per step) -> pg_mist_edge records
// and the 10 totals, in get_PAR_MIST.cpp:279-287 and :663-765 order.
static int mist_edges_to_user(pg_ctx *ctx, int n_dihedrals, const double *hmi, const int *hf, const int *ht,
                              const double *s1, pg_mist_edge *edges, double totals[10]) {
    const int nb = n_dihedrals + 2, na = n_dihedrals + 1, nd = n_dihedrals, D = nb + na + nd;
    double tB = 0, tA = 0, tD = 0, tm = 0, tp[6] = {0, 0, 0, 0, 0, 0};
    for (int k = 0; k < nb; k++) tB += s1[k];
    for (int k = 0; k < na; k++) tA += s1[nb + k];
    for (int k = 0; k < nd; k++) tD += s1[nb + na + k];
    for (int s = 0; s < D - 1; s++) {
        if (ht[s] < 0 || hf[s] < 0) return fail(ctx, PG_ERR_DATA, "MIST step %d found no candidate", s);
        const int t1 = dof_type(hf[s], nb, na), t2 = dof_type(ht[s], nb, na);
        const int off1 = t1 == TB ? 0 : (t1 == TA ? nb : nb + na);
        const int off2 = t2 == TB ? 0 : (t2 == TA ? nb : nb + na);
        edges[s].type_in = t1;
        edges[s].type_out = t2;
        edges[s].index_in = hf[s] - off1 + 1;
        edges[s].index_out = ht[s] - off2 + 1;
        edges[s].mi = hmi[s];
        edges[s].left = D - 1 - s;
        edges[s].pad_ = 0;
        tm += hmi[s];
        const int lo = std::min(t1, t2), hi = std::max(t1, t2);
        tp[lo == 0 ? hi : (lo == 1 ? 2 + hi : 5)] += hmi[s];
    }
    totals[0] = tB;
    totals[1] = tA;
    totals[2] = tD;
    for (int q = 0; q < 6; q++) totals[3 + q] = tp[q];
    totals[9] = tB + tA + tD - tm;
    return PG_OK;
}

extern "C" {

PG_API int pg_last_timings(const pg_ctx *ctx, double ms[5]) {
    if (!ctx || !ms) return PG_ERR_ARG;
    for (int k = 0; k < 5; k++) ms[k] = ctx->timings[k];
    return PG_OK;
}
PG_API int64_t pg_launch_count(const pg_ctx *ctx) { return ctx ? ctx->launches : -1; }
PG_API int pg_last_form(const pg_ctx *ctx) { return ctx ? ctx->last_form : 0; }
PG_API void *pg_stream(const pg_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

PG_API int pg_synth_device(pg_ctx *ctx, const pg_synth_spec *spec, void *bonds, void *angles,
                           void *dihedrals, int64_t ld) {
    if (!ctx) return fail(nullptr, PG_ERR_ARG, "null context");
    if (!synth_spec_ok(spec) || !bonds || !angles || (spec->n_atoms > 3 && !dihedrals) || ld < spec->n_frames)
        return fail(ctx, PG_ERR_ARG, "bad synthetic spec or buffers");
    CK(cudaSetDevice(ctx->device));
    std::vector<float> lat;
    std::vector<int> sw, sw_off;
    size_t lb = 0, sb = 0;
    const size_t total = synth_scratch_bytes(spec, &lb, &sb, lat, sw, sw_off);
    DevBuf tmp;
    CK(tmp.ensure(total));
    char *base = (char *)tmp.p;
    cudaStream_t st = ctx->stream;
    if (!lat.empty()) CK(cudaMemcpyAsync(base, lat.data(), lat.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    int *dsw = (int *)(base + lb);
    if (!sw.empty()) CK(cudaMemcpyAsync(dsw, sw.data(), sw.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    int *doff = dsw + sw.size();
    CK(cudaMemcpyAsync(doff, sw_off.data(), sw_off.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    CK(launch_synth_dev(spec, bonds, angles, dihedrals ? dihedrals : angles, ld, (const float *)base, dsw, doff, st));
    ctx->launches++;
    CK(cudaStreamSynchronize(st));
    tmp.release();
    return PG_OK;
}

PG_API int pg_predict_pair_ms(pg_ctx *ctx, int n_dihedrals, int n_frames, const int bins[6], int form,
                              double *ms) {
    if (!ctx || !bins || !ms || n_dihedrals < 0 || n_frames < 1) return fail(ctx, PG_ERR_ARG, "bad arguments");
    if (form != PG_FORM_HIST && form != PG_FORM_ONEHOT && form != PG_FORM_AUTO)
        return fail(ctx, PG_ERR_ARG, "unknown form %d", form);
    CK(cudaSetDevice(ctx->device));
    SysGeom g{};
    g.n_dih = n_dihedrals;
    g.nb = g.n_dih + 2;
    g.na = g.n_dih + 1;
    g.nd = g.n_dih;
    g.D = g.nb + g.na + g.nd;
    g.F = n_frames;
    g.ldb = bins_ld(g.F);
    for (int k = 0; k < 6; k++) {
        if (bins[k] < 1 || (k >= 3 && bins[k] > PG_MAX_BINS_2D)) return fail(ctx, PG_ERR_ARG, "bad bin count");
        g.bins[k] = bins[k];
    }
    const int f = form == PG_FORM_AUTO ? autotune_form(g) : form;
    const double s = predict_pair_seconds(g, f);
    if (s < 0.0) return fail(ctx, PG_ERR_UNSUPPORTED, "no prediction for this form and geometry");
    *ms = s * 1e3;
    return PG_OK;
}

PG_API int pg_probe_smem_red_rate(pg_ctx *ctx, double *reductions_per_s) {
    if (!ctx || !reductions_per_s) return fail(ctx, PG_ERR_ARG, "null argument");
    CK(cudaSetDevice(ctx->device));
    int n_sm = 0;
    CK(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, ctx->device));
    int nl = 0;
    const double r = probe_smem_red_rate(n_sm, ctx->stream, &nl);
    ctx->launches += nl;
    if (r <= 0) return fail(ctx, PG_ERR_CUDA, "shared-memory reduction probe failed");
    *reductions_per_s = r;
    return PG_OK;
}

PG_API int pg_check_wait_timeout(pg_ctx *ctx, double limit_ms) {
    if (!ctx || !(limit_ms > 0.0) || limit_ms > 10000.0) return fail(ctx, PG_ERR_ARG, "limit_ms must be in (0, 10000]");
    ctx->err.clear();
    cudaGetLastError();  // an error left by an earlier failed call of this thread is not this call's
    CK(cudaSetDevice(ctx->device));
    int khz = 0;
    CK(cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, ctx->device));
    CK(ctx->errw.ensure(ERR_WORDS * sizeof(int)));
    CK(cudaMemsetAsync(ctx->errw.p, 0, ERR_WORDS * sizeof(int), ctx->stream));
    CK(launch_wait_timeout_probe((long long)(limit_ms * (khz > 0 ? khz : 2000000)), (int *)ctx->errw.p, ctx->stream));
    ctx->launches++;
    return check_err_words(ctx);
}

PG_API int pg_device_alloc(pg_ctx *ctx, size_t bytes, void **ptr) {
    if (!ctx || !ptr) return fail(ctx, PG_ERR_ARG, "null argument");
    CK(cudaSetDevice(ctx->device));
    CK(cudaMalloc(ptr, bytes));
    return PG_OK;
}
PG_API int pg_device_free(pg_ctx *ctx, void *ptr) {
    if (!ctx) return PG_ERR_ARG;
    CK(cudaSetDevice(ctx->device));
    CK(cudaFree(ptr));
    return PG_OK;
}
PG_API int pg_memcpy(pg_ctx *ctx, void *dst, const void *src, size_t bytes, int kind) {
    if (!ctx || kind < 1 || kind > 3) return fail(ctx, PG_ERR_ARG, "bad memcpy arguments");
    const cudaMemcpyKind k = kind == 1 ? cudaMemcpyHostToDevice : (kind == 2 ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice);
    CK(cudaMemcpyAsync(dst, src, bytes, k, ctx->stream));
    return PG_OK;
}
PG_API int pg_host_alloc_pinned(size_t bytes, void **ptr) {
    if (!ptr) return PG_ERR_ARG;
    cudaError_t e = cudaHostAlloc(ptr, bytes, cudaHostAllocDefault);
    if (e != cudaSuccess) return fail(nullptr, PG_ERR_NOMEM, "cudaHostAlloc(%zu): %s", bytes, cudaGetErrorString(e));
    return PG_OK;
}
PG_API int pg_host_free_pinned(void *ptr) {
    cudaError_t e = cudaFreeHost(ptr);
    return e == cudaSuccess ? PG_OK : fail(nullptr, PG_ERR_CUDA, "cudaFreeHost: %s", cudaGetErrorString(e));
}
PG_API int pg_synchronize(pg_ctx *ctx) {
    if (!ctx) return PG_ERR_ARG;
    CK(cudaStreamSynchronize(ctx->stream));
    return PG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- batches

namespace {

// Byte offsets of one system's device data inside the batch arena.
struct BatchLayout {
    SysGeom g;
    int prec = 0;
    int64_t ld = 0;
    size_t cols = 0, bins = 0, dof = 0, par = 0, mi = 0, mist = 0, edges = 0;
    bool own_cols = false;
};

size_t al256(size_t x) { return (x + 255) / 256 * 256; }

}  // namespace

static int validate_view(pg_ctx *ctx, const pg_bat_view *tv, int k) {
    if (tv->n_dihedrals < 0 || tv->n_frames < 1 || (tv->double_prec != 0 && tv->double_prec != 1) ||
        tv->ld < tv->n_frames || !tv->bonds || !tv->angles || (tv->n_dihedrals > 0 && !tv->dihedrals))
        return fail(ctx, PG_ERR_ARG, "system %d: invalid trajectory view", k);
    return PG_OK;
}

extern "C" {

PG_API int pg_entropy_batch(pg_ctx *ctx, int n_sys, const pg_bat_view *trajs, const int bins[6], int form,
                            pg_par_body *outs, pg_mist_edge *const *edges, double *totals) {
    if (!ctx) return fail(nullptr, PG_ERR_ARG, "null context");
    ctx->err.clear();
    cudaGetLastError();  // an error left by an earlier failed call of this thread is not this call's
    if (n_sys < 1 || !trajs || !bins) return fail(ctx, PG_ERR_ARG, "need n_sys >= 1 systems and bins");
    if (form < PG_FORM_AUTO || form > PG_FORM_ONEHOT) return fail(ctx, PG_ERR_ARG, "unknown form %d", form);
    for (int k = 0; k < 6; k++) {
        if (bins[k] < 1) return fail(ctx, PG_ERR_ARG, "bin count %d (index %d) < 1", bins[k], k);
        if (k >= 3 && bins[k] > PG_MAX_BINS_2D)
            return fail(ctx, PG_ERR_UNSUPPORTED, "2D bin count %d > %d", bins[k], PG_MAX_BINS_2D);
        if (k < 3 && bins[k] > 16384) return fail(ctx, PG_ERR_UNSUPPORTED, "1D bin count %d > 16384", bins[k]);
    }
    CK(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    ctx->resident = false;

    // The form of the batch: one form for every system, in one pair launch.
    // Automatically the one-hot form where the autotuner picks it for every
    // system (the batched one-hot launch runs every system's tiles together).
    bool onehot = form == PG_FORM_ONEHOT;
    {
        bool all_supported = true;
        std::vector<SysGeom> geos((size_t)n_sys);
        for (int s = 0; s < n_sys; s++) {
            int rc = validate_view(ctx, &trajs[s], s);
            if (rc) return rc;
            SysGeom g{};
            g.n_dih = trajs[s].n_dihedrals;
            g.nb = g.n_dih + 2;
            g.na = g.n_dih + 1;
            g.nd = g.n_dih;
            g.D = g.nb + g.na + g.nd;
            g.F = trajs[s].n_frames;
            for (int k = 0; k < 6; k++) g.bins[k] = bins[k];
            all_supported = all_supported && pairs_onehot_supported(g);
            geos[s] = g;
        }
        if (form == PG_FORM_ONEHOT && !all_supported)
            return fail(ctx, PG_ERR_UNSUPPORTED, "one-hot tensor-core form unsupported for a system of the batch");
        if (form == PG_FORM_AUTO) onehot = autotune_batch_form(geos) == PG_FORM_ONEHOT;
    }

    // ---- layout of every system inside one arena
    std::vector<BatchLayout> sys((size_t)n_sys);
    size_t off = 0;
    int maxF = 1, maxD = 1;
    for (int s = 0; s < n_sys; s++) {
        const pg_bat_view &v = trajs[s];
        int rc = validate_view(ctx, &v, s);
        if (rc) return rc;
        BatchLayout &L = sys[s];
        SysGeom &g = L.g;
        g.n_dih = v.n_dihedrals;
        g.nb = g.n_dih + 2;
        g.na = g.n_dih + 1;
        g.nd = g.n_dih;
        g.D = g.nb + g.na + g.nd;
        g.F = v.n_frames;
        g.ldb = bins_ld(g.F);
        for (int k = 0; k < 6; k++) g.bins[k] = bins[k];
        set_bin_layout(g, onehot ? PG_FORM_ONEHOT : PG_FORM_HIST);
        L.prec = v.double_prec;
        L.own_cols = !v.on_device;
        L.ld = v.on_device ? v.ld : v.n_frames;
        if (L.own_cols) {
            L.cols = off;
            off = al256(off + (size_t)g.D * g.F * elem_size(v.double_prec));
        }
        L.bins = off;
        off = al256(off + bins_bytes(g));
        L.dof = off;
        off = al256(off + dof_bytes(g.D));
        L.par = off;
        off = al256(off + (size_t)par_layout(g.n_dih).total * sizeof(double));
        L.mi = off;
        off = al256(off + (size_t)g.D * g.D * sizeof(double));
        L.mist = off;
        off = al256(off + mist_scratch_bytes(g.D));
        L.edges = off;
        off = al256(off + (size_t)g.D * (sizeof(double) + 2 * sizeof(int)));
        maxF = std::max(maxF, g.F);
        maxD = std::max(maxD, g.D);
    }
    if (prep_smem_bytes(sys[0].g) > 200 * 1024) return fail(ctx, PG_ERR_UNSUPPORTED, "1D bin counts too large");
    CK(ctx->batch.ensure(off));
    CK(ctx->errw.ensure(ERR_WORDS * sizeof(int)));
    {
        int rc0 = ensure_fix_table(ctx, maxF);
        if (rc0) return rc0;
    }
    char *arena = (char *)ctx->batch.p;
    const int bmax = bmax_of(sys[0].g);
    const bool h32 = use_hist32(sys[0].g);
    int T = 0, fc = 0, nst = 0;
    if (!pairs_hist_config(bmax, &T, &fc, &nst)) return fail(ctx, PG_ERR_UNSUPPORTED, "2D bins too large");

    // ---- descriptors and the concatenated tile list
    auto dofs_at = [&](const BatchLayout &L) { return dof_at(arena + L.dof, L.g.D); };
    std::vector<SysDesc> sd((size_t)n_sys);
    std::vector<MistDesc> md((size_t)n_sys);
    std::vector<PairTile> tiles;
    std::vector<int> tsys;
    for (int s = 0; s < n_sys; s++) {
        const BatchLayout &L = sys[s];
        sd[s].geo = L.g;
        sd[s].bins = (const uint8_t *)(arena + L.bins);
        sd[s].dof = dofs_at(L);
        sd[s].out.par = (double *)(arena + L.par);
        sd[s].out.mi = (double *)(arena + L.mi);
        sd[s].out.L = par_layout(L.g.n_dih);
        sd[s].out.counts = nullptr;
        sd[s].out.counts_bmax = 0;
        sd[s].lnN = log((double)L.g.F);
        md[s].D = L.g.D;
        md[s].nb = L.g.nb;
        md[s].na = L.g.na;
        md[s].mi = (const double *)(arena + L.mi);
        md[s].scratch = arena + L.mist;
        md[s].edge_mi = (double *)(arena + L.edges);
        md[s].edge_from = (int *)(md[s].edge_mi + L.g.D);
        md[s].edge_to = md[s].edge_from + L.g.D;
    }
    // tiles of the systems with the most frames (the longest tiles) first, so
    // that the short ones fill the tail of the launch
    std::vector<int> order((size_t)n_sys);
    for (int s = 0; s < n_sys; s++) order[s] = s;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return sys[a].g.F > sys[b].g.F; });
    for (int s : order) {
        if (onehot) break;  // the one-hot launch builds its own tile list
        std::vector<PairTile> t = h32 ? build_tiles32(sys[s].g.D) : build_tiles(sys[s].g.D, T);
        tiles.insert(tiles.end(), t.begin(), t.end());
        tsys.insert(tsys.end(), t.size(), s);
    }
    std::vector<SysGeom> gs((size_t)n_sys);
    for (int s = 0; s < n_sys; s++) gs[s] = sys[s].g;
    if (onehot) CK(ctx->ohbatch.ensure(pairs_onehot_batch_bytes(gs)));
    // preprocessing of all systems in one launch per input precision: CTA
    // k handles DOF map[k].y of system map[k].x
    std::vector<PrepDesc> pd((size_t)n_sys);
    std::vector<int2> pmap[2];
    for (int s = 0; s < n_sys; s++) {
        const BatchLayout &L = sys[s];
        const pg_bat_view &v = trajs[s];
        const size_t es = elem_size(v.double_prec);
        PrepDesc &p = pd[s];
        p.geo = L.g;
        if (L.own_cols) {
            const char *c = arena + L.cols;
            p.cols[0] = c;
            p.cols[1] = c + (size_t)L.g.nb * L.g.F * es;
            p.cols[2] = L.g.nd ? c + (size_t)(L.g.nb + L.g.na) * L.g.F * es : p.cols[1];
        } else {
            p.cols[0] = v.bonds;
            p.cols[1] = v.angles;
            p.cols[2] = v.dihedrals ? v.dihedrals : v.angles;
        }
        p.ld = L.ld;
        p.prec = L.prec;
        p.dof = dofs_at(L);
        p.bins = (uint8_t *)(arena + L.bins);
        for (int g = 0; g < L.g.D; g++) pmap[L.prec].push_back(make_int2(s, g));
    }
    const size_t mo_sd = 0, mo_md = al256(sizeof(SysDesc) * n_sys), mo_t = mo_md + al256(sizeof(MistDesc) * n_sys),
                 mo_ts = mo_t + al256(sizeof(PairTile) * std::max<size_t>(tiles.size(), 1)),
                 mo_pd = mo_ts + al256(sizeof(int) * std::max<size_t>(tsys.size(), 1)),
                 mo_m0 = mo_pd + al256(sizeof(PrepDesc) * n_sys),
                 mo_m1 = mo_m0 + al256(sizeof(int2) * std::max<size_t>(pmap[0].size(), 1)),
                 mo_end = mo_m1 + al256(sizeof(int2) * std::max<size_t>(pmap[1].size(), 1));
    CK(ctx->batchmeta.ensure(mo_end));
    char *meta = (char *)ctx->batchmeta.p;

    // the graph depends on the arena/descriptor addresses and geometry; it is
    // recaptured when any of them change
    std::vector<int64_t> key = {(int64_t)n_sys, (int64_t)(uintptr_t)arena, (int64_t)(uintptr_t)meta,
                                (int64_t)(uintptr_t)ctx->nfix.p, (int64_t)(uintptr_t)ctx->errw.p};
    size_t sb32 = 0;
    if (h32) {
        sb32 = pairs_hist32_scratch_bytes(bmax, pairs_hist32_grid((int64_t)tiles.size()));
        CK(ctx->scratch.ensure(sb32));
    }
    key.push_back((int64_t)ctx->nfix_max);
    key.push_back(h32 ? (int64_t)(uintptr_t)ctx->scratch.p : -1);
    key.push_back(sys[0].g.codes);
    key.push_back(sys[0].g.ilv);
    key.push_back(onehot ? (int64_t)(uintptr_t)ctx->ohbatch.p : -1);
    for (int k = 0; k < 6; k++) key.push_back(bins[k]);
    for (int s = 0; s < n_sys; s++) {
        const pg_bat_view &v = trajs[s];
        key.insert(key.end(), {v.n_dihedrals, v.n_frames, v.double_prec, v.on_device, v.ld,
                               v.on_device ? (int64_t)(uintptr_t)v.bonds : 0,
                               v.on_device ? (int64_t)(uintptr_t)v.angles : 0,
                               v.on_device ? (int64_t)(uintptr_t)v.dihedrals : 0});
    }
    const bool reuse = ctx->graph && key == ctx->graph_key;
    CK(cudaEventRecord(ctx->ev[0], st));
    if (!reuse) {
        CK(cudaMemcpyAsync(meta + mo_sd, sd.data(), sizeof(SysDesc) * n_sys, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(meta + mo_md, md.data(), sizeof(MistDesc) * n_sys, cudaMemcpyHostToDevice, st));
        if (!tiles.empty()) {
            CK(cudaMemcpyAsync(meta + mo_t, tiles.data(), sizeof(PairTile) * tiles.size(), cudaMemcpyHostToDevice, st));
            CK(cudaMemcpyAsync(meta + mo_ts, tsys.data(), sizeof(int) * tsys.size(), cudaMemcpyHostToDevice, st));
        }
        CK(cudaMemcpyAsync(meta + mo_pd, pd.data(), sizeof(PrepDesc) * n_sys, cudaMemcpyHostToDevice, st));
        for (int q = 0; q < 2; q++)
            if (!pmap[q].empty())
                CK(cudaMemcpyAsync(meta + (q ? mo_m1 : mo_m0), pmap[q].data(), sizeof(int2) * pmap[q].size(),
                                   cudaMemcpyHostToDevice, st));
        CK(cudaStreamSynchronize(st));  // host vectors go out of scope
        if (onehot) {
            // descriptors, row tables and n ln n tables of the one-hot launch
            std::vector<const uint8_t *> bp((size_t)n_sys);
            std::vector<DofArrays> dp((size_t)n_sys);
            std::vector<PairOut> op((size_t)n_sys);
            for (int s = 0; s < n_sys; s++) {
                bp[s] = sd[s].bins;
                dp[s] = sd[s].dof;
                op[s] = sd[s].out;
            }
            CK(prepare_pairs_onehot_batch(gs, bp, dp, op, ctx->ohbatch.p, ctx->ohbatch.n, st));
            ctx->launches += n_sys;  // one n ln n table per system
        }
    }
    // host columns -> arena (outside the graph: their source is the caller's)
    for (int s = 0; s < n_sys; s++) {
        const BatchLayout &L = sys[s];
        if (!L.own_cols) continue;
        const pg_bat_view &v = trajs[s];
        const size_t es = elem_size(v.double_prec), F = (size_t)v.n_frames;
        char *dst = arena + L.cols;
        const void *src[3] = {v.bonds, v.angles, v.dihedrals};
        const int cnt[3] = {L.g.nb, L.g.na, L.g.nd};
        for (int t = 0; t < 3; t++) {
            if (cnt[t] == 0) continue;
            if ((size_t)v.ld == F) {
                // pulled by SM loads where the GPU can read the host memory
                // (about 3x the copy engine's rate here), else the copy engine
                bool pulled = false;
                CK(h2d_copy(dst, src[t], (size_t)cnt[t] * F * es, st, &pulled));
                if (pulled) ctx->launches++;
            } else {
                CK(cudaMemcpy2DAsync(dst, F * es, src[t], (size_t)v.ld * es, F * es, cnt[t], cudaMemcpyHostToDevice,
                                     st));
            }
            dst += (size_t)cnt[t] * F * es;
        }
    }
    CK(cudaEventRecord(ctx->ev[1], st));
    if (!reuse) {
        if (ctx->graph) {
            cudaGraphExecDestroy(ctx->graph);
            ctx->graph = nullptr;
        }
        cudaGraph_t graph = nullptr;
        CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = cudaMemsetAsync(ctx->errw.p, 0, ERR_WORDS * sizeof(int), st);
        for (int q = 0; q < 2 && e == cudaSuccess; q++)
            e = launch_prep_batch(sys[0].g, (const PrepDesc *)(meta + mo_pd), (const int2 *)(meta + (q ? mo_m1 : mo_m0)),
                                  (int)pmap[q].size(), q, (int *)ctx->errw.p, st);
        for (int s = 0; s < n_sys && e == cudaSuccess; s++) {
            const BatchLayout &L = sys[s];
            e = cudaMemcpyAsync(arena + L.par, dofs_at(L).s1, (size_t)L.g.D * sizeof(double), cudaMemcpyDeviceToDevice,
                                st);
        }
        int oh_launches = 0;
        if (e == cudaSuccess && onehot)
            e = launch_pairs_onehot_batch(gs, ctx->ohbatch.p, (int *)ctx->errw.p, st, &oh_launches);
        else if (e == cudaSuccess)
            e = h32 ? launch_pairs_hist32_batch(bmax, sys[0].g.codes != 0, sys[0].g.ilv != 0,
                                                (const SysDesc *)(meta + mo_sd),
                                                (const PairTile *)(meta + mo_t),
                                                (const int *)(meta + mo_ts), (int64_t)tiles.size(),
                                                (const unsigned long long *)ctx->nfix.p, ctx->nfix_scale,
                                                (int *)ctx->errw.p, ctx->scratch.p, sb32, st)
                    : launch_pairs_hist_batch(bmax, (const SysDesc *)(meta + mo_sd), (const PairTile *)(meta + mo_t),
                                              (const int *)(meta + mo_ts), (int64_t)tiles.size(),
                                              (const unsigned long long *)ctx->nfix.p, ctx->nfix_scale,
                                              (int *)ctx->errw.p, T, st);
        if (e == cudaSuccess) e = launch_mist_batch((const MistDesc *)(meta + mo_md), n_sys, maxD, st);
        cudaError_t e2 = cudaStreamEndCapture(st, &graph);
        if (e == cudaSuccess) e = e2;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&ctx->graph, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            ctx->graph = nullptr;
            return fail(ctx, PG_ERR_CUDA, "batch graph capture: %s", cudaGetErrorString(e));
        }
        ctx->graph_key = key;
    }
    CK(cudaGraphLaunch(ctx->graph, st));
    // preps, pair kernel (+ the one-hot finalize), MIST
    ctx->launches += (pmap[0].empty() ? 0 : 1) + (pmap[1].empty() ? 0 : 1) + (onehot ? 3 : 2);
    CK(cudaEventRecord(ctx->ev[2], st));
    int rc = check_err_words(ctx);
    float ms[2];
    cudaEventElapsedTime(&ms[0], ctx->ev[0], ctx->ev[1]);
    cudaEventElapsedTime(&ms[1], ctx->ev[1], ctx->ev[2]);
    ctx->timings[0] = 0;
    ctx->timings[1] = ms[1];
    ctx->timings[2] = 0;
    ctx->timings[3] = ms[0];
    ctx->timings[4] = ms[0] + ms[1];
    if (rc) return rc;
    ctx->last_form = onehot ? PG_FORM_ONEHOT : PG_FORM_HIST;

    // ---- results to the caller
    for (int s = 0; s < n_sys; s++) {
        const BatchLayout &L = sys[s];
        const ParLayout PL = par_layout(L.g.n_dih);
        if (outs) {
            const int rcb = body_to_host(ctx, (const double *)(arena + L.par), PL, &outs[s], s);
            if (rcb) return rcb;
        }
        if ((edges && edges[s]) || totals) {
            const int D = L.g.D;
            std::vector<double> hmi((size_t)D), s1((size_t)D);
            std::vector<int> hf((size_t)D), ht((size_t)D);
            const double *emi = (const double *)(arena + L.edges);
            const int *ef = (const int *)(emi + D), *et = ef + D;
            if (D > 1) {
                CK(cudaMemcpyAsync(hmi.data(), emi, (size_t)(D - 1) * sizeof(double), cudaMemcpyDeviceToHost, st));
                CK(cudaMemcpyAsync(hf.data(), ef, (size_t)(D - 1) * sizeof(int), cudaMemcpyDeviceToHost, st));
                CK(cudaMemcpyAsync(ht.data(), et, (size_t)(D - 1) * sizeof(int), cudaMemcpyDeviceToHost, st));
            }
            CK(cudaMemcpyAsync(s1.data(), (const double *)(arena + L.par), (size_t)D * sizeof(double),
                               cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            std::vector<pg_mist_edge> tmp((size_t)std::max(D - 1, 1));
            double tt[10];
            pg_mist_edge *e = (edges && edges[s]) ? edges[s] : tmp.data();
            rc = mist_edges_to_user(ctx, L.g.n_dih, hmi.data(), hf.data(), ht.data(), s1.data(), e, tt);
            if (rc) return rc;
            if (totals) memcpy(totals + 10 * (size_t)s, tt, sizeof tt);
        }
    }
    CK(cudaStreamSynchronize(st));
    return PG_OK;
}

}  // extern "C"
