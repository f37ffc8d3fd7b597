// Form and layout choice for a geometry: a cost model of each pair kernel,
// calibrated on this GPU by short probe launches.
//
// Both forms walk a tile list with a fixed amount of work per tile and frame:
//   - the histogram kernels are persistent (one CTA per SM strides over the
//     tiles), so a launch takes ceil(tiles / grid) tile times;
//   - the one-hot kernel runs one CTA pair per 256 x 512 block of C, two
//     SMs each, so a launch takes ceil(tiles / (SMs / 2)) tile times.
// A tile time is t0 + t1 * F (t0: per-tile set-up and epilogue; t1: the frame
// loop). The tile counts come from the geometry (D and the bin counts: the
// one-hot form has one tile per 256 x 512 block of the (DOF, bin) space, so
// its tile count grows as B^2), the constants from two probe launches per
// kernel (F = 4,096 and 32,768 frames, random bins, at least one full wave of
// tiles), measured once per process, device and kernel variant. The form with
// the smaller predicted time is picked; when probing is not possible the
// measured crossover (one-hot up to 15 bins, from 4,096 frames) decides.
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

#include <algorithm>
#include <chrono>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "../../include/parent_gb300.h"
#include "pg_internal.h"

namespace pg {

std::vector<PairTile> build_tiles(int D, int T);
ParLayout par_layout(int n_dih);

namespace {

int sm_count_now() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 1;
    return n;
}

int bmax_of(const SysGeom &g) { return std::max(g.bins[3], std::max(g.bins[4], g.bins[5])); }

struct TileCost {
    double t0 = 0.0, t1 = 0.0;  // seconds per tile, seconds per tile and frame
    double call = 0.0;          // seconds per call before the kernel runs (host set-up)
    bool ok = false;
};

// key: (device, kernel variant: 0 one-hot, 1 + layout, bmax)
std::mutex g_mu;
std::map<std::tuple<int, int, int>, TileCost> g_costs;

uint64_t mix(uint64_t x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdULL;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ULL;
    return x ^ (x >> 33);
}

// A probe system: D DOFs x F frames of random bins below B in the layout of
// the geometry, per-DOF arrays of a valid run, outputs in scratch. Every
// buffer is freed when the probe is done.
struct Probe {
    SysGeom g{};
    std::vector<void *> bufs;
    uint8_t *bins = nullptr;
    DofArrays dof{};
    PairOut out{};
    unsigned long long *nfix = nullptr;
    void *scratch = nullptr;
    size_t scratch_bytes = 0;
    int *err = nullptr;
    cudaError_t alloc(void **p, size_t bytes) {
        cudaError_t e = cudaMalloc(p, std::max<size_t>(bytes, 256));
        if (e == cudaSuccess) bufs.push_back(*p);
        return e;
    }
    ~Probe() {
        for (void *p : bufs) cudaFree(p);
        cudaGetLastError();
    }
};

cudaError_t make_probe(Probe &p, const SysGeom &like, int D, int F, cudaStream_t st) {
    SysGeom &g = p.g;
    g = like;
    g.n_dih = (D - 3) / 3;
    g.nb = g.n_dih + 2;
    g.na = g.n_dih + 1;
    g.nd = g.n_dih;
    g.D = g.nb + g.na + g.nd;
    g.F = F;
    g.ldb = bins_ld(F);
    cudaError_t e;
    const size_t nbins = bins_bytes(g);
    if ((e = p.alloc((void **)&p.bins, nbins))) return e;
    // every DOF's bins below its own 2D bin count, at the positions the
    // layout puts them (DOF rows ldb apart, or frame-group interleaved)
    std::vector<uint8_t> h(nbins, 0);
    for (int d = 0; d < g.D; d++) {
        const uint64_t B = (uint64_t)g.bins[3 + dof_type(d, g.nb, g.na)];
        for (int f = 0; f < F; f++) {
            const uint64_t r = mix(((uint64_t)d << 32) ^ (uint64_t)f);
            store_bin(h.data(), g, d, f, (int)(r % B));
        }
    }
    if ((e = cudaMemcpyAsync(p.bins, h.data(), nbins, cudaMemcpyHostToDevice, st))) return e;
    double *dd = nullptr;
    if ((e = p.alloc((void **)&dd, dof_bytes(g.D)))) return e;
    if ((e = cudaMemsetAsync(dd, 0, dof_bytes(g.D), st))) return e;  // m2 0: no 16-bit folds
    std::vector<int> hi((size_t)g.D, 0);
    for (int d = 0; d < g.D; d++) hi[d] = g.bins[3 + dof_type(d, g.nb, g.na)];  // b2
    p.dof = dof_at(dd, g.D);
    if ((e = cudaMemcpyAsync(p.dof.b2, hi.data(), hi.size() * sizeof(int), cudaMemcpyHostToDevice, st))) return e;
    const ParLayout L = par_layout(g.n_dih);
    if ((e = p.alloc((void **)&p.out.par, (size_t)L.total * sizeof(double)))) return e;
    p.out.mi = nullptr;
    p.out.L = L;
    p.out.counts = nullptr;
    p.out.counts_bmax = 0;
    if ((e = p.alloc((void **)&p.nfix, ((size_t)F + 1) * sizeof(unsigned long long)))) return e;
    if ((e = launch_nlogn_fix_table(p.nfix, F, nlogn_fix_scale(F), st))) return e;
    if ((e = p.alloc((void **)&p.err, ERR_WORDS * sizeof(int)))) return e;
    if ((e = cudaMemsetAsync(p.err, 0, ERR_WORDS * sizeof(int), st))) return e;
    // host vectors go out of scope
    return cudaStreamSynchronize(st);
}

// Device seconds of one launch of the variant's kernel over the probe's tile
// list (after one untimed launch), the per-CTA tile count of that launch and
// the host seconds of the launch's set-up.
cudaError_t time_launch(Probe &p, int variant, cudaStream_t st, double *sec, double *waves, double *setup) {
    const SysGeom &g = p.g;
    const int sms = sm_count_now();
    cudaError_t e;
    std::vector<PairTile> tl;
    void *dtiles = nullptr;
    int T = 0, fc = 0, nst = 0;
    if (variant == 0) {
        const size_t sb = pairs_onehot_scratch_bytes(g);
        if ((e = p.alloc(&p.scratch, sb))) return e;
        p.scratch_bytes = sb;
        *waves = ceil((double)pairs_onehot_tiles(g) / std::max(1, sms / 2));
    } else {
        if (variant - 1 == 0) {
            if (!pairs_hist_config(bmax_of(g), &T, &fc, &nst)) return cudaErrorInvalidValue;
            tl = build_tiles(g.D, T);
        } else {
            tl = build_tiles32(g.D);
            const size_t sb = pairs_hist32_scratch_bytes(bmax_of(g), pairs_hist32_grid((int64_t)tl.size()));
            if ((e = p.alloc(&p.scratch, sb))) return e;
            p.scratch_bytes = sb;
        }
        if ((e = p.alloc(&dtiles, tl.size() * sizeof(PairTile)))) return e;
        if ((e = cudaMemcpyAsync(dtiles, tl.data(), tl.size() * sizeof(PairTile), cudaMemcpyHostToDevice, st)))
            return e;
        const int64_t grid = std::min<int64_t>((int64_t)tl.size(), sms);
        *waves = ceil((double)tl.size() / (double)grid);
    }
    const double fix = nlogn_fix_scale(g.F);
    OnehotRun run;
    *setup = 0.0;
    if (variant == 0) {
        const auto t0 = std::chrono::steady_clock::now();
        if ((e = onehot_setup(g, p.bins, p.dof, p.out, st, p.scratch, p.scratch_bytes, &run))) return e;
        *setup = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    auto launch = [&]() -> cudaError_t {
        if (variant == 0) return onehot_run(run, p.err, st);
        if (variant - 1 == 0)
            return launch_pairs_hist(g, p.bins, p.dof, p.nfix, fix, (const PairTile *)dtiles, (int64_t)tl.size(), T,
                                     p.out, p.err, st);
        return launch_pairs_hist32(g, p.bins, p.dof, p.nfix, fix, (const PairTile *)dtiles, (int64_t)tl.size(),
                                   p.out, p.err, p.scratch, p.scratch_bytes, st);
    };
    if ((e = launch())) return e;
    cudaEvent_t a, b;
    if ((e = cudaEventCreate(&a))) return e;
    if ((e = cudaEventCreate(&b))) {
        cudaEventDestroy(a);
        return e;
    }
    cudaEventRecord(a, st);
    e = launch();
    cudaEventRecord(b, st);
    if (e == cudaSuccess) e = cudaEventSynchronize(b);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    *sec = ms * 1e-3;
    return e;
}

// t0, t1 of a kernel variant from two probe lengths
TileCost calibrate(const SysGeom &like, int variant) {
    TileCost c;
    const int sms = sm_count_now();
    int D;
    if (variant == 0) {
        // at least one full wave of CTA pairs: R = D B rows, tiles ~ R^2 / (2 256 512)
        const int B = bmax_of(like);
        const double R = sqrt(2.0 * 256.0 * 512.0 * (sms / 2) * 1.2);
        D = std::max(96, (int)ceil(R / B));
    } else {
        D = 3 * 60;  // 180 DOFs: ~2 waves of 32-slot tiles, ~7 of 16-slot tiles on 152 SMs
    }
    D = (D + 2) / 3 * 3;
    cudaStream_t st = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        return c;
    }
    const int Fs[2] = {4096, 32768};
    double t[2] = {0, 0}, setup = 0.0;
    bool ok = true;
    for (int k = 0; k < 2 && ok; k++) {
        Probe p;
        double sec = 0, waves = 1, su = 0;
        ok = make_probe(p, like, D, Fs[k], st) == cudaSuccess &&
             time_launch(p, variant, st, &sec, &waves, &su) == cudaSuccess;
        t[k] = sec / std::max(1.0, waves);
        setup = k == 0 ? su : std::min(setup, su);
    }
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    cudaGetLastError();
    if (!ok || t[1] <= 0.0) return c;
    c.t1 = std::max(0.0, (t[1] - t[0]) / (Fs[1] - Fs[0]));
    c.t0 = std::max(0.0, t[0] - c.t1 * Fs[0]);
    c.call = setup;
    c.ok = true;
    return c;
}

TileCost cost_of(const SysGeom &g, int variant) {
    int dev = 0;
    cudaGetDevice(&dev);
    // the one-hot tile costs the same at any bin count; histogram tiles
    // depend on the layout and the bin count
    const auto key = std::make_tuple(dev, variant, variant == 0 ? 0 : bmax_of(g));
    {
        std::lock_guard<std::mutex> lock(g_mu);
        auto it = g_costs.find(key);
        if (it != g_costs.end()) return it->second;
    }
    const TileCost c = calibrate(g, variant);
    std::lock_guard<std::mutex> lock(g_mu);
    g_costs[key] = c;
    return c;
}

// the bin layout a histogram-form run of g writes and reads
SysGeom as_hist(const SysGeom &g, int layout) {
    SysGeom h = g;
    h.codes = layout_codes(layout, bmax_of(g));
    h.ilv = layout_ilv(layout);
    return h;
}
SysGeom as_onehot(const SysGeom &g) {
    SysGeom h = g;
    h.codes = 0;
    h.ilv = 0;
    return h;
}

bool fallback_onehot(const SysGeom &g) {
    return pairs_onehot_supported(g) && bmax_of(g) <= 15 && g.F >= 4096;
}

bool autotune_enabled() {
    const char *e = getenv("PG_AUTOTUNE");
    return !(e && atoi(e) == 0);
}

}  // namespace

// The histogram layout, from measured pair-kernel times at 2,994 DOFs x
// 100,000 frames: the streamed 32-slot kernel up to 50 2D bins (93.0 ms at 50
// bins against 116.3 ms for the 16-slot kernel and 116.3 ms for the ring-fed
// 32-slot kernel; 76.9 against 79.7 ms at 30 bins), the 16-slot kernel above
// (its 32-bit counters reach 218 bins). PG_HIST_SLOTS=16 forces the 16-slot
// layout, PG_HIST_SLOTS=32 the ring-fed 32-slot one, PG_HIST_STREAM=0 keeps
// the streamed one off.
int hist_layout(const SysGeom &g) {
    const int bm = bmax_of(g);
    const char *e = getenv("PG_HIST_SLOTS");
    const char *st = getenv("PG_HIST_STREAM");
    if (e && atoi(e) == 16) return HIST16;
    if (e && atoi(e) == 32) return pairs_hist32_supported(bm) ? HIST32_RING : HIST16;
    if (st && atoi(st) == 0) return pairs_hist32_wide(bm) ? HIST32_RING : HIST16;
    return pairs_hist32_supported(bm) ? HIST32_STREAM : HIST16;
}

int layout_codes(int layout, int bmax) { return layout != HIST16 && !pairs_hist32_wide(bmax) ? 1 : 0; }
int layout_ilv(int layout) { return layout == HIST32_STREAM ? 1 : 0; }

// Predicted pair-kernel seconds of a geometry in a form (PG_FORM_HIST with
// the layout hist_layout picks, or PG_FORM_ONEHOT), or < 0 if unknown.
double predict_pair_seconds(const SysGeom &g, int form) {
    const int sms = sm_count_now();
    if (form == PG_FORM_ONEHOT) {
        if (!pairs_onehot_supported(g)) return -1.0;
        const SysGeom h = as_onehot(g);
        const TileCost c = cost_of(h, 0);
        if (!c.ok) return -1.0;
        const double waves = ceil((double)pairs_onehot_tiles(h) / std::max(1, sms / 2));
        return c.call + waves * (c.t0 + c.t1 * g.F);
    }
    const int layout = hist_layout(g);
    const SysGeom h = as_hist(g, layout);
    const TileCost c = cost_of(h, 1 + (layout == HIST16 ? 0 : layout));
    if (!c.ok) return -1.0;
    int64_t tiles;
    if (layout == HIST16) {
        int T = 0, fc = 0, nst = 0;
        if (!pairs_hist_config(bmax_of(g), &T, &fc, &nst)) return -1.0;
        tiles = (int64_t)build_tiles(g.D, T).size();
    } else {
        tiles = (int64_t)build_tiles32(g.D).size();
    }
    const int64_t grid = std::max<int64_t>(1, std::min<int64_t>(tiles, sms));
    return ceil((double)tiles / (double)grid) * (c.t0 + c.t1 * g.F);
}

// The form for PG_FORM_AUTO: the one with the smaller predicted pair-kernel
// time (PG_AUTOTUNE=0: the fixed crossover). Only geometries the one-hot form
// supports and where it can win are probed: from 24 bins up one update costs
// it 2 x 24^2 FP8 FLOPs, more than the histogram kernels' rate allows at the
// tensor cores' peak.
int autotune_form(const SysGeom &g) {
    if (!pairs_onehot_supported(g)) return PG_FORM_HIST;
    if (bmax_of(g) > 24) return PG_FORM_HIST;
    if (!autotune_enabled()) return fallback_onehot(g) ? PG_FORM_ONEHOT : PG_FORM_HIST;
    const double th = predict_pair_seconds(g, PG_FORM_HIST), to = predict_pair_seconds(g, PG_FORM_ONEHOT);
    if (th < 0.0 || to < 0.0) return fallback_onehot(g) ? PG_FORM_ONEHOT : PG_FORM_HIST;
    return to < th ? PG_FORM_ONEHOT : PG_FORM_HIST;
}

// The same choice for a batch run in one launch: summed tile work of all
// systems over the launch's concurrency.
int autotune_batch_form(const std::vector<SysGeom> &gs) {
    double th = 0.0, to = 0.0;
    const int sms = sm_count_now();
    for (const SysGeom &g : gs) {
        if (!pairs_onehot_supported(g) || bmax_of(g) > 24) return PG_FORM_HIST;
    }
    if (!autotune_enabled()) {
        for (const SysGeom &g : gs)
            if (!fallback_onehot(g)) return PG_FORM_HIST;
        return PG_FORM_ONEHOT;
    }
    for (const SysGeom &g : gs) {
        const int layout = hist_layout(g);
        const TileCost ch = cost_of(as_hist(g, layout), 1 + (layout == HIST16 ? 0 : layout));
        const TileCost co = cost_of(as_onehot(g), 0);
        if (!ch.ok || !co.ok) {
            for (const SysGeom &x : gs)
                if (!fallback_onehot(x)) return PG_FORM_HIST;
            return PG_FORM_ONEHOT;
        }
        int64_t tiles;
        if (layout == HIST16) {
            int T = 0, fc = 0, nst = 0;
            pairs_hist_config(bmax_of(g), &T, &fc, &nst);
            tiles = (int64_t)build_tiles(g.D, T).size();
        } else {
            tiles = (int64_t)build_tiles32(g.D).size();
        }
        // one launch for the whole batch (its set-up runs once, outside the
        // replayed graph)
        th += (double)tiles * (ch.t0 + ch.t1 * g.F) / sms;
        to += (double)pairs_onehot_tiles(as_onehot(g)) * (co.t0 + co.t1 * g.F) / std::max(1, sms / 2);
    }
    return to < th ? PG_FORM_ONEHOT : PG_FORM_HIST;
}

}  // namespace pg
