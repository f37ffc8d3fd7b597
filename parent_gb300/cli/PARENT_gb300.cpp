// Drop-in for PARENT.x (src/PARENT/PARENT.cpp): same argv, same .bat input,
// same .par output, computed on one GPU through the parent_gb300 C ABI.
//   PARENT_gb300 input.bat entropy.par b1D a1D d1D b2D a2D d2D
//
// Checkpoint/resume (the reference has none): with PG_SHARDS=K (K >= 2) the
// pair work runs as K shards (pg_entropy_shard); after each one the summed
// body so far is written to PG_CHECKPOINT (default entropy.par.ckpt), and a
// rerun with the same input, bins and K continues after the last finished
// shard. Shard sums are exact, so the .par is identical to a one-pass run.
// PG_STOP_AFTER_SHARDS=n ends the run (exit code 3) after n shards of this
// invocation, to exercise the resume path.
//
// The .bat columns are read straight into device memory (pg_bat_read_device);
// PG_BAT_READ=host reads them into pinned host memory instead.
#include <stdint.h>
#include <stdio.h>
#include <sys/stat.h>

#include <algorithm>
#include <string>
#include <vector>

#include "common.h"

namespace {

constexpr char kMagic[8] = {'P', 'G', 'C', 'K', 'P', 'T', '1', 0};

struct CkptHeader {
    char magic[8];
    int32_t n_dih, bins[6], shards, next_shard;
    int64_t n_frames, input_bytes, body_len;
};

int64_t file_bytes(const char *path) {
    struct stat st;
    return stat(path, &st) == 0 ? (int64_t)st.st_size : -1;
}

bool header_matches(const CkptHeader &h, const CkptHeader &want) {
    if (memcmp(h.magic, kMagic, 8) != 0) return false;
    for (int k = 0; k < 6; k++)
        if (h.bins[k] != want.bins[k]) return false;
    return h.n_dih == want.n_dih && h.shards == want.shards && h.n_frames == want.n_frames &&
           h.input_bytes == want.input_bytes && h.body_len == want.body_len && h.next_shard >= 0 &&
           h.next_shard <= h.shards;
}

// Loads a matching checkpoint into body; returns the next shard (0 if none).
int load_checkpoint(const std::string &path, const CkptHeader &want, std::vector<double> &body) {
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) return 0;
    CkptHeader h;
    int next = 0;
    if (fread(&h, sizeof h, 1, f) == 1 && header_matches(h, want) &&
        fread(body.data(), sizeof(double), body.size(), f) == body.size())
        next = h.next_shard;
    else
        std::fill(body.begin(), body.end(), 0.0);
    fclose(f);
    return next;
}

// Writes the checkpoint next to its final name and renames it into place, so
// an interruption never leaves a torn file.
bool save_checkpoint(const std::string &path, CkptHeader h, int next, const std::vector<double> &body) {
    h.next_shard = next;
    const std::string tmp = path + ".tmp";
    FILE *f = fopen(tmp.c_str(), "wb");
    if (!f) return false;
    bool ok = fwrite(&h, sizeof h, 1, f) == 1 && fwrite(body.data(), sizeof(double), body.size(), f) == body.size();
    ok = (fclose(f) == 0) && ok;
    return ok && rename(tmp.c_str(), path.c_str()) == 0;
}

}  // namespace

static const char *kUsage =
    " input.bat entropy.par #bondsbins1D #anglesbins1D #dihedralsbins1D #bondsbins2D "
    "#anglesbins2D #dihedralsbins2D\n";

int main(int argc, char **argv) {
    const double t1 = wall_seconds();
    if (argc != 9) {  // PARENT.cpp:190, :241-244
        fprintf(stderr, "USAGE: %s%s", argv[0], kUsage);
        return 1;
    }
    if (last_ext(argv[1]) != "bat" || last_ext(argv[2]) != "par") {  // PARENT.cpp:207-210
        fprintf(stderr, "USAGE: %s%s", argv[0], kUsage);
        return 1;
    }
    static const char *what[6] = {"1D bonds", "1D angles", "1D dihedrals", "2D bonds", "2D angles", "2D dihedrals"};
    int bins[6];
    for (int k = 0; k < 6; k++) {  // PARENT.cpp:211-234
        if (sscanf(argv[3 + k], "%d", &bins[k]) != 1) {
            fprintf(stderr, "ERROR: Could not read number of bins for %s from command line! Aborting\n", what[k]);
            return 1;
        }
    }
    const int form = env_form();
    if (form < 0) {
        fprintf(stderr, "ERROR: PG_FORM must be auto, hist or onehot\n");
        return 1;
    }
    printf("Reading file %s .\n", argv[1]);
    pg_bat *bat = nullptr;
    // the columns go straight to the device (records streamed up and
    // transposed there); PG_BAT_READ=host transposes on the host instead
    const char *eread = getenv("PG_BAT_READ");
    const bool host_read = eread && strcmp(eread, "host") == 0;
    if ((host_read ? pg_bat_read(argv[1], &bat) : pg_bat_read_device(argv[1], env_device(), &bat)) != PG_OK) {
        fprintf(stderr, "AN ERROR HAS OCCURED WHILE READING THE HEADER OF THE FILE %s . QUITTING PROGRAM.\n", argv[1]);
        return 1;
    }
    const int nd = pg_bat_n_dihedrals(bat), nb = nd + 2, na = nd + 1;
    pg_bat_view view;
    pg_bat_view_of(bat, &view);
    printf("%s specs:\nPrecision: %s #Atoms: %d #Frames: %d\n", argv[1],
           view.double_prec == 1 ? "double" : "single", nd + 3, view.n_frames);
    pg_ctx *ctx = nullptr;
    if (pg_create(&ctx, env_device()) != PG_OK) {
        fprintf(stderr, "ERROR: %s\n", pg_last_global_error());
        pg_bat_free(bat);
        return 1;
    }
    // the whole .par body in one buffer, blocks in body order
    const size_t sz[9] = {(size_t)nb, (size_t)na, (size_t)nd, (size_t)nb * (nb - 1) / 2, (size_t)nb * na,
                          (size_t)nb * nd, (size_t)na * (na - 1) / 2, (size_t)na * nd,
                          (size_t)nd * (nd > 0 ? nd - 1 : 0) / 2};
    size_t total = 0;
    for (size_t z : sz) total += z;
    std::vector<double> flat(total, 0.0), part;
    auto body_over = [&](std::vector<double> &v) {
        double *p[9];
        size_t o = 0;
        for (int k = 0; k < 9; k++) {
            p[k] = v.data() + o;
            o += sz[k];
        }
        return pg_par_body{p[0], p[1], p[2], p[3], p[4], p[5], p[6], p[7], p[8]};
    };
    pg_par_body body = body_over(flat);
    const double t2 = wall_seconds();
    const char *es = getenv("PG_SHARDS");
    const int shards = es ? atoi(es) : 1;
    int rc = PG_OK;
    std::string ckpt;
    if (shards >= 2) {
        if (form == PG_FORM_ONEHOT) {
            fprintf(stderr, "ERROR: PG_SHARDS needs the histogram form\n");
            pg_destroy(ctx);
            pg_bat_free(bat);
            return 1;
        }
        const char *ec = getenv("PG_CHECKPOINT");
        ckpt = ec ? ec : std::string(argv[2]) + ".ckpt";
        CkptHeader h{};
        memcpy(h.magic, kMagic, 8);
        h.n_dih = nd;
        for (int k = 0; k < 6; k++) h.bins[k] = bins[k];
        h.shards = shards;
        h.n_frames = view.n_frames;
        h.input_bytes = file_bytes(argv[1]);
        h.body_len = (int64_t)total;
        const int first = load_checkpoint(ckpt, h, flat);
        if (first > 0) printf("Resuming from %s: %d of %d shards done.\n", ckpt.c_str(), first, shards);
        const char *estop = getenv("PG_STOP_AFTER_SHARDS");
        const int stop_after = estop ? atoi(estop) : -1;
        part.assign(total, 0.0);
        pg_par_body pb = body_over(part);
        for (int s = first; s < shards && rc == PG_OK; s++) {
            rc = pg_entropy_shard(ctx, &view, bins, form, s, shards, &pb);
            if (rc != PG_OK) break;
            for (size_t i = 0; i < total; i++) flat[i] += part[i];  // disjoint entries: exact
            if (!save_checkpoint(ckpt, h, s + 1, flat)) {
                fprintf(stderr, "ERROR: could not write the checkpoint %s\n", ckpt.c_str());
                rc = PG_ERR_IO;
                break;
            }
            printf("Shard %d of %d done (checkpoint %s).\n", s + 1, shards, ckpt.c_str());
            if (stop_after > 0 && s + 1 - first >= stop_after && s + 1 < shards) {
                printf("Stopping after %d shard(s) as requested.\n", stop_after);
                pg_destroy(ctx);
                pg_bat_free(bat);
                return 3;
            }
        }
    } else {
        rc = pg_entropy(ctx, &view, bins, form, &body);
    }
    if (rc != PG_OK) {
        fprintf(stderr, "ERROR: %s\n", pg_last_error(ctx));
        pg_destroy(ctx);
        pg_bat_free(bat);
        return 1;
    }
    double ms[5];
    pg_last_timings(ctx, ms);
    printf("GPU form: %s; device time: preprocessing %.3f ms, pairs %.3f ms, copies %.3f ms\n",
           pg_last_form(ctx) == PG_FORM_ONEHOT ? "onehot" : "hist", ms[0], ms[1], ms[3]);
    const double t3 = wall_seconds();
    rc = pg_par_write(argv[2], bat, bins, &body);
    if (rc != PG_OK) fprintf(stderr, "AN ERROR HAS OCCURED WHILE WRITING THE FILE %s .\n", argv[2]);
    if (rc == PG_OK && !ckpt.empty()) remove(ckpt.c_str());
    const double t4 = wall_seconds();
    printf("Initialization + readin time: %g\n", t2 - t1);
    printf("Calculation time: %g\n", t3 - t2);
    printf("Output time: %g\n", t4 - t3);
    printf("Total execution time: %g\n", t4 - t1);
    pg_destroy(ctx);
    pg_bat_free(bat);
    if (rc == PG_OK) printf("PROGRAM FINISHED SUCCESSFULLY.\n");
    return rc == PG_OK ? 0 : 1;
}
