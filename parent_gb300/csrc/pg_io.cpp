// File formats of the reference suite, host side:
//   .bat  read_BAT_header / read_BAT_frame   (io_binary.cpp:107-200, :281-368)
//         write_BAT_header / write_BAT_frame (io_binary.cpp:43-102, :203-278)
//   .par  write_PAR_header / write_PAR_body  (io_binary.cpp:371-442, :606-631)
//         read_PAR_header / read_PAR_body    (io_binary.cpp:446-673)
//   text  get_PAR_MIE (get_PAR_MIE.cpp:109-199), get_PAR_MIST (get_PAR_MIST.cpp:667-765),
//         get_PAR_info (get_PAR_info.cpp:64-79)
// The .bat body is frame-major; it is transposed into DOF-major columns kept
// in the file's own precision, which is the layout the device kernels read:
// on the host (pg_bat_read, pinned memory) or on the device (pg_bat_read_device:
// raw records are streamed up and transposed by a kernel).
#include <cuda_runtime.h>
#include <errno.h>
#include <fcntl.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <functional>
#include <string>
#include <thread>
#include <vector>

#include "../../include/parent_gb300.h"
#include "pg_fmt.h"

namespace {

}  // namespace

namespace pg {
void set_global_error(const char *msg);
int mie_lines_device(pg_ctx *ctx, int nd, const pg_par_body *b, const std::function<bool(const char *, size_t)> &sink);
cudaError_t launch_bat_transpose(const uint8_t *raw, int nf, int64_t rec, int off0, int es, int n_dih,
                                 uint8_t *cols, int64_t ld, int64_t f0, cudaStream_t st);
}

namespace {

// Records the message for pg_last_global_error and prints it to stderr, as
// the reference's io library does.
int ioerr(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    pg::set_global_error(buf);
    fprintf(stderr, "%s\n", buf);
    return code;
}

}  // namespace

namespace pg {

// The header field checks of read_BAT_header (io_binary.cpp:127-145) and
// read_PAR_header (io_binary.cpp:477-519, :554-591), with the reference's
// messages on stderr. They return PG_OK or PG_ERR_FORMAT.
int check_bat_fields(int version, int prec, int n_dih, int n_frames) {
    if (version < 0) return ioerr(PG_ERR_FORMAT, "ERROR: FILE HEADER CORRUPTED. VERSION NUMBER (%d) < 0!", version);
    if (prec != 0 && prec != 1)
        return ioerr(PG_ERR_FORMAT, "ERROR: FILE HEADER CORRUPTED. DOUBLE PRECISION VALUE (%d) NEITHER 0 NOR 1!", prec);
    if (n_dih > 19997)
        fprintf(stderr, "WARNING: %d ATOMS DECLARED IN THE FILE HEADER (CORRUPTED?). THIS WILL LEAD TO LARGE OUTPUT.\n",
                n_dih + 3);
    if (n_dih < 0) return ioerr(PG_ERR_FORMAT, "ERROR: FILE HEADER CORRUPTED. NUMBER OF DIHEDRALS (%d) < 0!", n_dih);
    if (n_frames < 1) return ioerr(PG_ERR_FORMAT, "ERROR: FILE HEADER CORRUPTED. NUMBER OF FRAMES (%d) < 1!", n_frames);
    return PG_OK;
}

// bins in file order: b1D a1D d1D b2D a2D d2D
int check_par_fields(int version, int prec, int n_dih, int n_frames, const int bins[6]) {
    const int rc = check_bat_fields(version, prec, n_dih, n_frames);
    if (rc) return rc;
    static const char *nm[6] = {"BONDS IN 1D", "ANGLES IN 1D", "DIHEDRALS IN 1D", "BONDS IN 2D", "ANGLES IN 2D",
                                "DIHEDRALS IN 2D"};
    for (int k = 0; k < 6; k++)
        if (bins[k] < 1) return ioerr(PG_ERR_FORMAT, "ERROR: FILE HEADER CORRUPTED. NUMBER BINS FOR %s (%d) < 1!", nm[k], bins[k]);
    return PG_OK;
}

// one dihedral entry of a .par header (atoms, type, parent)
int check_par_dihedral(const int d[6]) {
    for (int k = 0; k < 4; k++)
        if (d[k] < 1) return ioerr(PG_ERR_FORMAT, "ERROR: FILE HEADER CORRUPTED. DIHEDRAL ID < 1 !");
    if (!(d[4] == 1 || d[4] == 0 || d[4] == -1))
        return ioerr(PG_ERR_FORMAT, "ERROR: FILE HEADER CORRUPTED. DIHEDRAL TYPE NEITHER 0, 1 NOR -1 !");
    if (d[5] < -1) return ioerr(PG_ERR_FORMAT, "ERROR: FILE HEADER CORRUPTED. DIHEDRAL IS PHASEANGLE OF A DIHEDRAL WITH NEGATIVE ID !");
    return PG_OK;
}

}  // namespace pg

namespace {

struct Header {
    int version = 3, double_prec = 1, n_dih = 0, n_frames = 0;
    std::vector<std::string> residues, atoms, molecules;
    std::vector<int> resnums;
    std::vector<int> dih;  // 6 per dihedral
    std::vector<float> masses;
};

bool rd(FILE *f, void *p, size_t n) { return fread(p, 1, n, f) == n; }
bool wr(FILE *f, const void *p, size_t n) { return fwrite(p, 1, n, f) == n; }

std::string cstr(const char *p, size_t n) {
    size_t k = 0;
    while (k < n && p[k]) k++;
    return std::string(p, k);
}

// atom block as write_BAT_header / write_PAR_header emit it: "%.7s" into 8
// zeroed bytes, int, "%.7s" into 8 zeroed bytes, "%.30s" into 31 zeroed bytes
bool write_atoms(FILE *f, const Header &h) {
    for (int i = 0; i < h.n_dih + 3; i++) {
        char b8[8], b31[31];
        memset(b8, 0, 8);
        strncpy(b8, h.residues[i].c_str(), 7);
        if (!wr(f, b8, 8) || !wr(f, &h.resnums[i], 4)) return false;
        memset(b8, 0, 8);
        strncpy(b8, h.atoms[i].c_str(), 7);
        if (!wr(f, b8, 8)) return false;
        memset(b31, 0, 31);
        strncpy(b31, h.molecules[i].c_str(), 30);
        if (!wr(f, b31, 31)) return false;
    }
    return true;
}

bool read_atoms(FILE *f, Header &h) {
    const int n = h.n_dih + 3;
    h.residues.resize(n);
    h.atoms.resize(n);
    h.molecules.resize(n);
    h.resnums.resize(n);
    for (int i = 0; i < n; i++) {
        char b8[8], b31[31];
        if (!rd(f, b8, 8)) return false;
        h.residues[i] = cstr(b8, 8);
        if (!rd(f, &h.resnums[i], 4)) return false;
        if (!rd(f, b8, 8)) return false;
        h.atoms[i] = cstr(b8, 8);
        if (!rd(f, b31, 31)) return false;
        h.molecules[i] = cstr(b31, 31);
    }
    return true;
}

void synthetic_header(Header &h) {
    const int n = h.n_dih + 3;
    h.residues.assign(n, "SYN");
    h.atoms.resize(n);
    h.molecules.assign(n, "synthetic_chain");
    h.resnums.resize(n);
    h.masses.assign(n, 12.011f);
    for (int i = 0; i < n; i++) {
        h.atoms[i] = "C" + std::to_string(i + 1);
        h.resnums[i] = i / 10 + 1;
    }
    h.dih.resize((size_t)6 * h.n_dih);
    for (int i = 0; i < h.n_dih; i++) {  // linear chain: dihedral i = atoms i+1..i+4 (1-based)
        for (int k = 0; k < 4; k++) h.dih[6 * i + k] = i + 1 + k;
        h.dih[6 * i + 4] = 0;
        h.dih[6 * i + 5] = -1;
    }
}

}  // namespace

struct pg_bat {
    Header h;
    void *cols = nullptr;  // DOF-major, bonds | angles | dihedrals; host (pinned or not) or device
    bool pinned = false;
    int device = -1;       // >= 0: cols is device memory on this device
    int64_t ld = 0;        // elements between columns
    size_t bytes = 0;
};

struct pg_par {
    Header h;
    int bins[6] = {0, 0, 0, 0, 0, 0};
    std::vector<double> body;
    int64_t off[10];
};

static void layout(int nd_, int64_t off[10]) {
    const int64_t nb = nd_ + 2, na = nd_ + 1, nd = nd_;
    const int64_t sz[9] = {nb, na, nd, nb * (nb - 1) / 2, nb * na, nb * nd, na * (na - 1) / 2, na * nd, nd * (nd - 1) / 2};
    off[0] = 0;
    for (int k = 0; k < 9; k++) off[k + 1] = off[k] + sz[k];
}

extern "C" {

// Reads the .bat header (read_BAT_header, io_binary.cpp:107-200) with its
// checks; leaves `f` at the first frame record.
static int read_bat_header(FILE *f, Header &h, const char *path) {
    if (!rd(f, &h.version, 4) || !rd(f, &h.double_prec, 4) || !rd(f, &h.n_dih, 4) || !rd(f, &h.n_frames, 4))
        return ioerr(PG_ERR_IO, "ERROR: could not read the header of %s", path);
    const int rc = pg::check_bat_fields(h.version, h.double_prec, h.n_dih, h.n_frames);
    if (rc) return rc;
    if (h.version >= 3) {
        if (!read_atoms(f, h)) return ioerr(PG_ERR_IO, "ERROR: truncated atom block in %s", path);
    } else {
        synthetic_header(h);  // pre-3 files carry no atom names
    }
    h.dih.resize((size_t)6 * h.n_dih);
    h.masses.resize((size_t)h.n_dih + 3);
    if ((h.n_dih && !rd(f, h.dih.data(), h.dih.size() * 4)) || !rd(f, h.masses.data(), h.masses.size() * 4))
        return ioerr(PG_ERR_IO, "ERROR: truncated dihedral/mass block in %s", path);
    return PG_OK;
}

static int reader_threads() { return (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency())); }

// Reads `bytes` at file offset `off` into dst with up to `nth` threads
// (positioned reads, so the slices share no file offset). False on a short
// read.
static bool pread_all(int fd, int64_t off, unsigned char *dst, size_t bytes, int nth) {
    const size_t slice = std::max<size_t>((size_t)4 << 20, (bytes + nth - 1) / nth);
    std::atomic<bool> ok{true};
    auto work = [&](size_t a, size_t b) {
        while (a < b) {
            const ssize_t n = pread(fd, dst + a, b - a, (off_t)(off + (int64_t)a));
            if (n < 0 && errno == EINTR) continue;
            if (n <= 0) {
                ok = false;
                return;
            }
            a += (size_t)n;
        }
    };
    std::vector<std::thread> th;
    for (size_t a = slice; a < bytes; a += slice) th.emplace_back(work, a, std::min(bytes, a + slice));
    work(0, std::min(bytes, slice));
    for (auto &t : th) t.join();
    return ok;
}

// Frame records: 11 floats (44 bytes), 6 root externals, b0 b1 a0, then
// (b, a, d) per dihedral (read_BAT_frame, io_binary.cpp:281-368).
static size_t record_bytes(const Header &h) { return 44 + (size_t)(9 + 3 * h.n_dih) * (h.double_prec ? 8 : 4); }
static int record_values_offset(const Header &h) { return 44 + 6 * (h.double_prec ? 8 : 4); }

// Column of value u of a record (u counted from b0): bonds | angles | dihedrals.
static size_t column_of_value(int u, int nb, int na) {
    if (u < 2) return (size_t)u;
    if (u == 2) return (size_t)nb;
    const int k = (u - 3) / 3, r = (u - 3) - 3 * k;
    return r == 0 ? (size_t)k + 2 : (r == 1 ? (size_t)nb + k + 1 : (size_t)nb + na + k);
}

static size_t chunk_bytes_setting() {
    if (const char *e = getenv("PG_BAT_CHUNK_BYTES")) {
        const long long v = atoll(e);
        if (v > 0) return (size_t)v;
    }
    return (size_t)64 << 20;
}

PG_API int pg_bat_read(const char *path, pg_bat **out) {
    if (!path || !out) return ioerr(PG_ERR_ARG, "pg_bat_read: null argument");
    *out = nullptr;
    FILE *f = fopen(path, "rb");
    if (!f) return ioerr(PG_ERR_IO, "ERROR: Could not open file %s !", path);
    pg_bat *b = new pg_bat;
    Header &h = b->h;
    int rc = read_bat_header(f, h, path);
    do {
        if (rc != PG_OK) break;
        const int64_t body = (int64_t)ftell(f);
        const int nb = h.n_dih + 2, na = h.n_dih + 1, nd = h.n_dih;
        const size_t F = (size_t)h.n_frames, es = h.double_prec ? 8 : 4;
        const size_t D = (size_t)nb + na + nd;
        b->ld = (int64_t)F;
        b->bytes = D * F * es;
        if (cudaHostAlloc(&b->cols, b->bytes, cudaHostAllocDefault) == cudaSuccess) {
            b->pinned = true;
        } else {
            cudaGetLastError();
            b->cols = malloc(b->bytes);
            if (!b->cols) { rc = ioerr(PG_ERR_NOMEM, "ERROR ALLOCATNG MEMORY! (%zu bytes)", b->bytes); break; }
        }
        const size_t rec = record_bytes(h), off0 = (size_t)record_values_offset(h);
        const size_t batch = std::max<size_t>(1, chunk_bytes_setting() / rec);
        std::vector<unsigned char> buf(batch * rec);
        unsigned char *cols = (unsigned char *)b->cols;
        const int nth = reader_threads(), nvals = 3 + 3 * nd;
        for (size_t f0 = 0; f0 < F && rc == PG_OK; f0 += batch) {
            const size_t nf = std::min(batch, F - f0);
            if (!pread_all(fileno(f), body + (int64_t)(f0 * rec), buf.data(), nf * rec, nth)) {
                rc = ioerr(PG_ERR_IO, "An ERROR has occurred while reading the file %s . (frame %zu)", path, f0);
                break;
            }
            // transpose: each thread owns a range of values (columns), and
            // walks 64-frame blocks so every column is written in runs
            const int nt = std::min(nth, std::max(1, nvals / 32));
            auto work = [&](int t) {
                const int ua = (int)((int64_t)nvals * t / nt), ub = (int)((int64_t)nvals * (t + 1) / nt);
                for (size_t i0 = 0; i0 < nf; i0 += 64) {
                    const size_t i1 = std::min(nf, i0 + 64);
                    for (int u = ua; u < ub; u++) {
                        unsigned char *dst = cols + (column_of_value(u, nb, na) * F + f0) * es;
                        const unsigned char *src = buf.data() + off0 + (size_t)u * es;
                        for (size_t i = i0; i < i1; i++) memcpy(dst + i * es, src + i * rec, es);
                    }
                }
            };
            std::vector<std::thread> th;
            for (int t = 1; t < nt; t++) th.emplace_back(work, t);
            work(0);
            for (auto &x : th) x.join();
        }
    } while (0);
    fclose(f);
    if (rc != PG_OK) {
        pg_bat_free(b);
        return rc;
    }
    *out = b;
    return PG_OK;
}

PG_API int pg_bat_read_device(const char *path, int device, pg_bat **out) {
    if (!path || !out) return ioerr(PG_ERR_ARG, "pg_bat_read_device: null argument");
    *out = nullptr;
    FILE *f = fopen(path, "rb");
    if (!f) return ioerr(PG_ERR_IO, "ERROR: Could not open file %s !", path);
    pg_bat *b = new pg_bat;
    Header &h = b->h;
    int rc = read_bat_header(f, h, path);
    const int64_t body = rc == PG_OK ? (int64_t)ftell(f) : 0;
    cudaGetLastError();  // an error left by an earlier failed call of this thread is not this call's
    int prev = 0;
    cudaGetDevice(&prev);
    const int nst = 3;  // staging ring: read chunk k+1 while chunk k is copied and transposed
    unsigned char *pin[nst] = {nullptr, nullptr, nullptr}, *raw[nst] = {nullptr, nullptr, nullptr};
    cudaEvent_t ev[nst] = {nullptr, nullptr, nullptr};
    cudaStream_t st = nullptr;
    auto cuda_fail = [&](cudaError_t e, const char *what) {
        cudaGetLastError();
        return ioerr(e == cudaErrorMemoryAllocation ? PG_ERR_NOMEM : PG_ERR_CUDA, "ERROR: %s (%s) while reading %s",
                     what, cudaGetErrorString(e), path);
    };
    do {
        if (rc != PG_OK) break;
        cudaError_t e = cudaSetDevice(device);
        if (e != cudaSuccess) { rc = cuda_fail(e, "cudaSetDevice"); break; }
        b->device = device;
        const int nb = h.n_dih + 2, na = h.n_dih + 1, nd = h.n_dih;
        const size_t F = (size_t)h.n_frames, es = h.double_prec ? 8 : 4;
        const size_t D = (size_t)nb + na + nd;
        b->ld = (int64_t)((F + 31) / 32 * 32);
        b->bytes = D * (size_t)b->ld * es;
        if ((e = cudaMalloc(&b->cols, b->bytes)) != cudaSuccess) {
            b->cols = nullptr;
            rc = cuda_fail(e, "device allocation of the columns");
            break;
        }
        const size_t rec = record_bytes(h);
        const int off0 = record_values_offset(h);
        size_t nfc = std::max<size_t>(32, chunk_bytes_setting() / rec / 32 * 32);
        nfc = std::min(nfc, (F + 31) / 32 * 32);
        for (int k = 0; k < nst && rc == PG_OK; k++) {
            if ((e = cudaHostAlloc(&pin[k], nfc * rec, cudaHostAllocDefault)) != cudaSuccess) pin[k] = nullptr;
            else if ((e = cudaMalloc(&raw[k], nfc * rec)) != cudaSuccess) raw[k] = nullptr;
            else e = cudaEventCreateWithFlags(&ev[k], cudaEventDisableTiming);
            if (e != cudaSuccess) rc = cuda_fail(e, "staging buffers");
        }
        if (rc != PG_OK) break;
        if ((e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking)) != cudaSuccess) {
            st = nullptr;
            rc = cuda_fail(e, "cudaStreamCreate");
            break;
        }
        const int nth = reader_threads();
        size_t c = 0;
        for (size_t f0 = 0; f0 < F; f0 += nfc, c++) {
            const int k = (int)(c % nst);
            if (c >= (size_t)nst && (e = cudaEventSynchronize(ev[k])) != cudaSuccess) {
                rc = cuda_fail(e, "staging");
                break;
            }
            const size_t nf = std::min(nfc, F - f0);
            if (!pread_all(fileno(f), body + (int64_t)(f0 * rec), pin[k], nf * rec, nth)) {
                rc = ioerr(PG_ERR_IO, "An ERROR has occurred while reading the file %s . (frame %zu)", path, f0);
                break;
            }
            if ((e = cudaMemcpyAsync(raw[k], pin[k], nf * rec, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
                (e = pg::launch_bat_transpose(raw[k], (int)nf, (int64_t)rec, off0, (int)es, nd,
                                              (uint8_t *)b->cols, b->ld, (int64_t)f0, st)) != cudaSuccess ||
                (e = cudaEventRecord(ev[k], st)) != cudaSuccess) {
                rc = cuda_fail(e, "upload");
                break;
            }
        }
        if (st) {
            e = cudaStreamSynchronize(st);
            if (e != cudaSuccess && rc == PG_OK) rc = cuda_fail(e, "transpose");
        }
    } while (0);
    fclose(f);
    if (st) cudaStreamDestroy(st);
    for (int k = 0; k < nst; k++) {
        if (ev[k]) cudaEventDestroy(ev[k]);
        if (raw[k]) cudaFree(raw[k]);
        if (pin[k]) cudaFreeHost(pin[k]);
    }
    cudaSetDevice(prev);
    if (rc != PG_OK) {
        pg_bat_free(b);
        return rc;
    }
    *out = b;
    return PG_OK;
}

PG_API void pg_bat_free(pg_bat *b) {
    if (!b) return;
    if (b->cols) {
        if (b->device >= 0) {
            int prev = 0;
            cudaGetDevice(&prev);
            cudaSetDevice(b->device);
            cudaFree(b->cols);
            cudaSetDevice(prev);
        } else if (b->pinned) {
            cudaFreeHost(b->cols);
        } else {
            free(b->cols);
        }
    }
    delete b;
}

PG_API int pg_bat_view_of(const pg_bat *b, pg_bat_view *v) {
    if (!b || !v) return PG_ERR_ARG;
    const size_t ld = (size_t)b->ld, es = b->h.double_prec ? 8 : 4;
    const int nb = b->h.n_dih + 2, na = b->h.n_dih + 1;
    v->n_dihedrals = b->h.n_dih;
    v->n_frames = b->h.n_frames;
    v->double_prec = b->h.double_prec;
    v->on_device = b->device >= 0 ? 1 : 0;
    v->ld = (int64_t)ld;
    v->bonds = b->cols;
    v->angles = (const char *)b->cols + (size_t)nb * ld * es;
    v->dihedrals = (const char *)b->cols + (size_t)(nb + na) * ld * es;
    return PG_OK;
}
PG_API int pg_bat_n_dihedrals(const pg_bat *b) { return b ? b->h.n_dih : -1; }
PG_API int pg_bat_dihedral_table(const pg_bat *b, int *dih) {
    if (!b || !dih) return ioerr(PG_ERR_ARG, "pg_bat_dihedral_table: null argument");
    if (!b->h.dih.empty()) memcpy(dih, b->h.dih.data(), b->h.dih.size() * sizeof(int));
    return PG_OK;
}
PG_API int pg_bat_n_frames(const pg_bat *b) { return b ? b->h.n_frames : -1; }

PG_API int pg_bat_write_synthetic(const char *path, const pg_bat_view *v) {
    if (!path || !v || v->on_device || v->n_dihedrals < 0 || v->n_frames < 1 || v->ld < v->n_frames)
        return ioerr(PG_ERR_ARG, "pg_bat_write_synthetic: bad arguments");
    FILE *f = fopen(path, "wb");
    if (!f) return ioerr(PG_ERR_IO, "ERROR: Could not open file %s !", path);
    Header h;
    h.version = 3;
    h.double_prec = v->double_prec;
    h.n_dih = v->n_dihedrals;
    h.n_frames = v->n_frames;
    synthetic_header(h);
    bool ok = wr(f, &h.version, 4) && wr(f, &h.double_prec, 4) && wr(f, &h.n_dih, 4) && wr(f, &h.n_frames, 4) &&
              write_atoms(f, h) && (h.n_dih == 0 || wr(f, h.dih.data(), h.dih.size() * 4)) &&
              wr(f, h.masses.data(), h.masses.size() * 4);
    const size_t es = v->double_prec ? 8 : 4, nd = (size_t)h.n_dih, ld = (size_t)v->ld;
    const size_t rec = record_bytes(h), off0 = (size_t)record_values_offset(h);
    const unsigned char *B = (const unsigned char *)v->bonds, *A = (const unsigned char *)v->angles,
                        *Dd = (const unsigned char *)v->dihedrals;
    const int nb = (int)nd + 2, na = (int)nd + 1, nvals = 3 + 3 * (int)nd;
    // batches of whole records, filled by threads that own value (column)
    // ranges and walk 64-frame blocks (the reader's transpose, reversed)
    const size_t F = (size_t)h.n_frames, batch = std::max<size_t>(1, chunk_bytes_setting() / rec);
    std::vector<unsigned char> buf(std::min(batch, F) * rec);
    const int nth = reader_threads();
    for (size_t f0 = 0; f0 < F && ok; f0 += batch) {
        const size_t nf = std::min(batch, F - f0);
        for (size_t i = 0; i < nf; i++) {  // time, precision, box and the 6 root externals
            unsigned char *r = buf.data() + i * rec;
            memset(r, 0, off0);
            const float time = (float)(f0 + i), prec = 1000.0f;
            memcpy(r, &time, 4);
            memcpy(r + 4, &prec, 4);
        }
        const int nt = std::min(nth, std::max(1, nvals / 32));
        auto work = [&](int t) {
            const int ua = (int)((int64_t)nvals * t / nt), ub = (int)((int64_t)nvals * (t + 1) / nt);
            for (size_t i0 = 0; i0 < nf; i0 += 64) {
                const size_t i1 = std::min(nf, i0 + 64);
                for (int u = ua; u < ub; u++) {
                    const size_t c = column_of_value(u, nb, na);
                    const unsigned char *col = c < (size_t)nb ? B + c * ld * es
                                                              : (c < (size_t)(nb + na) ? A + (c - nb) * ld * es
                                                                                        : Dd + (c - nb - na) * ld * es);
                    unsigned char *dst = buf.data() + off0 + (size_t)u * es;
                    for (size_t i = i0; i < i1; i++) memcpy(dst + i * rec, col + (f0 + i) * es, es);
                }
            }
        };
        std::vector<std::thread> th;
        for (int t = 1; t < nt; t++) th.emplace_back(work, t);
        work(0);
        for (auto &x : th) x.join();
        ok = wr(f, buf.data(), nf * rec);
    }
    if (fclose(f) != 0) ok = false;
    return ok ? PG_OK : ioerr(PG_ERR_IO, "AN ERROR HAS OCCURED WHILE WRITING THE FILE %s", path);
}

PG_API int pg_par_write(const char *path, const pg_bat *b, const int bins[6], const pg_par_body *body) {
    if (!path || !b || !bins || !body) return ioerr(PG_ERR_ARG, "pg_par_write: null argument");
    FILE *f = fopen(path, "wb");
    if (!f) return ioerr(PG_ERR_IO, "ERROR: Could not open file %s !", path);
    const Header &h = b->h;
    const int version = 4;
    bool ok = wr(f, &version, 4) && wr(f, &h.double_prec, 4) && wr(f, &h.n_dih, 4) && wr(f, &h.n_frames, 4);
    for (int k = 0; k < 6 && ok; k++) ok = wr(f, &bins[k], 4);  // b1D a1D d1D b2D a2D d2D
    ok = ok && write_atoms(f, h) && (h.n_dih == 0 || wr(f, h.dih.data(), h.dih.size() * 4)) &&
         wr(f, h.masses.data(), h.masses.size() * 4);
    int64_t off[10];
    layout(h.n_dih, off);
    const double *src[9] = {body->s1_b, body->s1_a, body->s1_d, body->bb, body->ba, body->bd, body->aa, body->ad, body->dd};
    for (int k = 0; k < 9 && ok; k++) {
        const int64_t n = off[k + 1] - off[k];
        if (n > 0) ok = src[k] && wr(f, src[k], (size_t)n * 8);
    }
    if (fclose(f) != 0) ok = false;
    return ok ? PG_OK : ioerr(PG_ERR_IO, "AN ERROR HAS OCCURED WHILE WRITING THE FILE %s .", path);
}

PG_API int pg_par_read(const char *path, pg_par **out) {
    if (!path || !out) return ioerr(PG_ERR_ARG, "pg_par_read: null argument");
    *out = nullptr;
    FILE *f = fopen(path, "rb");
    if (!f) return ioerr(PG_ERR_IO, "ERROR: COULD NOT OPEN FILE %s !", path);
    pg_par *p = new pg_par;
    Header &h = p->h;
    int rc = PG_OK;
    do {
        int hv[4];
        if (!rd(f, hv, 16) || !rd(f, p->bins, 24)) { rc = ioerr(PG_ERR_IO, "ERROR READING HEADER OF FILE %s !", path); break; }
        h.version = hv[0]; h.double_prec = hv[1]; h.n_dih = hv[2]; h.n_frames = hv[3];
        rc = pg::check_par_fields(h.version, h.double_prec, h.n_dih, h.n_frames, p->bins);
        if (rc) break;
        if (h.version >= 3) {
            if (!read_atoms(f, h)) { rc = ioerr(PG_ERR_IO, "ERROR READING HEADER OF FILE %s !", path); break; }
        } else {
            synthetic_header(h);
        }
        h.dih.resize((size_t)6 * h.n_dih);
        for (int i = 0; i < h.n_dih && rc == PG_OK; i++) {  // io_binary.cpp:554-596
            if (!rd(f, &h.dih[6 * i], 24)) { rc = ioerr(PG_ERR_IO, "ERROR READING HEADER OF FILE %s !", path); break; }
            rc = pg::check_par_dihedral(&h.dih[6 * i]);
            if (rc) break;
            if (h.version == 1 && h.dih[6 * i + 5] != -1) h.dih[6 * i + 5]++;
        }
        if (rc) break;
        h.masses.resize((size_t)h.n_dih + 3);
        if (!rd(f, h.masses.data(), h.masses.size() * 4)) { rc = ioerr(PG_ERR_IO, "ERROR READING HEADER OF FILE %s !", path); break; }
        layout(h.n_dih, p->off);
        try {
            p->body.resize((size_t)p->off[9]);
        } catch (...) {
            rc = ioerr(PG_ERR_NOMEM, "ERROR: ALLOCATION FOR PAR FILE BODY FAILED. MORE MEMORY NEEDED?");
            break;
        }
        if (p->off[9] && !rd(f, p->body.data(), (size_t)p->off[9] * 8)) { rc = ioerr(PG_ERR_IO, "ERROR READING FILE %s !", path); break; }
    } while (0);
    fclose(f);
    if (rc) {
        delete p;
        return rc;
    }
    *out = p;
    return PG_OK;
}

PG_API void pg_par_free(pg_par *p) { delete p; }
PG_API int pg_par_n_dihedrals(const pg_par *p) { return p ? p->h.n_dih : -1; }
PG_API int pg_par_bins(const pg_par *p, int bins[6]) {
    if (!p || !bins) return PG_ERR_ARG;
    memcpy(bins, p->bins, sizeof p->bins);
    return PG_OK;
}
PG_API int pg_par_body_of(const pg_par *p, pg_par_body *b) {
    if (!p || !b) return PG_ERR_ARG;
    double *base = const_cast<double *>(p->body.data());
    double **dst[9] = {&b->s1_b, &b->s1_a, &b->s1_d, &b->bb, &b->ba, &b->bd, &b->aa, &b->ad, &b->dd};
    for (int k = 0; k < 9; k++) *dst[k] = base + p->off[k];
    return PG_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ text

namespace {

// Buffered writer; doubles as C++ ostream precision(12) prints them (%.12g).
struct Out {
    FILE *f;
    std::vector<char> buf;
    size_t n = 0;
    explicit Out(FILE *fp) : f(fp), buf(1 << 22) {}
    void flush() {
        if (n) fwrite(buf.data(), 1, n, f);
        n = 0;
    }
    void room(size_t k) {
        if (n + k > buf.size()) flush();
    }
    Out &s(const char *t) {
        size_t k = strlen(t);
        room(k);
        memcpy(buf.data() + n, t, k);
        n += k;
        return *this;
    }
    Out &i(long long v) {
        room(32);
        n += (size_t)snprintf(buf.data() + n, 32, "%lld", v);
        return *this;
    }
    Out &d(double v) {
        room(40);
        n += (size_t)snprintf(buf.data() + n, 40, "%.12g", v);
        return *this;
    }
    ~Out() { flush(); }
};

double mutual(int type, int i1, int i2, int nd_, const pg_par_body *b) {  // util.cpp:47-81
    const int nb = nd_ + 2, na = nd_ + 1, nd = nd_;
    const int s = i1 < i2 ? i1 : i2, g = i1 < i2 ? i2 : i1;
    switch (type) {
    case 0: if (i1 == i2) break; return b->s1_b[s] + b->s1_b[g] - b->bb[(int64_t)(nb - s) * (nb - s - 1) / 2 + s - g];
    case 1: return b->s1_b[i1] + b->s1_a[i2] - b->ba[(int64_t)i1 * na + i2];
    case 2: return b->s1_b[i1] + b->s1_d[i2] - b->bd[(int64_t)i1 * nd + i2];
    case 3: if (i1 == i2) break; return b->s1_a[s] + b->s1_a[g] - b->aa[(int64_t)(na - s) * (na - s - 1) / 2 + s - g];
    case 4: return b->s1_a[i1] + b->s1_d[i2] - b->ad[(int64_t)i1 * nd + i2];
    case 5: if (i1 == i2) break; return b->s1_d[s] + b->s1_d[g] - b->dd[(int64_t)(nd - s) * (nd - s - 1) / 2 + s - g];
    }
    fprintf(stderr, "WARNING: REQUEST FOR MUTUAL INFORMATION TYPE %d WITH INDICES %d AND %dYIELDED NO RESULT.\n", type, i1, i2);
    return 0;
}

FILE *open_out(const char *path) { return path ? fopen(path, "w") : stdout; }
int close_out(const char *path, FILE *f) { return path ? (fclose(f) == 0 ? PG_OK : PG_ERR_IO) : (fflush(f), PG_OK); }

}  // namespace

extern "C" {

// MIE text pieces shared by the host and the device writers: the 1D lines
// with their totals, and the 2D block totals summed in the reference's line
// order (one thread: the order fixes the FP64 rounding).
static void mie_head(Out &o, int n_dih, const pg_par_body *b, double t1[3]) {
    const int nb = n_dih + 2, na = n_dih + 1, nd = n_dih;
    t1[0] = t1[1] = t1[2] = 0.0;
    for (int k = 0; k < nb; k++) { o.s("bond ").i(k + 1).s("   ").d(b->s1_b[k]).s("\n"); t1[0] += b->s1_b[k]; }
    for (int k = 0; k < na; k++) { o.s("angle ").i(k + 1).s("   ").d(b->s1_a[k]).s("\n"); t1[1] += b->s1_a[k]; }
    for (int k = 0; k < nd; k++) { o.s("dihedral ").i(k + 1).s("   ").d(b->s1_d[k]).s("\n"); t1[2] += b->s1_d[k]; }
}
static void mie_block_totals(int n_dih, const pg_par_body *b, double e[6], double m[6]) {
    const int nb = n_dih + 2, na = n_dih + 1, nd = n_dih;
    const int n1[6] = {nb, nb, nb, na, na, nd}, n2[6] = {nb, na, nd, na, nd, nd};
    const double *blk[6] = {b->bb, b->ba, b->bd, b->aa, b->ad, b->dd};
    for (int q = 0; q < 6; q++) {
        e[q] = m[q] = 0.0;
        const bool same = q == 0 || q == 3 || q == 5;
        int64_t counter = (int64_t)n1[q] * (n1[q] - 1) / 2 - 1;
        const int rows = same ? n1[q] - 1 : n1[q];
        for (int i = 0; i < rows; i++)
            for (int j = same ? i + 1 : 0; j < n2[q]; j++) {
                e[q] += same ? blk[q][counter--] : blk[q][(int64_t)i * n2[q] + j];
                m[q] += mutual(q, i, j, n_dih, b);
            }
    }
}
static void mie_tail(Out &o, const double t1[3], const double e[6], const double m[6]) {
    o.s("TOTAL 1D BONDS ENTROPY = ").d(t1[0]).s("\n");
    o.s("TOTAL 1D ANGLES ENTROPY = ").d(t1[1]).s("\n");
    o.s("TOTAL 1D DIHEDRALS ENTROPY = ").d(t1[2]).s("\n");
    const char *tn[6] = {"BONDS-BONDS", "BONDS-ANGLES", "BONDS-DIHEDRALS", "ANGLES-ANGLES", "ANGLES-DIHEDRALS", "DIHEDRALS-DIHEDRALS"};
    for (int q = 0; q < 6; q++) {
        o.s("TOTAL 2D ").s(tn[q]).s(" ENTROPY = ").d(e[q]).s("\n");
        o.s("TOTAL 2D ").s(tn[q]).s(" MUTUAL INFORMATION = ").d(m[q]).s("\n");
    }
    o.s("TOTAL CONFIGURATIONAL ENTROPY = ").d(t1[0] + t1[1] + t1[2] - m[0] - m[1] - m[2] - m[3] - m[4] - m[5]).s("\n");
}

PG_API int pg_write_mie_text_device(pg_ctx *ctx, const char *path, int n_dih, const pg_par_body *b) {
    if (!ctx || !b || n_dih < 0) return ioerr(PG_ERR_ARG, "pg_write_mie_text_device: bad arguments");
    FILE *f = open_out(path);
    if (!f) return ioerr(PG_ERR_IO, "ERROR: COULD NOT OPEN FILE %s !", path);
    int rc = PG_OK;
    {
        Out o(f);
        double t1[3], e[6], m[6];
        mie_head(o, n_dih, b, t1);
        o.flush();
        std::thread totals([&] { mie_block_totals(n_dih, b, e, m); });  // overlaps the device formatting
        rc = pg::mie_lines_device(ctx, n_dih, b, [&](const char *p, size_t n) { return fwrite(p, 1, n, f) == n; });
        totals.join();
        if (rc == PG_OK) mie_tail(o, t1, e, m);
    }
    const int rc2 = close_out(path, f);
    return rc != PG_OK ? rc : rc2;
}

PG_API int pg_format_g12(double v, char *out) {
    const int n = pg::format_g12(v, out);
    if (n < 0) return snprintf(out, 32, "%.12g", v);
    out[n] = 0;
    return n;
}

PG_API int pg_write_mie_text(const char *path, int n_dih, const pg_par_body *b) {
    if (!b || n_dih < 0) return ioerr(PG_ERR_ARG, "pg_write_mie_text: bad arguments");
    FILE *f = open_out(path);
    if (!f) return ioerr(PG_ERR_IO, "ERROR: COULD NOT OPEN FILE %s !", path);
    {
        Out o(f);
        const int nb = n_dih + 2, na = n_dih + 1, nd = n_dih;
        double t1[3], e[6] = {0}, m[6] = {0};
        mie_head(o, n_dih, b, t1);
        const char *nm[6] = {"bond-bond ", "bond-angle ", "bond-dihedral ", "angle-angle ", "angle-dihedral ", "dihedral-dihedral "};
        const int n1[6] = {nb, nb, nb, na, na, nd}, n2[6] = {nb, na, nd, na, nd, nd};
        const double *blk[6] = {b->bb, b->ba, b->bd, b->aa, b->ad, b->dd};
        // The block totals are summed in the reference's line order (one
        // thread); the lines themselves are formatted by all host threads in
        // row tasks of ~64k lines and written in order, a bounded batch at a time.
        struct Task {
            int q, i0, i1;
        };
        std::vector<Task> tasks;
        for (int q = 0; q < 6; q++) {
            const bool same = q == 0 || q == 3 || q == 5;
            int64_t counter = (int64_t)n1[q] * (n1[q] - 1) / 2 - 1;
            const int rows = same ? n1[q] - 1 : n1[q];
            int64_t acc = 0;
            int i0 = 0;
            for (int i = 0; i < rows; i++) {
                for (int j = same ? i + 1 : 0; j < n2[q]; j++) {
                    const double mu = mutual(q, i, j, n_dih, b);
                    const double s2 = same ? blk[q][counter--] : blk[q][(int64_t)i * n2[q] + j];
                    e[q] += s2;
                    m[q] += mu;
                }
                acc += same ? n2[q] - i - 1 : n2[q];
                if (acc >= 65536 || i == rows - 1) {
                    tasks.push_back({q, i0, i + 1});
                    i0 = i + 1;
                    acc = 0;
                }
            }
        }
        auto format_rows = [&](const Task &t, std::string &out) {
            const int q = t.q;
            const bool same = q == 0 || q == 3 || q == 5;
            const int64_t n = n1[q];
            // reverse-order index of the first line of row i0
            int64_t counter = n * (n - 1) / 2 - 1 - ((int64_t)t.i0 * (n - 1) - (int64_t)t.i0 * (t.i0 - 1) / 2);
            char line[160];
            for (int i = t.i0; i < t.i1; i++)
                for (int j = same ? i + 1 : 0; j < n2[q]; j++) {
                    const double mu = mutual(q, i, j, n_dih, b);
                    const double s2 = same ? blk[q][counter--] : blk[q][(int64_t)i * n2[q] + j];
                    const int k = snprintf(line, sizeof line, "%s%d  %d   %.12g   %.12g\n", nm[q], i + 1, j + 1, s2, mu);
                    out.append(line, (size_t)k);
                }
        };
        const int nthr = (int)std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
        for (size_t t0 = 0; t0 < tasks.size(); t0 += (size_t)nthr * 4) {
            const size_t t1 = std::min(tasks.size(), t0 + (size_t)nthr * 4);
            std::vector<std::string> bufs(t1 - t0);
            std::vector<std::thread> pool;
            for (int w = 0; w < nthr; w++)
                pool.emplace_back([&, w] {
                    for (size_t k = t0 + w; k < t1; k += (size_t)nthr) format_rows(tasks[k], bufs[k - t0]);
                });
            for (auto &th : pool) th.join();
            for (const std::string &sbuf : bufs) {
                o.flush();
                fwrite(sbuf.data(), 1, sbuf.size(), f);
            }
        }
        mie_tail(o, t1, e, m);
    }
    return close_out(path, f);
}

PG_API int pg_write_mist_text(const char *path, int n_dih, const pg_mist_edge *edges, const double totals[10]) {
    if (!edges || !totals || n_dih < 0) return ioerr(PG_ERR_ARG, "pg_write_mist_text: bad arguments");
    FILE *f = open_out(path);
    if (!f) return ioerr(PG_ERR_IO, "ERROR: COULD NOT OPEN FILE %s !", path);
    {
        Out o(f);
        const char ch[3] = {'b', 'a', 'd'};
        const int n = 3 * n_dih + 3 - 1;
        for (int s = 0; s < n; s++) {
            const char t[5] = {ch[edges[s].type_in], ' ', ch[edges[s].type_out], ' ', 0};
            o.s(t).i(edges[s].index_in).s(" ").i(edges[s].index_out).s("   MI: ").d(edges[s].mi).s("   left to process: ").i(edges[s].left).s("\n");
        }
        const char *lines[10] = {"TOTAL 1D BONDS ENTROPY = ", "TOTAL 1D ANGLES ENTROPY = ", "TOTAL 1D DIHEDRALS ENTROPY = ",
                                 "TOTAL 2D BONDS-BONDS MUTUAL INFORMATION = ", "TOTAL 2D BONDS-ANGLES MUTUAL INFORMATION = ",
                                 "TOTAL 2D BONDS-DIHEDRALS MUTUAL INFORMATION = ", "TOTAL 2D ANGLES-ANGLES MUTUAL INFORMATION = ",
                                 "TOTAL 2D ANGLES-DIHEDRALS MUTUAL INFORMATION = ", "TOTAL 2D DIHEDRALS-DIHEDRALS MUTUAL INFORMATION = ",
                                 "TOTAL CONFIGURATIONAL ENTROPY = "};
        for (int k = 0; k < 10; k++) o.s(lines[k]).d(totals[k]).s("\n");
    }
    return close_out(path, f);
}

PG_API int pg_write_info_text(const char *path, const pg_par *p) {
    if (!p) return ioerr(PG_ERR_ARG, "pg_write_info_text: null argument");
    const Header &h = p->h;
    if (h.n_dih < 1) return ioerr(PG_ERR_ARG, "pg_write_info_text: no dihedrals");
    FILE *f = open_out(path);
    if (!f) return ioerr(PG_ERR_IO, "ERROR: COULD NOT OPEN FILE %s !", path);
    {
        Out o(f);
        const int *d = h.dih.data();
        o.s("#bond #atom1 #atom2 \n");
        o.s("1 ").i(d[0]).s(" ").i(d[1]).s("\n");
        o.s("2 ").i(d[1]).s(" ").i(d[2]).s("\n");
        for (int i = 0; i < h.n_dih; i++) o.i(i + 3).s(" ").i(d[6 * i + 2]).s(" ").i(d[6 * i + 3]).s("\n");
        o.s("#angle #atom1 #atom2 #atom3\n");
        o.s("1 ").i(d[0]).s(" ").i(d[1]).s(" ").i(d[2]).s("\n");
        for (int i = 0; i < h.n_dih; i++) o.i(i + 2).s(" ").i(d[6 * i + 1]).s(" ").i(d[6 * i + 2]).s(" ").i(d[6 * i + 3]).s("\n");
        o.s("#dihedral #atom1 #atom2 #atom3 #atom4    dihedral_type(common=0,pseudo=1,improper=-1)   phaseangle_of(-1 if no phaseangle)\n");
        for (int i = 0; i < h.n_dih; i++)
            o.i(i + 1).s(" ").i(d[6 * i]).s(" ").i(d[6 * i + 1]).s(" ").i(d[6 * i + 2]).s(" ").i(d[6 * i + 3]).s(" ").i(d[6 * i + 4]).s(" ").i(d[6 * i + 5]).s("\n");
    }
    return close_out(path, f);
}

}  // extern "C"
