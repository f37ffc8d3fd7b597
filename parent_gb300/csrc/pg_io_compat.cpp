// The reference's binary I/O library with its own C++ signatures
// (src/util/io/io_binary.h:42-52), over this library's format checks: the
// declarations are in include/parent_gb300_io.h. A program written against
// io_binary.h links against libparent_gb300 instead of io_binary.cpp.
//
// Every function works at the stream's current position and accumulates the
// stream's fail bit after each read or write into its return value, as the
// reference does, so a truncated file returns the same nonzero status. The
// header checks are the ones pg_bat_read / pg_par_read apply (check_*_fields
// in pg_io.cpp, the reference's messages on stderr); a failed check returns 1.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <fstream>
#include <string>
#include <vector>

#include "../../include/parent_gb300.h"
#include "../../include/parent_gb300_io.h"

namespace pg {
int check_bat_fields(int version, int prec, int n_dih, int n_frames);
int check_par_fields(int version, int prec, int n_dih, int n_frames, const int bins[6]);
int check_par_dihedral(const int d[6]);
}  // namespace pg

namespace {

// Fail-bit accumulating stream access.
struct In {
    std::ifstream *s;
    int fail = 0;
    void get(void *p, size_t n) {
        s->read((char *)p, (std::streamsize)n);
        fail |= s->rdstate() & std::ifstream::failbit;
    }
    // a zero-padded name field of n bytes, up to its first zero byte
    std::string name(size_t n) {
        char b[32] = {0};
        get(b, n);
        size_t k = 0;
        while (k < n && b[k]) k++;
        return std::string(b, k);
    }
};

struct Out {
    std::ofstream *s;
    int fail = 0;
    void put(const void *p, size_t n) {
        s->write((const char *)p, (std::streamsize)n);
        fail |= s->rdstate() & std::ofstream::failbit;
    }
    void put_i(int v) { put(&v, sizeof v); }
    void put_f(float v) { put(&v, sizeof v); }
    // at most n - 1 characters of v, zero-padded to n bytes
    void name(const std::string &v, size_t n) {
        char b[32];
        memset(b, 0, sizeof b);
        memcpy(b, v.c_str(), std::min(v.size(), n - 1));
        put(b, n);
    }
};

// atom block (residue[8], residue number, atom[8], molecule[31] per atom)
void write_atoms(Out &o, int n_atoms, std::vector<std::string> *res, std::vector<int> *resnum,
                 std::vector<std::string> *atoms, std::vector<std::string> *mols) {
    for (int i = 0; i < n_atoms; i++) {
        o.name((*res)[i], 8);
        o.put_i((*resnum)[i]);
        o.name((*atoms)[i], 8);
        o.name((*mols)[i], 31);
    }
}

void read_atoms(In &in, int n_atoms, std::vector<std::string> *res, std::vector<int> *resnum,
                std::vector<std::string> *atoms, std::vector<std::string> *mols) {
    for (int i = 0; i < n_atoms; i++) {
        res->push_back(in.name(8));
        int r = 0;
        in.get(&r, 4);
        resnum->push_back(r);
        atoms->push_back(in.name(8));
        mols->push_back(in.name(31));
    }
}

void write_dihedrals_and_masses(Out &o, std::vector<std::vector<int> > *dih, std::vector<float> *masses) {
    const int n = (int)dih->size();
    for (int i = 0; i < n; i++)
        for (int k = 0; k < 6; k++) o.put_i((*dih)[i][k]);
    for (int i = 0; i < n + 3; i++) o.put_f((*masses)[i]);
}

// one value of a frame record in the file's precision, as double
double value(In &in, int prec) {
    if (prec == 1) {
        double v = 0.0;
        in.get(&v, 8);
        return v;
    }
    float f = 0.f;
    in.get(&f, 4);
    return (double)f;
}

void put_value(Out &o, int prec, double v) {
    if (prec == 1) o.put(&v, 8);
    else if (prec == 0) o.put_f((float)v);
}

}  // namespace

PG_IO_API int write_BAT_header(std::ofstream *outfile, int double_prec, int numframes,
                               std::vector<std::vector<int> > *dihedrals_top, std::vector<float> *masses,
                               std::vector<std::string> *residues, std::vector<int> *residueNumbers,
                               std::vector<std::string> *atomNames, std::vector<std::string> *belongsToMolecule) {
    Out o{outfile};
    const int n = (int)dihedrals_top->size();
    o.put_i(3);  // .bat version
    o.put_i(double_prec);
    o.put_i(n);
    o.put_i(numframes);
    write_atoms(o, n + 3, residues, residueNumbers, atomNames, belongsToMolecule);
    write_dihedrals_and_masses(o, dihedrals_top, masses);
    return o.fail;
}

PG_IO_API int read_BAT_header(std::ifstream *infile, int *double_prec, int *numFrames,
                              std::vector<std::vector<int> > *dihedrals_top, std::vector<float> *masses,
                              std::vector<std::string> *residues, std::vector<int> *residueNumbers,
                              std::vector<std::string> *atomNames, std::vector<std::string> *belongsToMolecule) {
    In in{infile};
    int version = 0, n = 0;
    in.get(&version, 4);
    in.get(double_prec, 4);
    in.get(&n, 4);
    in.get(numFrames, 4);
    if (in.fail) return in.fail;
    if (pg::check_bat_fields(version, *double_prec, n, *numFrames) != PG_OK) return 1;
    if (version >= 3) read_atoms(in, n + 3, residues, residueNumbers, atomNames, belongsToMolecule);
    if (in.fail) return in.fail;
    for (int i = 0; i < n; i++) {
        std::vector<int> d(6, 0);
        in.get(d.data(), 24);
        dihedrals_top->push_back(d);
    }
    for (int i = 0; i < n + 3; i++) {
        float m = 0.f;
        in.get(&m, 4);
        masses->push_back(m);
    }
    return in.fail;
}

PG_IO_API int write_BAT_frame(std::ofstream *outfile, int double_prec, int nDihedrals, float time, float xtcPrec,
                              float **box, double *root_origin_cartesian, double root_origin_theta,
                              double root_origin_phi, double root_origin_dihedral, double *bonds, double *angles,
                              double *dihedrals) {
    Out o{outfile};
    o.put_f(time);
    o.put_f(xtcPrec);
    o.put(box, 9 * sizeof(float));  // the box as the caller lays it out, nine floats from this address
    if (double_prec != 0 && double_prec != 1) return o.fail;
    for (int c = 0; c < 3; c++) put_value(o, double_prec, root_origin_cartesian[c]);
    put_value(o, double_prec, root_origin_theta);
    put_value(o, double_prec, root_origin_phi);
    put_value(o, double_prec, root_origin_dihedral);
    put_value(o, double_prec, bonds[0]);
    put_value(o, double_prec, bonds[1]);
    put_value(o, double_prec, angles[0]);
    for (int i = 0; i < nDihedrals; i++) {
        put_value(o, double_prec, bonds[i + 2]);
        put_value(o, double_prec, angles[i + 1]);
        put_value(o, double_prec, dihedrals[i]);
    }
    return o.fail;
}

PG_IO_API int read_BAT_frame(std::ifstream *infile, int precision, int nDihedrals, float *time, float *xtcPrec,
                             float **dbox, double *root_origin_cartesian, double *root_origin_theta,
                             double *root_origin_phi, double *root_origin_dihedral, double *my_bonds,
                             double *my_angles, double *my_dihedrals) {
    In in{infile};
    in.get(time, 4);
    in.get(xtcPrec, 4);
    in.get(dbox, 9 * sizeof(float));
    if (precision != 0 && precision != 1) return in.fail;
    for (int c = 0; c < 3; c++) root_origin_cartesian[c] = value(in, precision);
    *root_origin_theta = value(in, precision);
    *root_origin_phi = value(in, precision);
    *root_origin_dihedral = value(in, precision);
    my_bonds[0] = value(in, precision);
    my_bonds[1] = value(in, precision);
    my_angles[0] = value(in, precision);
    for (int i = 0; i < nDihedrals; i++) {
        my_bonds[i + 2] = value(in, precision);
        my_angles[i + 1] = value(in, precision);
        my_dihedrals[i] = value(in, precision);
    }
    return in.fail;
}

PG_IO_API int write_PAR_header(std::ofstream *outfile, int nDihedrals, int double_prec, int numFrames,
                               std::vector<std::vector<int> > *dihedrals_top, std::vector<float> *masses,
                               int bDens1D, int aDens1D, int dDens1D, int bDens, int aDens, int dDens,
                               std::vector<std::string> *residues, std::vector<int> *residueNumbers,
                               std::vector<std::string> *atomNames, std::vector<std::string> *belongsToMolecule) {
    (void)nDihedrals;  // the count written is the table's, as in the reference
    Out o{outfile};
    const int n = (int)dihedrals_top->size();
    o.put_i(4);  // .par version
    o.put_i(double_prec);
    o.put_i(n);
    o.put_i(numFrames);
    const int bins[6] = {bDens1D, aDens1D, dDens1D, bDens, aDens, dDens};
    for (int b : bins) o.put_i(b);
    write_atoms(o, n + 3, residues, residueNumbers, atomNames, belongsToMolecule);
    write_dihedrals_and_masses(o, dihedrals_top, masses);
    return o.fail;
}

PG_IO_API int read_PAR_header(std::ifstream *infile, int *nDihedrals, int *double_prec, int *numFrames,
                              std::vector<std::vector<int> > *dihedrals_top, std::vector<float> *masses,
                              int *version, int *bDens, int *aDens, int *dDens, int *bDens1D, int *aDens1D,
                              int *dDens1D, std::vector<std::string> *residues, std::vector<int> *residueNumbers,
                              std::vector<std::string> *atomNames, std::vector<std::string> *belongsToMolecule) {
    In in{infile};
    in.get(version, 4);
    in.get(double_prec, 4);
    in.get(nDihedrals, 4);
    in.get(numFrames, 4);
    int *bins[6] = {bDens1D, aDens1D, dDens1D, bDens, aDens, dDens};  // file order
    for (int *b : bins) in.get(b, 4);
    if (in.fail) return in.fail;
    const int bv[6] = {*bDens1D, *aDens1D, *dDens1D, *bDens, *aDens, *dDens};
    if (pg::check_par_fields(*version, *double_prec, *nDihedrals, *numFrames, bv) != PG_OK) return 1;
    const int n = *nDihedrals;
    if (*version >= 3) read_atoms(in, n + 3, residues, residueNumbers, atomNames, belongsToMolecule);
    if (in.fail) return in.fail;
    for (int i = 0; i < n; i++) {
        std::vector<int> d(6, 0);
        for (int k = 0; k < 6; k++) {
            in.get(&d[k], 4);
            // each field is checked as soon as it is read (a valid entry with
            // this one field replaced), so a bad entry stops the read where
            // the reference stops, with the partial entry appended
            int probe[6] = {1, 1, 1, 1, 0, -1};
            probe[k] = d[k];
            if (pg::check_par_dihedral(probe) != PG_OK) {
                dihedrals_top->push_back(d);
                return 1;
            }
        }
        if (*version == 1 && d[5] != -1) d[5]++;  // parent numbering of version-1 files
        dihedrals_top->push_back(d);
    }
    for (int i = 0; i < n + 3; i++) {
        float m = 0.f;
        in.get(&m, 4);
        masses->push_back(m);
    }
    return in.fail;
}

namespace {

void block_sizes(int nDihedrals, long long n[9]) {
    const long long nb = nDihedrals + 2, na = nDihedrals + 1, nd = nDihedrals;
    const long long v[9] = {nb, na, nd, nb * (nb - 1) / 2, nb * na, nb * nd, na * (na - 1) / 2, na * nd,
                            nd * (nd - 1) / 2};
    for (int k = 0; k < 9; k++) n[k] = v[k];
}

}  // namespace

PG_IO_API int write_PAR_body(std::ofstream *par_file, int nDihedrals, double *bondsEntropy1D,
                             double *anglesEntropy1D, double *dihedralsEntropy1D, double *bbEntropy,
                             double *baEntropy, double *bdEntropy, double *aaEntropy, double *adEntropy,
                             double *ddEntropy) {
    Out o{par_file};
    long long n[9];
    block_sizes(nDihedrals, n);
    double *blk[9] = {bondsEntropy1D, anglesEntropy1D, dihedralsEntropy1D, bbEntropy, baEntropy,
                      bdEntropy, aaEntropy, adEntropy, ddEntropy};
    for (int k = 0; k < 9; k++) o.put(blk[k], (size_t)n[k] * sizeof(double));
    return o.fail;
}

PG_IO_API int read_PAR_body(std::ifstream *par_file, int nDihedrals, double **bondsEntropy1D,
                            double **anglesEntropy1D, double **dihedralsEntropy1D, double **bbEntropy,
                            double **baEntropy, double **bdEntropy, double **aaEntropy, double **adEntropy,
                            double **ddEntropy) {
    long long n[9];
    block_sizes(nDihedrals, n);
    double **blk[9] = {bondsEntropy1D, anglesEntropy1D, dihedralsEntropy1D, bbEntropy, baEntropy,
                       bdEntropy, aaEntropy, adEntropy, ddEntropy};
    bool ok = true;
    for (int k = 0; k < 9; k++) {
        *blk[k] = (double *)malloc((size_t)n[k] * sizeof(double));
        ok = ok && (*blk[k] != nullptr || n[k] == 0);
    }
    if (!ok) {
        fprintf(stderr, "ERROR: ALLOCATION FOR PAR FILE BODY FAILED. MORE MEMORY NEEDED?\n");
        return 2;
    }
    In in{par_file};
    for (int k = 0; k < 9; k++) in.get(*blk[k], (size_t)n[k] * sizeof(double));
    return in.fail;
}
