/*
 * parent_gb300_io.h — the reference suite's binary I/O library, with the same
 * C++ signatures, exported by libparent_gb300.so.
 *
 * The reference ships its .bat/.par readers and writers as a small public
 * C++ library (src/util/io/io_binary.h:42-52, advertised for reuse in its
 * README) that every one of its programs links. These are the same eight
 * functions, implemented in this library (parent_gb300/csrc/pg_io_compat.cpp),
 * so that the reference's own post-processors (get_PAR_MIE, get_PAR_MIST,
 * get_PAR_info) or a user's program written against io_binary.h link against
 * libparent_gb300 instead of io_binary.cpp without a source change:
 *   - std::ifstream / std::ofstream positioned at the header or the frame;
 *   - headers append to the given vectors (push_back), as the reference's do;
 *   - read_PAR_body allocates the nine body arrays with malloc; the caller
 *     frees them with free();
 *   - return 0 on success; a stream failure returns the stream's fail bits,
 *     a header check prints the reference's message on stderr and returns 1,
 *     a failed body allocation returns 2.
 * C++ linkage (the reference's functions are C++ functions taking std types),
 * so the caller must be built with a compatible C++ standard library.
 */
#ifndef PARENT_GB300_IO_H
#define PARENT_GB300_IO_H

#ifdef __cplusplus
#include <fstream>
#include <string>
#include <vector>

#if defined(__GNUC__)
#define PG_IO_API __attribute__((visibility("default")))
#else
#define PG_IO_API
#endif

/* write_BAT_header, io_binary.cpp:43-102 (.bat version 3). */
PG_IO_API int write_BAT_header(std::ofstream *outfile, int double_prec, int numframes,
                               std::vector<std::vector<int> > *dihedrals_top, std::vector<float> *masses,
                               std::vector<std::string> *residues, std::vector<int> *residueNumbers,
                               std::vector<std::string> *atomNames, std::vector<std::string> *belongsToMolecule);

/* read_BAT_header, io_binary.cpp:107-200, with its checks (:127-145). */
PG_IO_API int read_BAT_header(std::ifstream *infile, int *double_prec, int *numFrames,
                              std::vector<std::vector<int> > *dihedrals_top, std::vector<float> *masses,
                              std::vector<std::string> *residues, std::vector<int> *residueNumbers,
                              std::vector<std::string> *atomNames, std::vector<std::string> *belongsToMolecule);

/* write_BAT_frame, io_binary.cpp:203-278: time, precision and box, then the
 * six root externals and every bond/angle/dihedral in double or, for
 * double_prec 0, converted to float. */
PG_IO_API int write_BAT_frame(std::ofstream *outfile, int double_prec, int nDihedrals, float time, float xtcPrec,
                              float **box, double *root_origin_cartesian, double root_origin_theta,
                              double root_origin_phi, double root_origin_dihedral, double *bonds, double *angles,
                              double *dihedrals);

/* read_BAT_frame, io_binary.cpp:281-368: FP32 values promoted to double. */
PG_IO_API int read_BAT_frame(std::ifstream *infile, int precision, int nDihedrals, float *time, float *xtcPrec,
                             float **dbox, double *root_origin_cartesian, double *root_origin_theta,
                             double *root_origin_phi, double *root_origin_dihedral, double *my_bonds,
                             double *my_angles, double *my_dihedrals);

/* write_PAR_header, io_binary.cpp:371-442 (.par version 4; the dihedral
 * count written is dihedrals_top->size(), as in the reference). */
PG_IO_API int write_PAR_header(std::ofstream *outfile, int nDihedrals, int double_prec, int numFrames,
                               std::vector<std::vector<int> > *dihedrals_top, std::vector<float> *masses,
                               int bDens1D, int aDens1D, int dDens1D, int bDens, int aDens, int dDens,
                               std::vector<std::string> *residues, std::vector<int> *residueNumbers,
                               std::vector<std::string> *atomNames, std::vector<std::string> *belongsToMolecule);

/* read_PAR_header, io_binary.cpp:446-604, with its checks (:477-519,
 * :554-591) and the version-1 parent renumbering. */
PG_IO_API int read_PAR_header(std::ifstream *infile, int *nDihedrals, int *double_prec, int *numFrames,
                              std::vector<std::vector<int> > *dihedrals_top, std::vector<float> *masses,
                              int *version, int *bDens, int *aDens, int *dDens, int *bDens1D, int *aDens1D,
                              int *dDens1D, std::vector<std::string> *residues, std::vector<int> *residueNumbers,
                              std::vector<std::string> *atomNames, std::vector<std::string> *belongsToMolecule);

/* write_PAR_body, io_binary.cpp:606-631: the nine blocks in body order. */
PG_IO_API int write_PAR_body(std::ofstream *par_file, int nDihedrals, double *bondsEntropy1D,
                             double *anglesEntropy1D, double *dihedralsEntropy1D, double *bbEntropy,
                             double *baEntropy, double *bdEntropy, double *aaEntropy, double *adEntropy,
                             double *ddEntropy);

/* read_PAR_body, io_binary.cpp:633-673: the nine blocks malloc'd here. */
PG_IO_API int read_PAR_body(std::ifstream *par_file, int nDihedrals, double **bondsEntropy1D,
                            double **anglesEntropy1D, double **dihedralsEntropy1D, double **bbEntropy,
                            double **baEntropy, double **bdEntropy, double **aaEntropy, double **adEntropy,
                            double **ddEntropy);

#endif /* __cplusplus */
#endif /* PARENT_GB300_IO_H */
