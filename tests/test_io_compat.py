"""The reference's io_binary functions with their own C++ signatures
(include/parent_gb300_io.h, exported by libparent_gb300.so).

A small C++ program built here against that header re-writes the golden
.par and .bat files through read_*/write_* and must reproduce them byte for
byte, and the reference's own post-processors (get_PAR_MIE.cpp,
get_PAR_info.cpp and get_PAR_MIST.cpp with their util.cpp, compiled from the
reference's sources where they exist) linked against libparent_gb300 instead
of io_binary.cpp must print the reference's own outputs for the golden .par
files. CPU only: nothing here touches a GPU.
"""
from __future__ import annotations

import gzip
import shutil
import subprocess
from pathlib import Path

import pytest

import oracle
from conftest import GOLDEN, ROOT

INCLUDE = ROOT / "include"
LIBDIR = ROOT / "parent_gb300" / "lib"

ROUNDTRIP = r'''
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>
#include "parent_gb300_io.h"
using namespace std;

static int par(const char *in, const char *out) {
    ifstream f(in, ios::binary);
    int nd, prec, nf, ver, b2, a2, d2, b1, a1, d1;
    vector<vector<int> > dih; vector<float> m; vector<string> res, at, mol; vector<int> rn;
    int rc = read_PAR_header(&f, &nd, &prec, &nf, &dih, &m, &ver, &b2, &a2, &d2, &b1, &a1, &d1, &res, &rn, &at, &mol);
    if (rc) return 10 + rc;
    double *blk[9];
    rc = read_PAR_body(&f, nd, &blk[0], &blk[1], &blk[2], &blk[3], &blk[4], &blk[5], &blk[6], &blk[7], &blk[8]);
    if (rc) return 20 + rc;
    ofstream o(out, ios::binary);
    rc = write_PAR_header(&o, nd, prec, nf, &dih, &m, b1, a1, d1, b2, a2, d2, &res, &rn, &at, &mol);
    rc |= write_PAR_body(&o, nd, blk[0], blk[1], blk[2], blk[3], blk[4], blk[5], blk[6], blk[7], blk[8]);
    for (int k = 0; k < 9; k++) free(blk[k]);
    return rc ? 30 : 0;
}

static int bat(const char *in, const char *out) {
    ifstream f(in, ios::binary);
    int prec, nf;
    vector<vector<int> > dih; vector<float> m; vector<string> res, at, mol; vector<int> rn;
    int rc = read_BAT_header(&f, &prec, &nf, &dih, &m, &res, &rn, &at, &mol);
    if (rc) return 40 + rc;
    const int nd = (int)dih.size();
    ofstream o(out, ios::binary);
    if (write_BAT_header(&o, prec, nf, &dih, &m, &res, &rn, &at, &mol)) return 50;
    vector<double> b(nd + 2), a(nd + 1), d(nd + 1);
    float box[3][3], t, xp;
    double cart[3], th, ph, di;
    for (int fr = 0; fr < nf; fr++) {
        if (read_BAT_frame(&f, prec, nd, &t, &xp, (float **)box, cart, &th, &ph, &di, b.data(), a.data(), d.data()))
            return 60;
        if (write_BAT_frame(&o, prec, nd, t, xp, (float **)box, cart, th, ph, di, b.data(), a.data(), d.data()))
            return 70;
    }
    return 0;
}

// a .par cut inside its body: the fail bit comes back, the header reads
static int truncated(const char *in) {
    ifstream f(in, ios::binary);
    int nd, prec, nf, ver, b2, a2, d2, b1, a1, d1;
    vector<vector<int> > dih; vector<float> m; vector<string> res, at, mol; vector<int> rn;
    if (read_PAR_header(&f, &nd, &prec, &nf, &dih, &m, &ver, &b2, &a2, &d2, &b1, &a1, &d1, &res, &rn, &at, &mol))
        return 80;
    double *blk[9];
    int rc = read_PAR_body(&f, nd, &blk[0], &blk[1], &blk[2], &blk[3], &blk[4], &blk[5], &blk[6], &blk[7], &blk[8]);
    for (int k = 0; k < 9; k++) free(blk[k]);
    return rc == 0 ? 81 : 0;
}

// a header field outside its range: 1, nothing more read
static int corrupt(const char *in) {
    ifstream f(in, ios::binary);
    int nd, prec, nf, ver, b2, a2, d2, b1, a1, d1;
    vector<vector<int> > dih; vector<float> m; vector<string> res, at, mol; vector<int> rn;
    int rc = read_PAR_header(&f, &nd, &prec, &nf, &dih, &m, &ver, &b2, &a2, &d2, &b1, &a1, &d1, &res, &rn, &at, &mol);
    return rc == 1 && res.empty() ? 0 : 90;
}

int main(int argc, char **argv) {
    if (!strcmp(argv[1], "par")) return par(argv[2], argv[3]);
    if (!strcmp(argv[1], "bat")) return bat(argv[2], argv[3]);
    if (!strcmp(argv[1], "truncated")) return truncated(argv[2]);
    if (!strcmp(argv[1], "corrupt")) return corrupt(argv[2]);
    return 2;
}
'''


def _link_flags():
    return ["-L", str(LIBDIR), "-lparent_gb300", f"-Wl,-rpath,{LIBDIR}"]


@pytest.fixture(scope="module")
def tool(tmp_path_factory):
    d = tmp_path_factory.mktemp("io_compat")
    src = d / "roundtrip.cpp"
    src.write_text(ROUNDTRIP)
    exe = d / "roundtrip"
    subprocess.run(["g++", "-O1", "-std=c++17", "-I", str(INCLUDE), str(src), "-o", str(exe)] + _link_flags(),
                   check=True)
    return exe


@pytest.mark.parametrize("stem", ["ubq_sub_ref", "synth_small_ref"])
def test_par_rewritten_byte_identical(tool, tmp_path, stem):
    out = tmp_path / "copy.par"
    r = subprocess.run([str(tool), "par", str(GOLDEN / f"{stem}.par"), str(out)])
    assert r.returncode == 0
    assert out.read_bytes() == (GOLDEN / f"{stem}.par").read_bytes()


@pytest.mark.parametrize("stem", ["ubq_sub", "synth_small"])   # FP64 and FP32 frames
def test_bat_rewritten_byte_identical(tool, tmp_path, stem):
    out = tmp_path / "copy.bat"
    r = subprocess.run([str(tool), "bat", str(GOLDEN / f"{stem}.bat"), str(out)])
    assert r.returncode == 0
    assert out.read_bytes() == (GOLDEN / f"{stem}.bat").read_bytes()


def test_truncated_body_and_corrupt_header(tool, tmp_path):
    raw = (GOLDEN / "ubq_sub_ref.par").read_bytes()
    cut = tmp_path / "cut.par"
    cut.write_bytes(raw[:len(raw) - 100])
    assert subprocess.run([str(tool), "truncated", str(cut)]).returncode == 0
    bad = bytearray(raw)
    bad[0:4] = (-2).to_bytes(4, "little", signed=True)          # version < 0
    p = tmp_path / "bad.par"
    p.write_bytes(bytes(bad))
    r = subprocess.run([str(tool), "corrupt", str(p)], capture_output=True, text=True)
    assert r.returncode == 0
    assert "ERROR: FILE HEADER CORRUPTED. VERSION NUMBER (-2) < 0!" in r.stderr


def _reference_src():
    src = oracle.reference_root() / "src"
    return src if (src / "process_output" / "get_PAR_MIE.cpp").exists() else None


@pytest.mark.parametrize("prog", ["get_PAR_MIE", "get_PAR_info", "get_PAR_MIST"])
@pytest.mark.parametrize("stem", ["ubq_sub", "synth_small"])
def test_reference_post_processors_link_against_this_library(tmp_path, prog, stem):
    src = _reference_src()
    if src is None:
        pytest.skip("the reference sources are not on this machine")
    exe = tmp_path / prog
    cmd = ["g++", "-O1", "-w", "-ffp-contract=off", str(src / "process_output" / f"{prog}.cpp"),
           str(src / "util" / "util.cpp"), "-o", str(exe)] + _link_flags()
    if prog == "get_PAR_MIST":
        cmd[1:1] = ["-fopenmp", "-I", str(ROOT / "oracle" / "mpi_stub")]
    # no io_binary.cpp: read_PAR_header/read_PAR_body come from libparent_gb300
    subprocess.run(cmd, check=True)
    par = GOLDEN / f"{stem}_ref.par"
    want = gzip.open(GOLDEN / f"{stem}_ref_{prog.split('_')[-1]}.txt.gz", "rt").read()
    if prog == "get_PAR_MIST":
        out = tmp_path / "mist.txt"
        r = subprocess.run([str(exe), str(par), str(out)], capture_output=True, text=True,
                           env={"OMP_NUM_THREADS": "1", "PATH": "/usr/bin:/bin"})
        assert r.returncode == 0, r.stderr[-2000:]
        got = out.read_text()
    else:
        r = subprocess.run([str(exe), str(par)], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-2000:]
        got = r.stdout
    assert got == want


def test_library_exports_every_io_function_declared():
    """Every function include/parent_gb300_io.h declares is defined in the
    library with that C++ signature (nm demangles the exported names)."""
    import re
    hdr = (INCLUDE / "parent_gb300_io.h").read_text()
    names = re.findall(r"PG_IO_API\s+int\s+(\w+)\s*\(", hdr)
    assert len(names) == 8
    nm = shutil.which("nm")
    if nm is None:
        pytest.skip("nm is not installed")
    out = subprocess.run([nm, "-D", "--defined-only", "-C", str(LIBDIR / "libparent_gb300.so")],
                         capture_output=True, text=True, check=True).stdout
    for n in names:
        assert re.search(rf"\bT {n}\(std::basic_[io]fstream", out), n
