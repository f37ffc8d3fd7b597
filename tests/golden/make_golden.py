"""Regenerates the golden fixtures in this directory from the reference itself.

Run where the reference sources exist (they are never read by the tests):
    python tests/golden/make_golden.py [REF_ROOT]

Steps:
1. build the reference programs from their own sources into oracle/_ref
   (oracle/Makefile, single-rank MPI stand-in header);
2. convert the reference's ubiquitin-dimer test system (test_system/UBQ_UBM2
   .top/.xtc) to .bat with the reference BAT_builder.x, then cut a DOF subset
   (the first K_SUB dihedrals with their bonds/angles, all 801 frames, FP64);
3. write a small seeded synthetic FP32 trajectory with the product's generator;
4. run the reference PARENT.x (50 bins), get_PAR_MIE.x, get_PAR_MIST.x (one
   OpenMP thread: the canonical tie order) and get_PAR_info.x on both;
5. copy the reference's shipped golden tails (sample_output_MIE.txt,
   sample_output_MIST.txt) for the full-system pin;
6. decode the test system's .xtc with the reference's xdrfile (oracle/_ref/
   xtc_dump.x) and keep the Cartesian coordinates of the atoms the subset's
   dihedrals use, renumbered in order of first use, with the subset's
   dihedral table (ubq_sub_xyz.npz): BAT_builder's conversion of exactly these
   coordinates is ubq_sub.bat.
Text outputs are stored gzip-compressed.
"""
from __future__ import annotations

import gzip
import os
import shutil
import struct
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

K_SUB = 30          # dihedrals in the ubiquitin subset (33 atoms, 93 DOFs)
SYN = dict(n_atoms=24, n_frames=2000, double_prec=0, seed=20261203, n_latents=8,
           frac_bimodal_dih=0.2, frac_bimodal_bond=0.05, p_switch=1e-3)
BINS = (50,) * 6


def run(cmd, **kw):
    print("+", " ".join(map(str, cmd)))
    return subprocess.run(list(map(str, cmd)), check=True, **kw)


def subset_bat(src: Path, dst: Path, k: int) -> None:
    """Writes the first k dihedrals (plus the root bonds/angle) of a .bat."""
    raw = src.read_bytes()
    version, prec, nd, nf = struct.unpack_from("<4i", raw, 0)
    assert version >= 3
    es = 8 if prec else 4
    off = 16
    atoms = raw[off: off + (nd + 3) * 51]
    off += (nd + 3) * 51
    dih = raw[off: off + nd * 24]
    off += nd * 24
    masses = raw[off: off + (nd + 3) * 4]
    off += (nd + 3) * 4
    fb = 44 + (9 + 3 * nd) * es
    out = bytearray(struct.pack("<4i", version, prec, k, nf))
    out += atoms[: (k + 3) * 51] + dih[: k * 24] + masses[: (k + 3) * 4]
    keep = 44 + (9 + 3 * k) * es
    for f in range(nf):
        out += raw[off + f * fb: off + f * fb + keep]
    assert off + nf * fb == len(raw)
    dst.write_bytes(bytes(out))


def gz(src: Path, dst: Path) -> None:
    with open(src, "rb") as fi, open(dst, "wb") as raw:
        with gzip.GzipFile(fileobj=raw, mode="wb", compresslevel=9, mtime=0) as fo:
            shutil.copyfileobj(fi, fo)


def reference_outputs(ref: Path, bat: Path, stem: str, work: Path) -> None:
    par = work / f"{stem}.par"
    env = dict(os.environ, OMP_NUM_THREADS="1")
    run([ref / "PARENT.x", bat, par, *BINS], env=env, stdout=subprocess.DEVNULL)
    shutil.copy(par, HERE / f"{stem}_ref.par")
    with open(work / f"{stem}_MIE.txt", "w") as f:
        run([ref / "get_PAR_MIE.x", par], stdout=f)
    gz(work / f"{stem}_MIE.txt", HERE / f"{stem}_ref_MIE.txt.gz")
    run([ref / "get_PAR_MIST.x", par, work / f"{stem}_MIST.txt"], env=env, stdout=subprocess.DEVNULL)
    gz(work / f"{stem}_MIST.txt", HERE / f"{stem}_ref_MIST.txt.gz")
    with open(work / f"{stem}_info.txt", "w") as f:
        run([ref / "get_PAR_info.x", par], stdout=f)
    gz(work / f"{stem}_info.txt", HERE / f"{stem}_ref_info.txt.gz")


def ubq_sub_cartesian(ref: Path, xtc: Path, full_bat: Path, work: Path, k: int) -> None:
    """Step 6: Cartesian input of the BAT conversion for the first k dihedrals."""
    import numpy as np
    raw_path = work / "ubq_xyz.raw"
    run([ref / "xtc_dump.x", xtc, raw_path], stdout=subprocess.DEVNULL)
    raw = raw_path.read_bytes()
    na, nf = struct.unpack_from("<2i", raw, 0)
    xyz = np.frombuffer(raw[8:], dtype=np.float32).reshape(nf, na, 3)
    braw = full_bat.read_bytes()
    _, _, nd, _ = struct.unpack_from("<4i", braw, 0)
    off = 16 + (nd + 3) * 51
    dih = np.frombuffer(braw[off: off + nd * 24], dtype=np.int32).reshape(nd, 6)[:k].copy()
    atoms = []
    for row in dih:
        for a in row[:4]:
            if int(a) not in atoms:
                atoms.append(int(a))
    assert len(atoms) == k + 3 and (dih[:, 5] <= k).all()
    renum = {a: i + 1 for i, a in enumerate(atoms)}
    for row in dih:
        row[:4] = [renum[int(a)] for a in row[:4]]
    sub = np.ascontiguousarray(xyz[:, [a - 1 for a in atoms], :])
    np.savez_compressed(HERE / "ubq_sub_xyz.npz", xyz=sub, dih=dih)


def main() -> None:
    ref_root = Path(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
    run(["make", "-s", "-C", ROOT / "oracle", "ref", f"REF_ROOT={ref_root}", "-j4"])
    ref = ROOT / "oracle" / "_ref"
    import tempfile
    work = Path(tempfile.mkdtemp(prefix="pg_golden_"))

    ts = ref_root / "test_system"
    run([ref / "BAT_builder.x", "-t", ts / "UBQ_UBM2.top", "-x", ts / "UBQ_UBM2.xtc", "-o",
         work / "ubq.bat", "-bb", "CA C N H1 O1"], stdout=subprocess.DEVNULL)
    subset_bat(work / "ubq.bat", HERE / "ubq_sub.bat", K_SUB)
    reference_outputs(ref, HERE / "ubq_sub.bat", "ubq_sub", work)

    import parent_gb300 as pg
    t = pg.synth_host(**SYN)
    pg.write_bat(HERE / "synth_small.bat", t)
    reference_outputs(ref, HERE / "synth_small.bat", "synth_small", work)

    for name in ("sample_output_MIE.txt", "sample_output_MIST.txt"):
        shutil.copy(ts / "sample_output" / name, HERE / f"ubq_full_{name}")
    ubq_sub_cartesian(ref, ts / "UBQ_UBM2.xtc", work / "ubq.bat", work, K_SUB)
    shutil.rmtree(work, ignore_errors=True)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
