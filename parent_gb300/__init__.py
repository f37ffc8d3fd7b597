"""parent_gb300 — Python binding of the GB300 engine for PARENT's hot path.

A thin ctypes layer over the C ABI in include/parent_gb300.h (the library is
parent_gb300/lib/libparent_gb300.so, built in-tree by parent_gb300/build.py).
It mirrors the reference's stages:

  Engine.entropy(traj, bins)      PARENT.x                (src/PARENT/PARENT.cpp)
  Engine.mist(n_dih, body)        get_PAR_MIST.x          (src/process_output/get_PAR_MIST.cpp)
  write_mie_text / write_info_text  get_PAR_MIE.x / get_PAR_info.x
  read_bat / write_par / read_par   the io library      (src/util/io/io_binary.cpp)

Errors raise PGError carrying the C status code and message. There is no CPU
fallback: without the built library (or without a GPU for the compute calls)
every call fails loudly.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "lib" / "libparent_gb300.so"
BIN_DIR = _PKG / "bin"

PG_OK, PG_ERR_ARG, PG_ERR_IO, PG_ERR_FORMAT, PG_ERR_DATA, PG_ERR_CUDA, PG_ERR_NOMEM, PG_ERR_TIMEOUT, PG_ERR_UNSUPPORTED = range(9)
FORM_AUTO, FORM_HIST, FORM_ONEHOT = 0, 1, 2
FORMS = {"auto": FORM_AUTO, "hist": FORM_HIST, "onehot": FORM_ONEHOT}
TYPE_B, TYPE_A, TYPE_D = 0, 1, 2
MAX_BINS_2D = 218


class PGError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[pg status {code}] {msg}")
        self.code = code


class BatView(C.Structure):
    _fields_ = [("n_dihedrals", C.c_int), ("n_frames", C.c_int), ("double_prec", C.c_int),
                ("on_device", C.c_int), ("ld", C.c_int64), ("bonds", C.c_void_p),
                ("angles", C.c_void_p), ("dihedrals", C.c_void_p)]


class ParBodyC(C.Structure):
    _fields_ = [(n, C.POINTER(C.c_double)) for n in
                ("s1_b", "s1_a", "s1_d", "bb", "ba", "bd", "aa", "ad", "dd")]


class MistEdge(C.Structure):
    _fields_ = [("type_in", C.c_int), ("type_out", C.c_int), ("index_in", C.c_int),
                ("index_out", C.c_int), ("mi", C.c_double), ("left", C.c_int), ("pad_", C.c_int)]


_EDGE_DTYPE = np.dtype([("type_in", "<i4"), ("type_out", "<i4"), ("index_in", "<i4"), ("index_out", "<i4"),
                        ("mi", "<f8"), ("left", "<i4"), ("pad_", "<i4")])
assert _EDGE_DTYPE.itemsize == C.sizeof(MistEdge)


def _edges_array(buf, n: int) -> np.ndarray:
    """The first n pg_mist_edge structs of a ctypes array as a numpy record
    array (t1, t2, i1, i2, mi, left), read in place."""
    raw = np.frombuffer(buf, dtype=_EDGE_DTYPE, count=n)
    arr = np.empty(n, dtype=[("t1", "i4"), ("t2", "i4"), ("i1", "i4"), ("i2", "i4"), ("mi", "f8"), ("left", "i4")])
    for f, g in (("t1", "type_in"), ("t2", "type_out"), ("i1", "index_in"), ("i2", "index_out"), ("mi", "mi"),
                 ("left", "left")):
        arr[f] = raw[g]
    return arr


class SynthSpec(C.Structure):
    _fields_ = [("n_atoms", C.c_int), ("n_frames", C.c_int), ("double_prec", C.c_int),
                ("n_latents", C.c_int), ("seed", C.c_uint64), ("frac_bimodal_dih", C.c_double),
                ("frac_bimodal_bond", C.c_double), ("p_switch", C.c_double)]


_lib = None


def lib() -> C.CDLL:
    """Loads the C-ABI library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise PGError(PG_ERR_UNSUPPORTED,
                      f"{LIB_PATH} is missing: build it with `python -c \"import __graft_entry__ as g; g.build()\"`")
    L = C.CDLL(str(LIB_PATH))
    vp, i, i64, dp, cp = C.c_void_p, C.c_int, C.c_int64, C.POINTER(C.c_double), C.c_char_p
    sig = {
        "pg_create": (i, [C.POINTER(vp), i]),
        "pg_destroy": (None, [vp]),
        "pg_last_error": (cp, [vp]),
        "pg_last_global_error": (cp, []),
        "pg_entropy": (i, [vp, C.POINTER(BatView), C.POINTER(C.c_int), i, C.POINTER(ParBodyC)]),
        "pg_mist": (i, [vp, i, C.POINTER(ParBodyC), C.POINTER(MistEdge), dp]),
        "pg_entropy_batch": (i, [vp, i, C.POINTER(BatView), C.POINTER(C.c_int), i, C.POINTER(ParBodyC),
                                 C.POINTER(C.POINTER(MistEdge)), dp]),
        "pg_entropy_shard": (i, [vp, C.POINTER(BatView), C.POINTER(C.c_int), i, i, i, C.POINTER(ParBodyC)]),
        "pg_shard_mask": (i, [i, C.POINTER(C.c_int), i, i, C.POINTER(C.c_uint8)]),
        "pg_last_timings": (i, [vp, dp]),
        "pg_launch_count": (i64, [vp]),
        "pg_last_form": (i, [vp]),
        "pg_stream": (vp, [vp]),
        "pg_predict_pair_ms": (i, [vp, i, i, C.POINTER(C.c_int), i, dp]),
        "pg_pair_counts": (i, [vp, C.POINTER(BatView), C.POINTER(C.c_int), i, i, C.POINTER(C.c_int),
                               C.POINTER(C.c_int), C.POINTER(C.c_int64), i64]),
        "pg_dof_stats": (i, [vp, dp, dp, dp]),
        "pg_bat_read": (i, [cp, C.POINTER(vp)]),
        "pg_bat_read_device": (i, [cp, i, C.POINTER(vp)]),
        "pg_bat_from_cartesian": (i, [vp, vp, i, i, i, C.POINTER(C.c_int), i, C.POINTER(BatView)]),
        "pg_bat_free": (None, [vp]),
        "pg_bat_view_of": (i, [vp, C.POINTER(BatView)]),
        "pg_bat_n_dihedrals": (i, [vp]),
        "pg_bat_dihedral_table": (i, [vp, C.POINTER(C.c_int)]),
        "pg_bat_n_frames": (i, [vp]),
        "pg_bat_write_synthetic": (i, [cp, C.POINTER(BatView)]),
        "pg_par_write": (i, [cp, vp, C.POINTER(C.c_int), C.POINTER(ParBodyC)]),
        "pg_par_read": (i, [cp, C.POINTER(vp)]),
        "pg_par_free": (None, [vp]),
        "pg_par_n_dihedrals": (i, [vp]),
        "pg_par_body_of": (i, [vp, C.POINTER(ParBodyC)]),
        "pg_par_bins": (i, [vp, C.POINTER(C.c_int)]),
        "pg_write_mie_text": (i, [cp, i, C.POINTER(ParBodyC)]),
        "pg_write_mie_text_device": (i, [vp, cp, i, C.POINTER(ParBodyC)]),
        "pg_format_g12": (i, [C.c_double, cp]),
        "pg_check_wait_timeout": (i, [vp, C.c_double]),
        "pg_write_mist_text": (i, [cp, i, C.POINTER(MistEdge), dp]),
        "pg_write_info_text": (i, [cp, vp]),
        "pg_synth_host": (i, [C.POINTER(SynthSpec), vp, vp, vp, i64, i]),
        "pg_synth_device": (i, [vp, C.POINTER(SynthSpec), vp, vp, vp, i64]),
        "pg_prefetch": (i, [vp, C.POINTER(BatView)]),
        "pg_entropy_ahead": (i, [vp, C.POINTER(BatView), C.POINTER(C.c_int), i, C.POINTER(ParBodyC),
                                 C.POINTER(BatView)]),
        "pg_probe_smem_red_rate": (i, [vp, dp]),
        "pg_device_alloc": (i, [vp, C.c_size_t, C.POINTER(vp)]),
        "pg_device_free": (i, [vp, vp]),
        "pg_memcpy": (i, [vp, vp, vp, C.c_size_t, i]),
        "pg_host_alloc_pinned": (i, [C.c_size_t, C.POINTER(vp)]),
        "pg_host_free_pinned": (i, [vp]),
        "pg_synchronize": (i, [vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def exported_symbols() -> list[str]:
    """Names of every pg_* function the header declares (for ABI checks)."""
    import re
    hdr = (_PKG.parent / "include" / "parent_gb300.h").read_text()
    return re.findall(r"PG_API\s+[\w\s\*]+?\b(pg_\w+)\s*\(", hdr)


def _check(rc: int, ctx=None) -> None:
    if rc != PG_OK:
        L = lib()
        msg = (L.pg_last_error(ctx) if ctx else L.pg_last_global_error()) or b""
        raise PGError(rc, msg.decode(errors="replace"))


# ----------------------------------------------------------------- data

def block_sizes(n_dih: int) -> dict[str, int]:
    nb, na, nd = n_dih + 2, n_dih + 1, n_dih
    return {"s1_b": nb, "s1_a": na, "s1_d": nd, "bb": nb * (nb - 1) // 2, "ba": nb * na,
            "bd": nb * nd, "aa": na * (na - 1) // 2, "ad": na * nd, "dd": nd * (nd - 1) // 2}


@dataclass
class ParBody:
    """Entropies in .par body layout (write_PAR_body, io_binary.cpp:606-631)."""
    n_dih: int
    blocks: dict

    @classmethod
    def empty(cls, n_dih: int) -> "ParBody":
        return cls(n_dih, {k: np.zeros(n, dtype=np.float64) for k, n in block_sizes(n_dih).items()})

    def c(self) -> ParBodyC:
        b = ParBodyC()
        for k, arr in self.blocks.items():
            assert arr.dtype == np.float64 and arr.flags.c_contiguous
            setattr(b, k, arr.ctypes.data_as(C.POINTER(C.c_double)))
        return b

    def flat(self) -> np.ndarray:
        return np.concatenate([self.blocks[k] for k in block_sizes(self.n_dih)])


class DeviceParBody:
    """A .par body in device memory of the engine's GPU: one flat buffer of
    doubles in block_sizes order (e.g. a torch CUDA tensor's data_ptr()),
    usable as the output of Engine.entropy_shard and the input of
    Engine.mist, so a sharded body can be reduced and fed to MIST without
    passing through the host."""

    def __init__(self, n_dih: int, ptr: int):
        self.n_dih = n_dih
        self.ptr = int(ptr)

    def c(self) -> ParBodyC:
        b = ParBodyC()
        o = 0
        for k, n in block_sizes(self.n_dih).items():
            setattr(b, k, C.cast(C.c_void_p(self.ptr + 8 * o), C.POINTER(C.c_double)))
            o += n
        return b


@dataclass
class Trajectory:
    """DOF-major columns: bonds (nDih+2, F), angles (nDih+1, F), dihedrals (nDih, F)."""
    bonds: np.ndarray
    angles: np.ndarray
    dihedrals: np.ndarray

    @property
    def n_dih(self) -> int:
        return self.dihedrals.shape[0]

    @property
    def n_frames(self) -> int:
        return self.bonds.shape[1]

    @property
    def double_prec(self) -> int:
        return 1 if self.bonds.dtype == np.float64 else 0

    def view(self) -> BatView:
        dt = self.bonds.dtype
        for a in (self.bonds, self.angles, self.dihedrals):
            if a.dtype != dt or not a.flags.c_contiguous or a.dtype not in (np.float32, np.float64):
                raise PGError(PG_ERR_ARG, "columns must be C-contiguous float32/float64 of one dtype")
        return BatView(self.n_dih, self.n_frames, self.double_prec, 0, self.n_frames,
                       self.bonds.ctypes.data, self.angles.ctypes.data,
                       self.dihedrals.ctypes.data if self.dihedrals.size else self.angles.ctypes.data)

    def as_float64(self) -> "Trajectory":
        return Trajectory(*(np.ascontiguousarray(a, dtype=np.float64)
                            for a in (self.bonds, self.angles, self.dihedrals)))


def synth_host(n_atoms: int, n_frames: int, double_prec: int = 1, seed: int = 1, n_latents: int = 8,
               frac_bimodal_dih: float = 0.0, frac_bimodal_bond: float = 0.0,
               p_switch: float = 1e-3, threads: int = 0) -> Trajectory:
    """Seeded synthetic linear-chain trajectory generated on the host."""
    dt = np.float64 if double_prec else np.float32
    nd = n_atoms - 3
    t = Trajectory(np.empty((nd + 2, n_frames), dt), np.empty((nd + 1, n_frames), dt),
                   np.empty((nd, n_frames), dt))
    spec = SynthSpec(n_atoms, n_frames, double_prec, n_latents, seed, frac_bimodal_dih,
                     frac_bimodal_bond, p_switch)
    _check(lib().pg_synth_host(C.byref(spec), t.bonds.ctypes.data, t.angles.ctypes.data,
                               t.dihedrals.ctypes.data if nd else t.angles.ctypes.data,
                               n_frames, threads))
    return t


# ----------------------------------------------------------------- engine

class Engine:
    """One GPU context (pg_create) with its own stream."""

    def __init__(self, device: int = 0):
        self._ctx = C.c_void_p()
        _check(lib().pg_create(C.byref(self._ctx), device))

    def close(self) -> None:
        if self._ctx:
            lib().pg_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> C.c_void_p:
        return self._ctx

    def entropy(self, traj: Trajectory | BatView, bins=(50,) * 6, form: str | int = "auto",
                out: ParBody | None = None, keep_result: bool = True,
                next: Trajectory | BatView | None = None) -> ParBody | None:
        """PARENT.x on a trajectory; returns the .par body (or None if
        keep_result=False). next: a host trajectory whose upload runs on the
        copy engine during this call, for the following call on it
        (pg_entropy_ahead)."""
        v = traj if isinstance(traj, BatView) else traj.view()
        b = (C.c_int * 6)(*bins)
        f = FORMS[form] if isinstance(form, str) else int(form)
        if keep_result and out is None:
            out = ParBody.empty(v.n_dihedrals)
        body = out.c() if keep_result else None
        if next is None:
            _check(lib().pg_entropy(self._ctx, C.byref(v), b, f, C.byref(body) if body else None), self._ctx)
        else:
            nv = next if isinstance(next, BatView) else next.view()
            self._prefetched = (next, nv)  # the host columns stay alive until used
            _check(lib().pg_entropy_ahead(self._ctx, C.byref(v), b, f, C.byref(body) if body else None,
                                          C.byref(nv)), self._ctx)
        return out if keep_result else None

    def bat_from_cartesian(self, xyz: np.ndarray, dih: np.ndarray, double_prec: int = 1) -> BatView:
        """BAT_builder's conversion on the GPU: xyz (frames, nDih+3, 3) float32
        in nm (host array), dih the .bat dihedral table (nDih, 6). Returns a
        device view of the BAT columns (valid until the next conversion)."""
        xyz = np.ascontiguousarray(xyz, dtype=np.float32)
        dih = np.ascontiguousarray(dih, dtype=np.int32)
        if xyz.ndim != 3 or xyz.shape[2] != 3 or dih.ndim != 2 or dih.shape[1] != 6:
            raise PGError(PG_ERR_ARG, "xyz must be (frames, atoms, 3) and dih (n_dih, 6)")
        if xyz.shape[1] != dih.shape[0] + 3:
            raise PGError(PG_ERR_ARG, "atoms must equal n_dih + 3")
        v = BatView()
        _check(lib().pg_bat_from_cartesian(self._ctx, xyz.ctypes.data, 0, xyz.shape[0], dih.shape[0],
                                           dih.ctypes.data_as(C.POINTER(C.c_int)), int(double_prec), C.byref(v)),
               self._ctx)
        return v

    def write_mie_text(self, path: str | Path | None, body: ParBody) -> None:
        """get_PAR_MIE.x's text with the pair lines formatted on this GPU."""
        bc = body.c()
        _check(lib().pg_write_mie_text_device(self._ctx, str(path).encode() if path else None, body.n_dih,
                                              C.byref(bc)), self._ctx)

    def mist(self, n_dih: int, body: "ParBody | DeviceParBody | None" = None):
        """MIST tree: (edges as a structured numpy array, totals[10]), from the
        resident MI matrix or from a host or device body."""
        n = 3 * n_dih + 2
        edges = (MistEdge * max(n, 1))()
        totals = (C.c_double * 10)()
        bc = body.c() if body is not None else None
        _check(lib().pg_mist(self._ctx, n_dih, C.byref(bc) if bc else None, edges, totals), self._ctx)
        return _edges_array(edges, n), np.array(totals[:], dtype=np.float64)

    def entropy_batch(self, trajs, bins=(50,) * 6, form: str | int = "auto", bodies: bool = True,
                      trees: bool = True):
        """PARENT.x + get_PAR_MIST.x on many independent trajectories in one
        run (pg_entropy_batch). bodies: True (allocate), False (no bodies) or
        a list of ParBody to fill. Returns (bodies, trees): a list of ParBody
        (or None) and a list of (edges, totals) as Engine.mist returns them
        (or None)."""
        views = [t if isinstance(t, BatView) else t.view() for t in trajs]
        n = len(views)
        arr = (BatView * n)(*views)
        b = (C.c_int * 6)(*bins)
        f = FORMS[form] if isinstance(form, str) else int(form)
        if isinstance(bodies, (list, tuple)):
            outs = list(bodies)           # caller's buffers (e.g. in pinned memory)
        else:
            outs = [ParBody.empty(v.n_dihedrals) for v in views] if bodies else None
        oc = (ParBodyC * n)(*[o.c() for o in outs]) if outs else None
        ebufs = [(MistEdge * max(3 * v.n_dihedrals + 2, 1))() for v in views] if trees else None
        ep = (C.POINTER(MistEdge) * n)(*[C.cast(e, C.POINTER(MistEdge)) for e in ebufs]) if trees else None
        totals = np.zeros(10 * n) if trees else None
        _check(lib().pg_entropy_batch(self._ctx, n, arr, b, f, oc, ep,
                                      totals.ctypes.data_as(C.POINTER(C.c_double)) if trees else None),
               self._ctx)
        res = None
        if trees:
            res = []
            for k, (v, e) in enumerate(zip(views, ebufs)):
                res.append((_edges_array(e, 3 * v.n_dihedrals + 2), totals[10 * k:10 * k + 10].copy()))
        return outs, res

    def prefetch(self, traj: Trajectory | BatView) -> None:
        """Queue the upload of a host view's columns for the next entropy()
        call on the same view (pg_prefetch): the copy engine moves them while
        the current work runs."""
        v = traj if isinstance(traj, BatView) else traj.view()
        self._prefetched = (traj, v)  # the host columns stay alive until used
        _check(lib().pg_prefetch(self._ctx, C.byref(v)), self._ctx)

    def entropy_shard(self, traj: Trajectory | BatView, bins, shard: int, n_shards: int,
                      form: str | int = "auto", out: "ParBody | DeviceParBody | None" = None):
        """Shard `shard` of `n_shards` of PARENT.x (pg_entropy_shard): this shard's
        2D entropies (and, for shard 0, the 1D entropies), zeros elsewhere,
        into `out` (host or device body; a new host body by default)."""
        v = traj if isinstance(traj, BatView) else traj.view()
        b = (C.c_int * 6)(*bins)
        f = FORMS[form] if isinstance(form, str) else int(form)
        if out is None:
            out = ParBody.empty(v.n_dihedrals)
        body = out.c()
        _check(lib().pg_entropy_shard(self._ctx, C.byref(v), b, f, shard, n_shards, C.byref(body)), self._ctx)
        return out

    def pair_counts(self, traj: Trajectory | BatView, bins, pairs, form: str = "hist") -> list[np.ndarray]:
        """Raw 2D histograms of explicit (g1 < g2) pairs from the GPU pair kernel."""
        v = traj if isinstance(traj, BatView) else traj.view()
        b = (C.c_int * 6)(*bins)
        nb, na = v.n_dihedrals + 2, v.n_dihedrals + 1
        tb = lambda g: 0 if g < nb else (1 if g < nb + na else 2)
        g1 = (C.c_int * len(pairs))(*[p[0] for p in pairs])
        g2 = (C.c_int * len(pairs))(*[p[1] for p in pairs])
        stride = max(bins[3:]) ** 2
        out = np.zeros((len(pairs), stride), dtype=np.int64)
        _check(lib().pg_pair_counts(self._ctx, C.byref(v), b, FORMS[form], len(pairs), g1, g2,
                                    out.ctypes.data_as(C.POINTER(C.c_int64)), stride), self._ctx)
        res = []
        for k, (a, c) in enumerate(pairs):
            B1, B2 = bins[3 + tb(a)], bins[3 + tb(c)]
            res.append(out[k, :B1 * B2].reshape(B1, B2).copy())
        return res

    def predict_pair_ms(self, n_dih: int, n_frames: int, bins, form: str = "auto") -> float:
        """The autotuner's predicted pair-kernel milliseconds for a geometry."""
        ms = C.c_double()
        _check(lib().pg_predict_pair_ms(self._ctx, n_dih, n_frames, (C.c_int * 6)(*bins), FORMS[form],
                                        C.byref(ms)), self._ctx)
        return ms.value

    def dof_stats(self, D: int):
        mn, mx, sh = (np.zeros(D) for _ in range(3))
        P = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        _check(lib().pg_dof_stats(self._ctx, P(mn), P(mx), P(sh)), self._ctx)
        return mn, mx, sh

    def timings(self) -> np.ndarray:
        ms = (C.c_double * 5)()
        lib().pg_last_timings(self._ctx, ms)
        return np.array(ms[:])

    def launch_count(self) -> int:
        return int(lib().pg_launch_count(self._ctx))

    def last_form(self) -> str:
        return {FORM_HIST: "hist", FORM_ONEHOT: "onehot"}.get(lib().pg_last_form(self._ctx), "none")

    def probe_smem_red_rate(self) -> float:
        """Measured peak of conflict-free warp-wide shared-memory reductions (per s)."""
        r = C.c_double()
        _check(lib().pg_probe_smem_red_rate(self._ctx, C.byref(r)), self._ctx)
        return r.value

    def stream(self) -> int:
        return lib().pg_stream(self._ctx) or 0

    # device memory through the library
    def alloc(self, nbytes: int) -> int:
        p = C.c_void_p()
        _check(lib().pg_device_alloc(self._ctx, nbytes, C.byref(p)), self._ctx)
        return p.value

    def free(self, ptr: int) -> None:
        _check(lib().pg_device_free(self._ctx, C.c_void_p(ptr)), self._ctx)

    def memcpy(self, dst: int, src: int, nbytes: int, kind: int) -> None:
        _check(lib().pg_memcpy(self._ctx, C.c_void_p(dst), C.c_void_p(src), nbytes, kind), self._ctx)

    def synchronize(self) -> None:
        _check(lib().pg_synchronize(self._ctx), self._ctx)

    def synth_device(self, n_atoms: int, n_frames: int, double_prec: int, ptrs, ld: int, seed: int = 1,
                     n_latents: int = 8, frac_bimodal_dih: float = 0.0, frac_bimodal_bond: float = 0.0,
                     p_switch: float = 1e-3) -> None:
        spec = SynthSpec(n_atoms, n_frames, double_prec, n_latents, seed, frac_bimodal_dih,
                         frac_bimodal_bond, p_switch)
        _check(lib().pg_synth_device(self._ctx, C.byref(spec), *(C.c_void_p(p) for p in ptrs), ld), self._ctx)


# ----------------------------------------------------------------- files

class BatFile:
    """A .bat: header + DOF-major columns, read by pg_bat_read into pinned host
    memory, or with device=<index> by pg_bat_read_device into device memory
    (records streamed up and transposed on the GPU)."""

    def __init__(self, path: str | Path, device: int | None = None):
        self._h = C.c_void_p()
        if device is None:
            _check(lib().pg_bat_read(str(path).encode(), C.byref(self._h)))
        else:
            _check(lib().pg_bat_read_device(str(path).encode(), int(device), C.byref(self._h)))

    def view(self) -> BatView:
        v = BatView()
        _check(lib().pg_bat_view_of(self._h, C.byref(v)))
        return v

    @property
    def handle(self):
        return self._h

    def dihedral_table(self) -> np.ndarray:
        """The header's dihedral table, (nDih, 6) int32 (atoms 1-based, type, parent)."""
        n = lib().pg_bat_n_dihedrals(self._h)
        t = np.zeros((max(n, 0), 6), np.int32)
        _check(lib().pg_bat_dihedral_table(self._h, t.ctypes.data_as(C.POINTER(C.c_int))))
        return t

    def close(self):
        if self._h:
            lib().pg_bat_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ParFile:
    """A .par read by pg_par_read."""

    def __init__(self, path: str | Path):
        self._h = C.c_void_p()
        _check(lib().pg_par_read(str(path).encode(), C.byref(self._h)))
        self.n_dih = lib().pg_par_n_dihedrals(self._h)
        bc = ParBodyC()
        _check(lib().pg_par_body_of(self._h, C.byref(bc)))
        self.body = ParBody(self.n_dih, {k: np.ctypeslib.as_array(getattr(bc, k), (n,)).copy() if n else np.zeros(0)
                                         for k, n in block_sizes(self.n_dih).items()})
        b = (C.c_int * 6)()
        _check(lib().pg_par_bins(self._h, b))
        self.bins = tuple(b)

    @property
    def handle(self):
        return self._h

    def __del__(self):
        try:
            if self._h:
                lib().pg_par_free(self._h)
        except Exception:
            pass


def write_bat(path: str | Path, traj: Trajectory) -> None:
    _check(lib().pg_bat_write_synthetic(str(path).encode(), C.byref(traj.view())))


def write_par(path: str | Path, bat: BatFile, bins, body: ParBody) -> None:
    b = (C.c_int * 6)(*bins)
    bc = body.c()
    _check(lib().pg_par_write(str(path).encode(), bat.handle, b, C.byref(bc)))


def write_mie_text(path: str | Path | None, body: ParBody) -> None:
    bc = body.c()
    _check(lib().pg_write_mie_text(str(path).encode() if path else None, body.n_dih, C.byref(bc)))


def write_mist_text(path: str | Path | None, n_dih: int, edges: np.ndarray, totals) -> None:
    n = len(edges)
    arr = (MistEdge * max(n, 1))()
    for k, e in enumerate(edges):
        arr[k] = MistEdge(int(e["t1"]), int(e["t2"]), int(e["i1"]), int(e["i2"]), float(e["mi"]), int(e["left"]), 0)
    t = (C.c_double * 10)(*totals)
    _check(lib().pg_write_mist_text(str(path).encode() if path else None, n_dih, arr, t))


def write_info_text(path: str | Path | None, par: ParFile) -> None:
    _check(lib().pg_write_info_text(str(path).encode() if path else None, par.handle))
