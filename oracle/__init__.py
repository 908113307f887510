"""CPU oracle for the two-site H_eff path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this package, as the checker or the timed CPU baseline; the product never
imports it.  See heff_oracle.c for what each function restates and for the
parity status (integer bookkeeping pinned to the reference's known answers;
matvec pinned to a literal transliteration and physics known answers, not to
reference-run outputs -- the Rust reference cannot be built here).

build() compiles heff_oracle.c twice with gcc: liborc.so, the checker
(-O3 -fopenmp -std=c11: ISO C mode keeps floating-point contraction off, so
its sums round the same on every host), and liborc_timed.so, the timed CPU
baseline (-O3 -std=gnu11 -ffp-contract=fast -funroll-loops: multiply-adds
fuse into FMA, as a tuned CPU build of the reference would; no -march, so the
same flags build on x86-64 and on aarch64, whose base ISA has FMA and NEON).
load() / load(timed=True) bind them with ctypes.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "heff_oracle.c"
BUILD = HERE / "_build"
LIB = BUILD / "liborc.so"
LIB_TIMED = BUILD / "liborc_timed.so"
FLAGS = {LIB: ["-O3", "-fopenmp", "-std=c11"],
         LIB_TIMED: ["-O3", "-fopenmp", "-std=gnu11", "-ffp-contract=fast", "-funroll-loops"]}


class orc_qindex(C.Structure):
    _fields_ = [("n_sectors", C.c_int32), ("charges", C.POINTER(C.c_int32)), ("dims", C.POINTER(C.c_int64))]


class orc_bst(C.Structure):
    _fields_ = [("kind", C.c_int32), ("rank", C.c_int32), ("legs", C.POINTER(orc_qindex)),
                ("n_blocks", C.c_int64), ("keys", C.POINTER(C.c_uint64)), ("offsets", C.POINTER(C.c_int64)),
                ("data", C.POINTER(C.c_double))]


def _build_one(lib: Path, force: bool) -> Path:
    if not force and lib.exists() and lib.stat().st_mtime >= SRC.stat().st_mtime:
        return lib
    BUILD.mkdir(parents=True, exist_ok=True)
    tmp = lib.with_suffix(".so.tmp")
    cmd = ["gcc", *FLAGS[lib], "-fPIC", "-shared", "-Wall", str(SRC), "-o", str(tmp), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


def build(force: bool = False) -> Path:
    """Builds the checker and the timed baseline; returns the checker's path."""
    _build_one(LIB_TIMED, force)
    return _build_one(LIB, force)


_libs = {}


def load(timed: bool = False) -> C.CDLL:
    if timed in _libs:
        return _libs[timed]
    path = _build_one(LIB_TIMED if timed else LIB, False)
    lib = C.CDLL(str(path))
    P = C.POINTER
    sig = {
        "orc_qn_pack": (C.c_uint64, [C.c_int, P(C.c_int32)]),
        "orc_qn_unpack": (None, [C.c_int, C.c_uint64, P(C.c_int32)]),
        "orc_key_pack": (C.c_uint64, [C.c_int, C.c_int, P(C.c_int32)]),
        "orc_key_unpack": (None, [C.c_int, C.c_int, C.c_uint64, P(C.c_int32)]),
        "orc_check_flux_rule": (C.c_int, [C.c_int, C.c_int, P(C.c_int32), P(C.c_int32), P(C.c_int8)]),
        "orc_enumerate_valid_sectors": (C.c_int64, [C.c_int, C.c_int, P(orc_qindex), P(C.c_int32), P(C.c_int8),
                                                    P(C.c_int32), C.c_int64]),
        "orc_heff_dense_build": (C.c_int, [P(orc_bst), P(orc_bst), C.c_int64, C.c_int64, P(C.c_double),
                                           C.c_int64, C.c_int64, P(C.c_double), P(C.c_double)]),
        "orc_dense_matvec": (None, [C.c_int64, P(C.c_double), P(C.c_double), P(C.c_double)]),
        "orc_heff_apply_dense": (C.c_int, [C.c_int64, C.c_int64, C.c_int64, C.c_int64, C.c_int64, P(C.c_double),
                                           P(C.c_double), C.c_int64, P(C.c_double), C.c_int64, P(C.c_double),
                                           P(C.c_double), P(C.c_double)]),
        "orc_bs_create": (C.c_void_p, [C.c_int, P(orc_qindex), P(orc_qindex), P(orc_qindex), P(orc_qindex),
                                       P(C.c_int32), C.c_int64, C.c_int64, C.c_int64, P(C.c_double), P(C.c_double),
                                       P(C.c_double), P(C.c_double)]),
        "orc_bs_destroy": (None, [C.c_void_p]),
        "orc_bs_total": (C.c_int64, [C.c_void_p]),
        "orc_bs_n_blocks": (C.c_int64, [C.c_void_p]),
        "orc_bs_blocks": (None, [C.c_void_p, P(C.c_int32), P(C.c_int64)]),
        "orc_bs_apply": (C.c_int, [C.c_void_p, P(C.c_double), P(C.c_double)]),
        "orc_bs_flops": (C.c_double, [C.c_void_p]),
        "orc_bs_to_dense": (None, [C.c_void_p, P(C.c_double), P(C.c_double)]),
        "orc_bs_from_dense": (None, [C.c_void_p, P(C.c_double), P(C.c_double)]),
        "orc_num_threads": (C.c_int, []),
        "orc_set_num_threads": (None, [C.c_int]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _libs[timed] = lib
    return lib


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class _Keep:
    def __init__(self):
        self.k = []

    def qindex(self, charges, dims):
        ch = np.ascontiguousarray(np.asarray(charges, dtype=np.int32).reshape(-1))
        dm = np.ascontiguousarray(np.asarray(dims, dtype=np.int64))
        self.k += [ch, dm]
        return orc_qindex(len(dm), ch.ctypes.data_as(C.POINTER(C.c_int32)), dm.ctypes.data_as(C.POINTER(C.c_int64)))


def qn_pack(kind: int, q) -> int:
    a = np.asarray(list(q) + [0], dtype=np.int32)
    return int(load().orc_qn_pack(kind, a.ctypes.data_as(C.POINTER(C.c_int32))))


def qn_unpack(kind: int, bits: int, ncomp: int) -> tuple:
    a = np.zeros(2, dtype=np.int32)
    load().orc_qn_unpack(kind, bits, a.ctypes.data_as(C.POINTER(C.c_int32)))
    return tuple(int(x) for x in a[:ncomp])


def key_pack(kind: int, qns) -> int:
    a = np.asarray(qns, dtype=np.int32).reshape(-1)
    return int(load().orc_key_pack(kind, len(qns), a.ctypes.data_as(C.POINTER(C.c_int32))))


def key_unpack(kind: int, rank: int, key: int, ncomp: int) -> list:
    a = np.zeros(rank * 2, dtype=np.int32)
    load().orc_key_unpack(kind, rank, key, a.ctypes.data_as(C.POINTER(C.c_int32)))
    return [tuple(int(x) for x in a[i * ncomp:(i + 1) * ncomp]) for i in range(rank)]


def check_flux_rule(kind: int, qns, flux, dirs) -> bool:
    q = np.asarray(qns, dtype=np.int32).reshape(-1)
    f = np.asarray(list(flux) + [0], dtype=np.int32)
    d = np.asarray(dirs, dtype=np.int8)
    return bool(load().orc_check_flux_rule(kind, len(dirs), q.ctypes.data_as(C.POINTER(C.c_int32)),
                                           f.ctypes.data_as(C.POINTER(C.c_int32)),
                                           d.ctypes.data_as(C.POINTER(C.c_int8))))


def enumerate_valid_sectors(kind: int, legs, flux, dirs) -> np.ndarray:
    """legs: list of (charges[n_sectors][ncomp], dims); returns sector-index tuples in DFS order."""
    kp = _Keep()
    arr = (orc_qindex * len(legs))(*[kp.qindex(c, d) for c, d in legs])
    f = np.asarray(list(flux) + [0], dtype=np.int32)
    d = np.asarray(dirs, dtype=np.int8)
    lib = load()
    P32 = C.POINTER(C.c_int32)
    n = lib.orc_enumerate_valid_sectors(kind, len(legs), arr, f.ctypes.data_as(P32),
                                        d.ctypes.data_as(C.POINTER(C.c_int8)), None, 0)
    out = np.zeros((max(n, 1), len(legs)), dtype=np.int32)
    lib.orc_enumerate_valid_sectors(kind, len(legs), arr, f.ctypes.data_as(P32),
                                    d.ctypes.data_as(C.POINTER(C.c_int8)), out.ctypes.data_as(P32), n)
    return out[:n]


def _bst(kp: _Keep, kind, legs, keys, offsets, data):
    arr = (orc_qindex * len(legs))(*[kp.qindex(c, d) for c, d in legs])
    keys = np.ascontiguousarray(keys, dtype=np.uint64)
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    data = np.ascontiguousarray(data, dtype=np.float64)
    kp.k += [arr, keys, offsets, data]
    return orc_bst(kind, len(legs), arr, len(keys), keys.ctypes.data_as(C.POINTER(C.c_uint64)),
                   offsets.ctypes.data_as(C.POINTER(C.c_int64)), _d(data))


def heff_dense(kind, wi, wj, L, R) -> np.ndarray:
    """Literal dense H (environments/mod.rs:491-602).  wi/wj: (legs, keys, offsets, data)."""
    kp = _Keep()
    bi, bj = _bst(kp, kind, *wi), _bst(kp, kind, *wj)
    L = np.ascontiguousarray(L, dtype=np.float64)
    R = np.ascontiguousarray(R, dtype=np.float64)
    d_i = int(np.sum(wi[0][0][1]))
    d_j = int(np.sum(wj[0][0][1]))
    dim = d_i * d_j * L.shape[2] * R.shape[2]
    H = np.zeros((dim, dim))
    load().orc_heff_dense_build(C.byref(bi), C.byref(bj), L.shape[2], L.shape[1], _d(L), R.shape[2], R.shape[1],
                                _d(R), _d(H))
    return H


def heff_apply_dense(Wi, Wj, L, R, x) -> np.ndarray:
    """Factored dense matvec; Wi (d,d,wl,wm), Wj (d,d,wm,wr) dense global."""
    Wi = np.ascontiguousarray(Wi, dtype=np.float64)
    Wj = np.ascontiguousarray(Wj, dtype=np.float64)
    L = np.ascontiguousarray(L, dtype=np.float64)
    R = np.ascontiguousarray(R, dtype=np.float64)
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros_like(x)
    rc = load().orc_heff_apply_dense(Wi.shape[0], Wj.shape[0], Wi.shape[2], Wi.shape[3], Wj.shape[3], _d(Wi),
                                     _d(Wj), L.shape[2], _d(L), R.shape[2], _d(R), _d(x), _d(y))
    if rc != 0:
        raise MemoryError("oracle dense apply failed")
    return y


class BlockSparseOracle:
    """Block-sparse FP64 matvec in the FlatBlockStorage layout.  timed=False:
    the checker build; timed=True: the FMA build timed as the CPU baseline."""

    def __init__(self, kind, phys_i, phys_j, bond_l, bond_r, flux, Wi, Wj, L, R, timed: bool = False):
        self._lib = load(timed)
        self._kp = _Keep()
        kp = self._kp
        self.Wi = np.ascontiguousarray(Wi, dtype=np.float64)
        self.Wj = np.ascontiguousarray(Wj, dtype=np.float64)
        self.L = np.ascontiguousarray(L, dtype=np.float64)
        self.R = np.ascontiguousarray(R, dtype=np.float64)
        qi, qj, ql, qr = (kp.qindex(*phys_i), kp.qindex(*phys_j), kp.qindex(*bond_l), kp.qindex(*bond_r))
        self._q = (qi, qj, ql, qr)
        fl = None
        if flux is not None:
            self._flux = np.asarray(list(flux) + [0], dtype=np.int32)
            fl = self._flux.ctypes.data_as(C.POINTER(C.c_int32))
        lib = self._lib
        self._h = lib.orc_bs_create(kind, C.byref(qi), C.byref(qj), C.byref(ql), C.byref(qr), fl,
                                    self.Wi.shape[2], self.Wi.shape[3], self.Wj.shape[3], _d(self.Wi), _d(self.Wj),
                                    _d(self.L), _d(self.R))
        if not self._h:
            raise MemoryError("oracle plan allocation failed")
        self.total = int(lib.orc_bs_total(self._h))
        self.n_blocks = int(lib.orc_bs_n_blocks(self._h))
        self.dense_dim = self.Wi.shape[0] * self.Wj.shape[0] * self.L.shape[2] * self.R.shape[2]

    def __del__(self):
        try:
            if self._h:
                self._lib.orc_bs_destroy(self._h)
        except Exception:
            pass

    def apply(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(self.total)
        self._lib.orc_bs_apply(self._h, _d(x), _d(y))
        return y

    def apply_into(self, x: np.ndarray, y: np.ndarray) -> None:
        self._lib.orc_bs_apply(self._h, _d(x), _d(y))

    def flops(self) -> float:
        return float(self._lib.orc_bs_flops(self._h))

    def to_dense(self, xb):
        out = np.zeros(self.dense_dim)
        self._lib.orc_bs_to_dense(self._h, _d(np.ascontiguousarray(xb)), _d(out))
        return out

    def from_dense(self, xd):
        out = np.zeros(self.total)
        self._lib.orc_bs_from_dense(self._h, _d(np.ascontiguousarray(xd)), _d(out))
        return out

    def blocks(self):
        sec = np.zeros((self.n_blocks, 4), dtype=np.int32)
        off = np.zeros(self.n_blocks, dtype=np.int64)
        self._lib.orc_bs_blocks(self._h, sec.ctypes.data_as(C.POINTER(C.c_int32)), off.ctypes.data_as(C.POINTER(C.c_int64)))
        return sec, off


def set_threads(n: int, timed: bool = False) -> None:
    load(timed).orc_set_num_threads(n)


def num_threads(timed: bool = False) -> int:
    return int(load(timed).orc_num_threads())
